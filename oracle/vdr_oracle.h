/*
 * vdr_oracle.h -- CPU oracle for the Vanadis EBE HEX8 directional-residual
 * (DR) solve.  TEST INFRASTRUCTURE ONLY: the product library never links,
 * loads or calls anything declared here.  Only the test suite, the smoke
 * check and the CPU-baseline leg of the benchmark use it, to check the
 * product against.
 *
 * Every function restates, from its mathematics, one routine of the
 * reference Fortran CPU build `src_updates/vanadis_full_DR_OpenMP_timing.for`
 * (cited below as OT:line) or of the Linux/CUDA driver
 * `src_v2026_2_1/VANADIS.FOR` (VF:line).  Arrays keep the reference's
 * layouts so that fixtures can be compared element for element:
 *
 *   xx, yy, zz   double[N]            nodal coordinates
 *   iss          int[8*E]             Fortran iss(E,8), column-major,
 *                                     1-based node ids: iss[s*E + e]
 *   kod          int[6*E]             Fortran kod(E,6), column-major
 *   bb           double[64*E]         BB[64e + 8i + j] = A_e(i, j)
 *                                     (row i = test function W_i)
 *   bc           int[N]               1 = homogeneous Dirichlet node
 *   vel          double[3*E]          per-element velocity, (E,3) col-major
 *   lam, pdec, q double[E]            diffusivity, decay rate, source [kg/s]
 *
 * The file is compiled with -ffp-contract=off so that x86 and aarch64 hosts
 * round exactly as the reference's gfortran -O3 build does (no FMA).
 */
#ifndef VDR_ORACLE_H
#define VDR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* DR variants of gauss_point_hex8DR.
 *  0  OT: streamline length from axis edge lengths, lambda_s = lambda(1),
 *         coth(Pe) through exp (OT:1567-1716).  Overflows to NaN for
 *         Pe > ~709.78, exactly as the reference does.
 *  1  GP: streamline length 2/|J^-1 e|, lambda_s = lambda(1), coth through
 *         exp (src_updates/gauss_point_hex8DR.for:1-174).
 *  2  VF: streamline length 2/|J^-1 e|, lambda_s = e^T Lambda e, safe
 *         beta(Pe) (VF:1868-2023). */
enum { OR_DR_OT = 0, OR_DR_GP = 1, OR_DR_VF = 2 };

/* Dirichlet face tables of mark_face_nodes.
 *  0  OT:1761-1810 (faces 5/6 mark the interior node rows y=1, y=nay-2)
 *  1  VF:2063-2110 (faces 5/6 mark the boundary node rows) */
enum { OR_MASK_OT = 0, OR_MASK_VF = 1 };

/* ---- mesh and indexing (bit-exact integer work) ---- */
void or_siatka(int nax, int nay, int naz, const double *dx, const double *dy,
               const double *dz, double *xx, double *yy, double *zz);
void or_w_el(int nax, int nay, int naz, int *iss);
void or_kod_el_dr(int nax, int nay, int naz, int *kod);
void or_build_bc_nodes(int nax, int nay, int naz, const int *iss,
                       const int *kod, int mask_mode, int *bc);

/* ---- element kernel ---- */
void or_gauss_point(int variant, double xi, double eta, double zeta,
                    const double *xn, const double *yn, const double *zn,
                    const double *lambda3, const double *v3, double *detj,
                    double *n, double *w, double *dnx, double *dny,
                    double *dnz);
/* el3d: H = diffusion + DR advection + P*M + alpha*Robin(face 3),
 * M = int W N (cma_n), f = (Q/vol) int W.  Row-major 8x8 outputs. */
void or_el3d(int variant, const double *xn, const double *yn,
             const double *zn, double lam, double pdec, const double *v3,
             double q, int robin, double alpha, double *H, double *M,
             double *f);

/* Assembly over all elements (przest3d OT:649-740 generalised):
 *   BB_e = aH*H_e + aM*M_e
 *   b   += cf*f_e - (H_e - rM*M_e) . T_old|_e     (T_old may be NULL)
 *   diag += diag(BB_e)
 * Any of bb, b, diag may be NULL.  b and diag are zeroed first.
 * robin_alpha is applied on elements with kod(e,3) == 3 when kod != NULL. */
void or_assemble(int variant, int nnode, int nelem, const double *xx,
                 const double *yy, const double *zz, const int *iss,
                 const int *kod, const double *vel, const double *lam,
                 const double *pdec, const double *q, double robin_alpha,
                 double aH, double aM, double cf, double rM,
                 const double *t_old, double *bb, double *b, double *diag,
                 int nthreads);

/* ---- operator applies (OT:1837-1933).  xin is masked IN PLACE. ---- */
void or_matvec0(int nnode, int nelem, const int *iss, const double *bb,
                const int *bc, double *xin, double *xout);
void or_mttvec0(int nnode, int nelem, const int *iss, const double *bb,
                const int *bc, double *xin, double *xout);
/* The same applies, parallel over the elements of one colour at a time
 * (colour lists as built by or_color_lists).  Labelled OpenMP variant. */
void or_matvec0_omp(int nnode, int nelem, const int *iss, const double *bb,
                    const int *bc, const int *color_elems,
                    const int *color_offsets, int ncolors, int transpose,
                    double *xin, double *xout, int nthreads);

/* ---- Krylov solvers ---- */
/* dbcg_simple OT:906-984: Jacobi BiCG, serial.  Returns 0 converged,
 * 1 not converged.  *iter is 0 when the initial guess already meets tol. */
int or_dbcg(int n, int nelem, const double *b, double *x, double tol,
            int itmax, int *iter, double *err, const double *bb,
            const int *iss, const double *diag, const int *bc);
/* Jacobi-preconditioned BiCGStab on the same operator (right
 * preconditioning, van der Vorst 1992).  Same stopping rule. */
int or_bicgstab(int n, int nelem, const double *b, double *x, double tol,
                int itmax, int *iter, double *err, const double *bb,
                const int *iss, const double *diag, const int *bc,
                const int *color_elems, const int *color_offsets,
                int ncolors, int nthreads);

/* ---- diagnostics used as known-answer tests ---- */
double or_dominance_factor(int nnode, int nelem, const int *iss,
                           const double *bb);              /* OT:2122-2177 */
int or_is_diag_dominant(int nnode, int nelem, const int *iss,
                        const double *bb);                 /* OT:1936-1991 */
double or_integrate_mass(int nelem, const int *iss, const double *xx,
                         const double *yy, const double *zz,
                         const double *c);                 /* OT:2181-2285 */

/* ---- element colouring ---- */
/* Parity colouring of cudatest_coloring_gtx1060_optimized.cu:50-74. */
void or_parity_colors(int nax, int nay, int naz, int *color);
/* First-fit greedy colouring in element index order over shared nodes.
 * Returns the number of colours (<= 32) or -1 if more were needed. */
int or_greedy_colors(int nnode, int nelem, const int *iss, int *color);
/* Compact per-colour lists (cudatest_coloring...cu:82-106). */
void or_color_lists(int nelem, const int *color, int ncolors,
                    int *color_elems, int *color_offsets);

#ifdef __cplusplus
}
#endif
#endif
