/*
 * vdr.h -- C ABI of libvdr.so, the GB300 (sm_103a) element-by-element HEX8
 * directional-residual (DR) solve of the Vanadis transport model.
 *
 * Two families of entry points:
 *
 * 1. kernel_dbcg_simple_ -- the reference's own solve entry point, same
 *    symbol, same arguments, same meaning.  It replaces
 *      src_v2026_2_1/cudatest.cu:301-305
 *      (= src_v2026_2_1/cudatest_coloring_gtx1060_optimized.cu:434-438),
 *    which the Fortran driver calls at src_v2026_2_1/VANADIS.FOR:809-810 as
 *      CALL kernel_dbcg_simple(NON,FMV3,TNW2,TOL,IL_I,ITER,ERR,BB,
 *                              ISS,DIAG,NAX,NAY,NAZ,bc_dirichlet)
 *    through an implicit interface (every argument by reference, trailing
 *    underscore).  The driver links against libvdr.so unchanged.
 *
 * 2. vdr_* -- a handle API that keeps the mesh, the per-element fields and
 *    the operator resident on the GPU across time steps and recomputes the
 *    DR element terms on the device (no host-assembled BB).  Its arrays use
 *    the reference driver's layouts: node coordinates xx/yy/zz[N]
 *    (siatka, vanadis_full_DR_OpenMP_timing.for:201-219), connectivity
 *    iss(E,8) column-major 1-based (w_el, :221-251), face codes kod(E,6)
 *    (kod_el_dr, :253-295), velocity (E,3) column-major and per-element
 *    scalars (the values atmosfera, :163-199, returns per element), the
 *    Dirichlet node mask bc_dirichlet[N] (build_bc_nodes, :1719-1810).
 *
 * All host pointers are caller-owned and only read during the call unless
 * documented as outputs.  "_device" variants take device pointers and run
 * on the handle's stream (vdr_stream), returning before the GPU finishes
 * unless stated.  No entry point ever calls exit(); errors come back as
 * status codes and vdr_last_error() describes the latest one.
 * A handle is not thread-safe; distinct handles may be used from distinct
 * host threads.
 */
#ifndef VDR_H
#define VDR_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define VDR_OK 0
#define VDR_NOT_CONVERGED 1
#define VDR_BREAKDOWN 2
#define VDR_CUDA_ERROR 3
#define VDR_BAD_ARGUMENT 4
#define VDR_TIMEOUT 5
#define VDR_IO_ERROR 6   /* a text output file could not be written */

/* ---- DR variants (gauss_point_hex8DR) ----
 * VDR_DR_OT: vanadis_full_DR_OpenMP_timing.for:1567-1716 (axis lengths,
 *            exp-based coth; NaN for element Peclet > 709.78, as there)
 * VDR_DR_GP: src_updates/gauss_point_hex8DR.for:1-174
 * VDR_DR_VF: src_v2026_2_1/VANADIS.FOR:1868-2023 (numerically safe) */
#define VDR_DR_OT 0
#define VDR_DR_GP 1
#define VDR_DR_VF 2

/* ---- scatter of element results to nodes ---- */
#define VDR_SCATTER_AUTO 0   /* measured choice: atomic */
#define VDR_SCATTER_ATOMIC 1 /* fp64 atomics, elements in natural order */
#define VDR_SCATTER_COLOR 2  /* colour by colour, no atomics, deterministic */
#define VDR_SCATTER_WARP 3   /* fp64 atomics aggregated within a warp: on the
                                structured numbering neighbouring lanes add
                                their shared face nodes by shuffles first
                                (half the atomics of the FP64 apply); plain
                                atomics elsewhere */

/* ---- operator apply ---- */
#define VDR_APPLY_AUTO 0        /* measured choice: stored */
#define VDR_APPLY_STORED 1      /* element matrices built on the GPU by the
                                   DR recompute kernel, kept in HBM */
#define VDR_APPLY_MATRIX_FREE 2 /* DR terms recomputed at every apply */

/* ---- element-matrix store (VDR_APPLY_STORED) ---- */
#define VDR_STORE_AUTO 0 /* measured choice: double-float */
#define VDR_STORE_FP64 1 /* FP64 entries, FP64 8x8 contraction */
#define VDR_STORE_DF 2   /* each FP64 entry as an FP32 pair hi + lo (48-bit
                            significand, same 8 bytes); the contraction runs
                            on the FP32 pipe in double-float arithmetic.
                            Falls back to FP64 when an entry or an input lies
                            outside the FP32 exponent range. */

/* ---- Krylov method ---- */
#define VDR_SOLVER_BICGSTAB 0 /* Jacobi right-preconditioned BiCGStab */
#define VDR_SOLVER_BICG 1     /* Jacobi BiCG, the reference's dbcg_simple */

/* How vdr_solve, vdr_solve_device and vdr_time_steps reach their FP64
 * tolerance: VDR_PRECISION_FP64 -- Krylov in FP64 on the FP64-accurate
 * operator; VDR_PRECISION_MIXED -- FP64 iterative refinement around inner
 * BiCGStab solves with the FP32 operator (as vdr_solve_mixed_device with
 * inner_tol 1e-5): the same FP64 true-residual criterion, fewer bytes per
 * iteration. */
#define VDR_PRECISION_FP64 0
#define VDR_PRECISION_MIXED 1

typedef struct vdr_options {
  int dr_variant;      /* VDR_DR_* (default VDR_DR_VF) */
  int scatter;         /* VDR_SCATTER_* */
  int apply_mode;      /* VDR_APPLY_* */
  int solver;          /* VDR_SOLVER_* */
  int iters_per_graph; /* iterations per CUDA-graph launch (0 -> 8) */
  int device;          /* CUDA device ordinal */
  int matrix_storage;  /* VDR_STORE_* */
  int precision;       /* VDR_PRECISION_* (default FP64) */
  int reserved[8];
} vdr_options;

typedef struct vdr_handle vdr_handle;

/* Fills *opt with the defaults. */
int vdr_default_options(vdr_options *opt);

/* Creates a handle for a HEX8 mesh.  iss is iss(E,8), column-major,
 * 1-based; kod is kod(E,6) column-major or NULL (then no element carries
 * the face-3 Robin term).  opt may be NULL (defaults). */
int vdr_create(vdr_handle **h, int nnode, int nelem, const double *xx,
               const double *yy, const double *zz, const int *iss,
               const int *kod, const vdr_options *opt);

/* Per-element fields: vel (E,3) column-major, lam[E] isotropic
 * diffusivity, pdec[E] decay rate (NULL = 0), q[E] source in kg/s
 * (NULL = 0), robin_alpha the face-3 transfer coefficient (licz_alfa). */
int vdr_set_fields(vdr_handle *h, const double *vel, const double *lam,
                   const double *pdec, const double *q, double robin_alpha);

/* Homogeneous Dirichlet node mask, bc[N] (1 = Dirichlet).  The operator
 * returns 0 on these rows and ignores these columns (matvec_0,
 * vanadis_full_DR_OpenMP_timing.for:1837-1881). */
int vdr_set_dirichlet(vdr_handle *h, const int *bc);

/* Selects the system matrix A = aH*H + aM*M (H = diffusion + DR advection
 * + decay*M + Robin, M = int W N).  Steady problems: (1, 0).  The
 * reference's theta-scheme: (2, 3/dt) (przest3d, :691-716). */
int vdr_set_operator(vdr_handle *h, double aH, double aM);

/* How the element build (el3d's per-element loop, vanadis_full_DR_OpenMP_
 * timing.for:431-610) gets the element geometry.  AUTO: the mesh's
 * geometric factors -- J^-1 and detJ at the 8 Gauss points and the
 * unit-diffusivity stiffness int gradN_i . gradN_j, 928 bytes per element --
 * are formed on the GPU once per handle (at the first build; a handle's
 * coordinates never change) and every later build forms the element
 * matrices from them and the current fields.  RECOMPUTE: every build
 * evaluates the Jacobians from the coordinates.  AUTO falls back to
 * RECOMPUTE where the factors would take more than half of the free device
 * memory, where a factor lies outside the double-float window, and for
 * Robin elements with a nonzero Robin coefficient.  Results agree to
 * double-float rounding (~1e-15 relative).  Setting the mode marks the
 * operator stale. */
#define VDR_BUILD_AUTO 0
#define VDR_BUILD_RECOMPUTE 1
int vdr_set_build_mode(vdr_handle *h, int mode);
/* *cached = 1 when the geometric factors are held (bytes of device memory
 * in *bytes), 0 when not (yet) formed, -1 when they cannot be used. */
int vdr_geometry_status(vdr_handle *h, int *cached, long long *bytes);
/* Diagnostic of the element build's double-float beta(Pe) = coth(Pe) -
 * 1/Pe (VF variant): beta[i] for the n host values pe[i] > 0, evaluated on
 * the current device as the build evaluates it (pe split into a pair,
 * result merged to FP64). */
int vdr_diag_beta_vf(int n, const double *pe, double *beta);

/* y = P A P x (transpose = 0) or y = P A^T P x, host arrays of length N. */
int vdr_apply(vdr_handle *h, const double *x, double *y, int transpose);
int vdr_apply_device(vdr_handle *h, const double *d_x, double *d_y,
                     int transpose);
/* d_y += P A P d_x (or the transpose) without clearing d_y first; Dirichlet
 * rows of d_y are left as they are. */
int vdr_apply_accumulate_device(vdr_handle *h, const double *d_x, double *d_y,
                                int transpose);

/* y = P A32 P x with the FP32 operator (DR terms and element matrices
 * computed in FP32; FP64 vectors, FP32 arithmetic inside the element). */
int vdr_apply32_device(vdr_handle *h, const double *d_x, double *d_y,
                       int transpose);

/* Right-hand side b = cf*f - (H - rM*M) T_old, assembled on the GPU, with
 * b = 0 on Dirichlet nodes (przest3d :691-716, :766-772).  t_old may be
 * NULL (steady: b = cf*f).  Host arrays of length N. */
int vdr_assemble_rhs(vdr_handle *h, double cf, double rM, const double *t_old,
                     double *b);
int vdr_assemble_rhs_device(vdr_handle *h, double cf, double rM,
                            const double *d_t_old, double *d_b);

/* Jacobi diagonal of the current operator (1 on Dirichlet nodes). */
int vdr_get_diag(vdr_handle *h, double *diag);

/* The current operator's element matrices in the reference's BB layout
 * (sklad_wd, vanadis_full_DR_OpenMP_timing.for:880-904): bb[64 e + 8 i + j]
 * = A_e(i,j) in FP64, e in the caller's element order, unmasked (Dirichlet
 * rows and columns are applied by the solver, as the reference does).  What
 * kernel_dbcg_simple_ takes as BB.  bb holds 64 E doubles (host array, or
 * device array for the _device form).  Stored operator only. */
int vdr_get_element_matrices(vdr_handle *h, double *bb);
int vdr_get_element_matrices_device(vdr_handle *h, double *d_bb);

/* Solves A x = b.  x holds the initial guess on entry (Dirichlet entries
 * are zeroed, as the reference does) and the solution on exit.  Stops when
 * ||r||_2/||b||_2 <= tol (recursively updated residual, as dbcg_simple) or
 * after itmax iterations.  Returns VDR_OK, VDR_NOT_CONVERGED,
 * VDR_BREAKDOWN or an error.  *iter = iterations done (0 if x already met
 * tol), *err = final relative residual. */
int vdr_solve(vdr_handle *h, const double *b, double *x, double tol,
              int itmax, int *iter, double *err);
int vdr_solve_device(vdr_handle *h, const double *d_b, double *d_x,
                     double tol, int itmax, int *iter, double *err);

/* Mixed precision: FP64 iterative refinement (residual b - A x and update
 * x += d in FP64 with the FP64 operator) around inner solves A32 d = r with
 * the FP32 operator (see vdr_set_mixed_operator).  Each inner solve stops at
 * max(inner_tol, 0.5 tol ||b|| / ||r||) relative to ||r||: no tighter than
 * the outer residual needs to reach tol.  Stops when the FP64 true relative
 * residual ||b - A x||/||b|| <= tol or after max_outer corrections; *err is
 * that FP64 residual.  Device arrays. */
/* The inner operator of the mixed solve (and the FP32 operator of
 * vdr_apply32_device):
 * VDR_MIXED_ROUNDED -- the FP64 element matrices rounded to FP32 (the hi
 * parts of the double-float store; no second build);
 * VDR_MIXED_RECOMPUTE -- element Jacobians and DR terms recomputed in FP32;
 * VDR_MIXED_HALF (default; the faster inner solve, measured: 23 vs 34 ms on
 * the 8.4M-element step) -- the Jacobi-scaled projected operator P A P D^-1 in
 * binary16 with one power-of-two scale per element (128 B per element
 * instead of 256), built from the FP64 element matrices when the operator
 * changes; the inner BiCGStab then runs without preconditioner vectors and
 * the correction is D^-1 of its solution.  Stored operator and BiCGStab
 * only (elsewhere, and where an element's scale leaves the binary16 range,
 * the rounded FP32 operator is used). */
#define VDR_MIXED_ROUNDED 0
#define VDR_MIXED_RECOMPUTE 1
#define VDR_MIXED_HALF 2
int vdr_set_mixed_operator(vdr_handle *h, int mode);
int vdr_solve_mixed_device(vdr_handle *h, const double *d_b, double *d_x,
                           double tol, double inner_tol, int max_outer,
                           int inner_itmax, int *outer_iters, int *inner_iters,
                           double *err);

/* y = A^ x with the binary16 inner operator A^ = P A P D^-1 of
 * VDR_MIXED_HALF (FP32 device vectors of length N); builds the store if the
 * operator changed.  For tests and measurement of that operator alone. */
int vdr_apply_half_device(vdr_handle *h, const float *d_x, float *d_y);

/* Device-resident time loop of the reference program (the do-while loop of
 * VANADIS.FOR:71-86 / vanadis_full_DR_OpenMP_timing.for:59-74 around
 * przest3d and integrate_mass_hex8): for k = 1..nsteps
 *   b = cf*f - (H - rM*M) T      (GPU, Dirichlet rows zero)
 *   T = A^-1 b                   (GPU solve, initial guess T, tolerance tol)
 *   masses[k-1] = int T dOmega   (GPU, read back once at the end)
 * with A the operator set by vdr_set_operator.  d_t holds T_0 on entry and
 * T_nsteps on exit.  masses, iters, errs are host arrays of nsteps entries
 * (each may be NULL).  Stops at the first solve that does not return
 * VDR_OK and returns its status; *steps_done counts completed steps.  With
 * the stored operator the first step also keeps M and F = sum_e f_e, and
 * the later steps (whose T is zero on Dirichlet nodes) form b from them as
 * cf*F - (A T)/aH + (aM/aH + rM) M T. */
int vdr_time_steps(vdr_handle *h, int nsteps, double cf, double rM,
                   double *d_t, double tol, int itmax, double *masses,
                   int *iters, double *errs, int *steps_done);

/* ---- many right-hand sides with one operator ----
 * Block arrays are N x K, node-major: X[n*K + k] (the K values of a node
 * contiguous).  K <= VDR_MAX_BLOCK_RHS; the TF32 tensor-core paths need
 * K = 16, 32 or 64. */
#define VDR_MAX_BLOCK_RHS 64
#define VDR_BLOCK_FP64 0 /* FP64 vectors, FP64-accurate (double-float) apply */
#define VDR_BLOCK_TF32 1 /* FP32 vectors, TF32 tensor-core apply
                            (mma.sync m16n8k8, FP32 accumulate) */
#define VDR_BLOCK_TF32X3 2 /* FP32 vectors, split TF32 (three MMAs per
                              product: FP32-level accuracy) */

/* Data movement of the tensor-core block apply: VDR_BLOCK_APPLY_AUTO
 * (default) is the node tile below, or for K = 64 the tcgen05 box apply
 * when the handle's first 64-column block solve measured it faster;
 * VDR_BLOCK_APPLY_TCGEN05 takes, for K = 64, boxes of 4 x 4 x 4 elements,
 * assembles each box's 125 x 125 operator in tensor memory and multiplies
 * it with the box's node rows on the fifth-generation tensor cores
 * (tcgen05.mma kind::tf32, node rows by TMA; other K use the node tile);
 * VDR_BLOCK_APPLY_TILE takes boxes of 8 x 2 x 2 elements of a mesh in the
 * canonical structured numbering, reads each node row of a box once into
 * shared memory and adds each result row once, one float4 atomic per 4
 * columns (mma.sync; other meshes, and colour-ordered storage, use the LSU
 * variant, as do the two forms above);
 * VDR_BLOCK_APPLY_LSU gathers X rows with 16-byte loads and scatters with
 * float4 atomics, per element; VDR_BLOCK_APPLY_BULK moves each element's
 * K-wide node rows into shared memory with cp.async.bulk (mbarrier
 * completion, three elements ahead per warp) and scatters with
 * cp.reduce.async.bulk -- limited by the copy engine's per-operation cost
 * on 64-256-byte rows. */
#define VDR_BLOCK_APPLY_BULK 0
#define VDR_BLOCK_APPLY_LSU 1
#define VDR_BLOCK_APPLY_TILE 2
#define VDR_BLOCK_APPLY_TCGEN05 3
#define VDR_BLOCK_APPLY_AUTO 4
int vdr_set_block_apply(vdr_handle *h, int variant);
/* Diagnostic of the bounded device wait used by VDR_BLOCK_APPLY_BULK (the
 * tcgen05 box apply bounds its waits the same way): one
 * warp waits on an mbarrier that nothing completes, with a ~1 ms budget;
 * the wait gives up, flags it and returns.  Returns VDR_TIMEOUT when that
 * path works (the handle stays usable). */
int vdr_diag_wait_timeout(vdr_handle *h);
/* Diagnostic of the bounded grid barrier of the mixed solve's fused inner
 * kernels (cooperative launches): one block of a two-block launch never
 * arrives, the other waits with a ~1 ms budget, gives up and marks the solve
 * state.  Returns VDR_TIMEOUT when that path works (the handle stays
 * usable). */
int vdr_diag_barrier_timeout(vdr_handle *h);

/* B[n*K + k] = cf * f(Q_k): the right-hand sides of K source fields at once.
 * d_Q is K x E (row k = per-element source of column k, kg/s, the caller's
 * element order).  Dirichlet rows are zero. */
int vdr_assemble_rhs_block_device(vdr_handle *h, int K, const double *d_Q,
                                  double cf, double *d_B);
/* Y = P A P X for K columns at once; precision VDR_BLOCK_FP64 (double
 * arrays, any K <= 64) or VDR_BLOCK_TF32 / VDR_BLOCK_TF32X3 (float arrays,
 * K = 16, 32 or 64). */
int vdr_apply_block_device(vdr_handle *h, int K, const void *d_X, void *d_Y,
                           int precision);
/* Y += P A P X, the same without zeroing Y first.  Both are ordered on the
 * handle's stream without a host synchronisation (the bulk-copy variant
 * synchronises to report a device wait that ran out). */
int vdr_apply_block_accumulate_device(vdr_handle *h, int K, const void *d_X,
                                      void *d_Y, int precision);
/* Solves A X = B for K columns (K = 16, 32 or 64): FP64 refinement per
 * column (residual with the FP64-accurate operator, FP64 update) around K
 * simultaneous FP32 Jacobi-BiCGStab inner solves with the tensor-core apply
 * (precision VDR_BLOCK_TF32 or VDR_BLOCK_TF32X3), column k to
 * max(inner_tol, 0.5 tol / err_k) relative to its residual (err_k its FP64
 * relative residual); columns already at tol sit out.
 * d_X holds the initial guess.  Returns VDR_OK when every column's FP64
 * relative residual is <= tol.  errs: K host doubles (final per-column FP64
 * residuals) or NULL.  No counterpart in the reference, which solves one
 * right-hand side per call. */
int vdr_solve_block_device(vdr_handle *h, int K, int precision,
                           const double *d_B, double *d_X, double tol,
                           double inner_tol, int max_outer, int inner_itmax,
                           int *outer_iters, int *inner_iters, double *errs);

/* ---- learned preconditioner ----
 * A 3-level 3D U-Net (16/32/64 channels, 3x3x3 convolutions, BF16 weights
 * and activations, FP32 accumulation) on the structured node grid of the
 * handle's mesh.  Inputs: r / rms(r) and the nodal velocity and
 * ln(lambda) - ln(1e-4) (element values averaged at the nodes); output: a
 * nodal correction c.  As a right preconditioner
 *     M(r) = D^-1 r + (rms(r) / dbar) c(r / rms(r)),
 * dbar = mean assembled diagonal over free nodes, zero on Dirichlet nodes.
 * Training pairs come from the solver's own iterates: r = b - A x_k,
 * e = x* - x_k, target (e - D^-1 r) dbar / rms(r).  No counterpart in the
 * reference. */
typedef struct vdr_net vdr_net;
/* Needs the structured numbering (the handle detected nax, nay, naz).  The
 * network is bound to the handle (its stream, mask and operator). */
int vdr_net_create(vdr_handle *h, unsigned long long seed, vdr_net **net);
int vdr_net_destroy(vdr_net *net);
/* The forward convolutions' kernels: VDR_NET_CONV_TCGEN05 (the default when
 * the TMA tensor maps of the network's inputs can be made) -- implicit GEMM
 * on the fifth-generation tensor cores (tcgen05.mma from TMA-loaded halo
 * slabs, FP32 accumulators in tensor memory); VDR_NET_CONV_MMA -- the
 * warp-level mma.sync kernels (the backward passes always use these).
 * VDR_BAD_ARGUMENT for TCGEN05 when its maps could not be made. */
#define VDR_NET_CONV_MMA 0
#define VDR_NET_CONV_TCGEN05 1
int vdr_net_set_conv(vdr_net *net, int mode);
/* The mode in use (nullable) and VDR_TIMEOUT if a tcgen05 convolution gave
 * up waiting for its operands since the last call (the flag is cleared);
 * synchronises the handle's stream. */
int vdr_net_conv_status(vdr_net *net, int *mode);
int vdr_net_param_count(vdr_net *net, long long *count);
/* FP32 master parameters / last gradients (host arrays of param_count). */
int vdr_net_get_params(vdr_net *net, float *host);
int vdr_net_set_params(vdr_net *net, const float *host);
int vdr_net_get_grads(vdr_net *net, float *host);
/* Nodal features and dbar from the handle's current fields and operator;
 * d_feat_out (N x 4 floats, nullable) and dbar_out receive copies. */
int vdr_net_update_features(vdr_net *net, float *d_feat_out, double *dbar_out);
int vdr_net_set_features_device(vdr_net *net, const float *d_feat, double dbar);
/* Training pair from an iterate x_k of the solve A x = b with converged
 * solution x*: r = b - A x_k, e = x* - x_k (FP64, length N) ->
 * rhat = r / rms(r), target = (e - D^-1 r) dbar / rms(r) (FP32). */
int vdr_net_make_pair_device(vdr_net *net, const double *d_b,
                             const double *d_xk, const double *d_xstar,
                             float *d_rhat, float *d_target);
/* Network output c for the normalised residual rhat (FP32, length N). */
int vdr_net_forward_device(vdr_net *net, const float *d_rhat, float *d_out);
/* Relative loss sum_free (c - t)^2 / sum_free t^2 and the gradients of
 * every parameter (read them with vdr_net_get_grads). */
int vdr_net_loss_grad_device(vdr_net *net, const float *d_rhat,
                             const float *d_target, double *loss);
/* Residual loss of a normalised residual rhat with the handle's current
 * operator: z = D^-1 rhat + c / dbar, L = ||rhat - A z||^2 / ||rhat||^2 over
 * free nodes (the quantity a minimal-residual Krylov step reduces), and the
 * gradients of every parameter (back through A with the transpose apply). */
int vdr_net_residual_loss_grad_device(vdr_net *net, const float *d_rhat,
                                      double *loss);
int vdr_net_adam_step(vdr_net *net, float lr, float beta1, float beta2,
                      float eps);
/* residual_loss_grad + Adam (0.9, 0.999, 1e-8). */
int vdr_net_train_step_residual_device(vdr_net *net, const float *d_rhat,
                                       float lr, double *loss);
/* loss_grad + Adam (0.9, 0.999, 1e-8); loss (nullable) is the step's loss. */
int vdr_net_train_step_device(vdr_net *net, const float *d_rhat,
                              const float *d_target, float lr, double *loss);
/* Jacobi post-smoothing of the preconditioner: after the network,
 * `steps` times out += omega D^-1 (in - A out) (default 1 step, omega 1). */
int vdr_net_set_smoothing(vdr_net *net, int steps, double omega);
/* d_out = M(d_in). */
int vdr_net_precondition_device(vdr_net *net, const double *d_in,
                                double *d_out);
/* Flexible BiCGStab (FP64) right-preconditioned by M.  A solve whose
 * residual has not dropped 1% in stall_window iterations (0: never) or that
 * breaks down continues with plain Jacobi-BiCGStab from its iterate
 * (*fell_back = 1).  iter counts both phases. */
int vdr_solve_learned_device(vdr_handle *h, vdr_net *net, const double *d_b,
                             double *d_x, double tol, int itmax,
                             int stall_window, int *iter, double *err,
                             int *fell_back);
/* Restarted GCR(restart) (1 <= restart <= 32), FP64, right-preconditioned
 * by Jacobi or, with net, by M: the flexible minimal-residual method (M is
 * applied to the current residual and ||r|| never increases).  With a
 * network, a stall (no 1% residual drop in stall_window iterations) or a
 * breakdown continues with Jacobi-BiCGStab from the iterate
 * (*fell_back = 1). */
int vdr_solve_gcr_device(vdr_handle *h, vdr_net *net, const double *d_b,
                         double *d_x, double tol, int itmax, int restart,
                         int stall_window, int *iter, double *err,
                         int *fell_back);
/* learned_steps (1..32) GCR steps with the network's preconditioner, then
 * Jacobi-BiCGStab from that iterate: the network only improves the start
 * of the solve.  iter counts both phases. */
int vdr_solve_learned_hybrid_device(vdr_handle *h, vdr_net *net,
                                    const double *d_b, double *d_x,
                                    double tol, int itmax, int learned_steps,
                                    int *iter, double *err);
/* vdr_solve_gcr_device (no fallback) recording x after every iteration into
 * d_hist (max_hist x N doubles); *n_hist = number recorded. */
int vdr_solve_gcr_record_device(vdr_handle *h, vdr_net *net, const double *d_b,
                                double *d_x, double tol, int itmax,
                                int restart, double *d_hist, int max_hist,
                                int *n_hist, int *iter, double *err);
/* Jacobi-BiCGStab recording the iterate x after every iteration into d_hist
 * (max_hist x N doubles); *n_hist = number recorded (the last entries may
 * repeat the converged x). */
int vdr_solve_record_device(vdr_handle *h, const double *d_b, double *d_x,
                            double tol, int itmax, double *d_hist,
                            int max_hist, int *n_hist, int *iter, double *err);

/* ---- many independent meshes in one handle ----
 * Build the handle on the concatenation of the meshes (node ids of mesh m
 * offset by node_off[m], elements concatenated); vdr_set_segments declares
 * the node ranges [node_off[m], node_off[m+1]) (nseg + 1 offsets; no element
 * may couple two ranges).  The element build and the operator applies then
 * cover every mesh in single launches, and the segmented solve runs
 * Jacobi-BiCGStab with per-mesh scalars and per-mesh convergence (a mesh
 * that converges freezes), all meshes advancing together in one CUDA graph.
 * The tile shape of the per-mesh reductions is chosen by measurement at the
 * first segmented solve (vdr_segment_tuning reports it).  No counterpart in
 * the reference, which solves one mesh per call. */
int vdr_set_segments(vdr_handle *h, int nseg, const int *node_off);
/* iters, errs, statuses: host arrays of nseg (nullable).  Returns VDR_OK
 * when every mesh met tol. */
int vdr_solve_segmented_device(vdr_handle *h, const double *d_b, double *d_x,
                               double tol, int itmax, int *iters,
                               double *errs, int *statuses);
int vdr_segment_tuning(vdr_handle *h, int *tile_nodes, int *threads);

/* Launch shapes of the operator applies, chosen by measurement on the
 * handle's own operator (no counterpart in the reference): the first build
 * of the stored operator times the stored apply's grid at 2, 4, 8, 16 and
 * 32 resident blocks per SM and keeps the fastest, the first build of the
 * binary16 inner operator does the same for its apply, and the first
 * 64-column block solve times the node-tile block apply's (box height,
 * column halves) at (2, 2), (2, 1) and (4, 2) and the tcgen05 box apply.
 * Meshes below 65,536 elements keep the defaults (8 blocks per SM; node
 * tile (2, 2)) and report zero times.  The stored and binary16 choices are
 * cached per scatter form, store and element-count octave for the process;
 * the block apply's per handle. */
typedef struct vdr_apply_tuning_info {
  int apply_blocks_per_sm, half_blocks_per_sm;
  int block_tile_y, block_halves;
  int grid_candidates[5];  /* blocks per SM tried, in the order of the times */
  float apply_ms[5], half_ms[5];  /* time per apply of each candidate */
  float block_ms[4];              /* node tile (2,2), (2,1), (4,2); tcgen05 */
  int block_tcgen05;              /* 1: the tcgen05 box apply was chosen */
} vdr_apply_tuning_info;
int vdr_apply_tuning(vdr_handle *h, vdr_apply_tuning_info *info);

/* Statistics of the handle's most recent solve. */
typedef struct vdr_solve_stats {
  int iterations;      /* Krylov iterations done */
  int status;          /* VDR_* status of that solve */
  int graph_launches;  /* CUDA-graph launches (iters_per_graph iterations each) */
  int kernel_launches; /* kernels launched by the solve, graph nodes included */
  int breakdown;       /* 0, or which quantity vanished: 1 (r0,r) 2 (r0,v)
                          3 (t,t) 4 omega 5 non-finite residual; 6 the
                          solve stalled (stall_window) */
  int reserved[3];
} vdr_solve_stats;
int vdr_last_solve_stats(vdr_handle *h, vdr_solve_stats *stats);

/* Number of CUDA kernels this library has launched in the process so far
 * (graph nodes counted per graph launch). */
long long vdr_kernel_launch_count(void);

/* True relative residual ||b - A x||/||b|| computed on the GPU in FP64. */
int vdr_true_residual_device(vdr_handle *h, const double *d_b,
                             const double *d_x, double *rel);

/* Total mass int c dOmega, 2x2x2 Gauss (integrate_mass_hex8,
 * vanadis_full_DR_OpenMP_timing.for:2181-2285). */
int vdr_mass(vdr_handle *h, const double *c, double *mass);
int vdr_mass_device(vdr_handle *h, const double *d_c, double *mass);

/* Host only, no GPU needed: the element colouring used by
 * VDR_SCATTER_COLOR.  On the reference's structured numbering (w_el) it is
 * the parity colouring of cudatest_coloring_gtx1060_optimized.cu:50-74,
 * (i&1) + 2(j&1) + 4(k&1); otherwise first-fit greedy in element order.
 * colors[nelem] out.  Returns the number of colours, or -VDR_BAD_ARGUMENT. */
int vdr_color_elements(int nnode, int nelem, const int *iss, int *colors);

/* The handle's CUDA stream (cudaStream_t). */
void *vdr_stream(vdr_handle *h);

int vdr_destroy(vdr_handle *h);

/* Message of the most recent failure in this thread ("" if none). */
/* ---- text outputs of a time step (host arrays, host threads) ----
 * The reference's result file T_sssss.TXT (vanadis_full_DR_OpenMP_timing
 * .for:797-806): per node x, y, z, t * scale (the reference writes
 * TNW2 * 1d6, kg/m^3 -> mg/m^3) in Fortran format (e12.5, 2x, e12.5, 2x,
 * e12.5, 2x, e12.5), one node per 55-byte line ending in '\n', written
 * as dir/T_sssss.TXT (the reference: output\T_sssss.TXT). */
int vdr_write_result_txt(const char *dir, int step, long nnode,
                         const double *xx, const double *yy, const double *zz,
                         const double *t, double scale);
/* The same text into buf (nnode * 55 bytes, no terminator). */
int vdr_format_result_txt(char *buf, long nnode, const double *xx,
                          const double *yy, const double *zz, const double *t,
                          double scale);
/* The 2-D slice files vanadis_files (vanadis_full_DR_OpenMP_timing.for:
 * 1089-1184) splits from T_sssss.TXT on an nax x nay x naz node grid
 * (x fastest): X_sssss_iii.TXT per x plane (y, z, s), Y_sssss_iii.TXT per
 * y row (z, x, s), Z_sssss_iii.TXT per z plane (y, x, s), s = t * scale,
 * format (e12.5, 2x, e12.5, 2x, e12.5); at most 999 nodes per axis (the
 * names carry i3.3 numbers). */
int vdr_write_slices_txt(const char *dir, int step, int nax, int nay, int naz,
                         const double *xx, const double *yy, const double *zz,
                         const double *t, double scale);

const char *vdr_last_error(void);

/* No counterpart in the reference.  The Jacobi BiCG solve of
 * kernel_dbcg_simple_ for callers that cannot allocate device memory: a
 * program whose device memory belongs to someone else after start-up (a
 * framework's caching allocator that has reserved the device, a fixed
 * memory budget set when the job starts), where a cudaMalloc would fail or
 * would take memory another component counts on.  This entry point calls no
 * cudaMalloc, cudaFree or allocating library routine.  Every pointer is a
 * DEVICE pointer owned by the caller, with the meaning of the
 * kernel_dbcg_simple_ arguments below (b, x in/out, bb in the BB[64e+8i+j]
 * layout, iss(E,8) column-major 1-based, diag, bc or NULL); sizes are
 * passed by value; stream is a cudaStream_t (NULL = default).  The call
 * returns when the solve has ended: it waits on its stream while it
 * iterates.  Its work vectors live in one fixed device array inside the
 * library, sized for n <= VDR_NOALLOC_MAX_NODES (about 3 MB, held on every
 * GPU that loads the library until the process exits); larger n is rejected
 * with VDR_BAD_ARGUMENT.  The first call on a device looks up that array's
 * device address (cudaGetSymbolAddress) and keeps it for the process, so
 * make that first call before any stream capture, and do not call this entry
 * point again after a cudaDeviceReset of that device.  All calls share the
 * array and each clears what it needs at its start: calls that overlap on
 * the GPU (two streams, two host threads) race.  An iss entry outside 1..n
 * returns VDR_BAD_ARGUMENT before any iteration runs (x then only has its
 * Dirichlet entries zeroed, as the solve masks its initial guess).  Returns
 * a VDR_* status; *iter, *err as kernel_dbcg_simple_ reports them. */
#define VDR_NOALLOC_MAX_NODES 65536
int vdr_bicg_noalloc_device(int n, int nax, int nay, int naz, const double *b,
                            double *x, double tol, int itmax,
                            const double *bb, const int *iss,
                            const double *diag, const int *bc, void *stream,
                            int *iter, double *err);

/* Drop-in for src_v2026_2_1/cudatest.cu:301-305.  N: number of unknowns;
 * B[N] right-hand side; X[N] initial guess in, solution out; TOL, ITMAX;
 * ITER out; ERR out (||r||/||b||); BB[64*E] element matrices as sklad_wd
 * lays them out (BB[64e+8i+j] = A_e(i,j)); ISS(E,8) column-major 1-based;
 * DIAG[N] Jacobi diagonal; NAX,NAY,NAZ node counts, E =
 * (NAX-1)(NAY-1)(NAZ-1); bc_dirichlet[N].  Jacobi BiCG as dbcg_simple.
 * Like the reference it returns nothing; on a CUDA failure ERR is set to
 * +Inf (so the caller's ERR > TOL test reports it) and vdr_last_error()
 * holds the message.  Device buffers persist between calls and are reused
 * while the sizes fit. */
void kernel_dbcg_simple_(int *N, double *B, double *X, double *TOL,
                         int *ITMAX, int *ITER, double *ERR, double *BB,
                         int *ISS, double *DIAG, int *NAX, int *NAY, int *NAZ,
                         int *bc_dirichlet);

#ifdef __cplusplus
}
#endif
#endif /* VDR_H */
