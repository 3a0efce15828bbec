/*
 * vdr_oracle.c -- CPU oracle for the Vanadis EBE HEX8 DR solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the test suite, the
 * smoke check and the CPU-baseline leg of the benchmark call it; the product
 * library never does.  It restates the reference's CPU path from its
 * mathematics, keeping the reference's operation order where the result's
 * last bits depend on it (sums left to right, products as written), so that
 * the known-answer values printed in src_v2026_2_1/vanadis_log.txt can be
 * reproduced.  Citations: OT = src_updates/vanadis_full_DR_OpenMP_timing.for,
 * VF = src_v2026_2_1/VANADIS.FOR, GP = src_updates/gauss_point_hex8DR.for,
 * CC = src_v2026_2_1/cudatest_coloring_gtx1060_optimized.cu.
 *
 * Parity pinning: the assembly, the Dirichlet mask (VF face table), the
 * BiCG solve and the mass integral are pinned by the dominance factor,
 * iteration counts and per-step masses of the reference's only recorded run
 * (vanadis_log.txt:45-240); the parity colouring is pinned by fixtures
 * generated from the reference's own colouring functions (CC:50-106).
 */
#include "vdr_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Reference-cube node signs, par_3d OT:297-338. */
static const double KSI[8] = {-1.0, 1.0, 1.0, -1.0, -1.0, 1.0, 1.0, -1.0};
static const double ETA[8] = {-1.0, -1.0, 1.0, 1.0, -1.0, -1.0, 1.0, 1.0};
static const double ZET[8] = {-1.0, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 1.0};
/* The Gauss abscissa literal of OT:335 (not 1/sqrt(3) to the last bit). */
static const double GAUSS_C = 0.577350269189626;
/* Face-3 node table i_pow(3,:) = (1,4,8,5), OT:350-353, 0-based here. */
static const int FACE3[4] = {0, 3, 7, 4};

/* ------------------------------------------------------------------ */
/* mesh and indexing                                                    */
/* ------------------------------------------------------------------ */

/* siatka OT:201-219: node id = jx + nax*(jy-1) + nax*nay*(jz-1), x fastest. */
void or_siatka(int nax, int nay, int naz, const double *dx, const double *dy,
               const double *dz, double *xx, double *yy, double *zz) {
  long i = 0;
  for (int jz = 0; jz < naz; jz++)
    for (int jy = 0; jy < nay; jy++)
      for (int jx = 0; jx < nax; jx++) {
        xx[i] = dx[jx];
        yy[i] = dy[jy];
        zz[i] = dz[jz];
        i++;
      }
}

/* w_el OT:221-251, restated as the running counter it is: k walks the
 * lower-front-left node of each element, skipping the last node of every
 * x-row and restarting at each new z-layer (offset ik2*ik). */
void or_w_el(int nax, int nay, int naz, int *iss) {
  const long E = (long)(nax - 1) * (nay - 1) * (naz - 1);
  const long ik2 = (long)nay * nax;
  long k = 1, ik = 0;
  for (long j = 1; j <= E; j++) {
    const long base = k + ik2 * ik;
    iss[0 * E + (j - 1)] = (int)(base);
    iss[1 * E + (j - 1)] = (int)(base + 1);
    iss[2 * E + (j - 1)] = (int)(base + 1 + nax);
    iss[3 * E + (j - 1)] = (int)(base + nax);
    iss[4 * E + (j - 1)] = (int)(base + (long)nax * nay);
    iss[5 * E + (j - 1)] = (int)(base + 1 + (long)nax * nay);
    iss[6 * E + (j - 1)] = (int)(base + 1 + (long)nax * nay + nax);
    iss[7 * E + (j - 1)] = (int)(base + (long)nax * nay + nax);
    k = k + 1;
    if (j % (nax - 1) == 0) k = k + 1;
    if (j % ((long)(nax - 1) * (nay - 1)) == 0) {
      k = 1;
      ik = ik + 1;
    }
  }
}

/* kod_el_dr OT:253-295: face codes 1 (z-min layer), 2 (z-max layer),
 * 3 (x-min column), 4 (x-max column), 6 (first y-row of every layer),
 * 5 (last y-row of every layer).  Loop bounds restated 1-based. */
void or_kod_el_dr(int nax, int nay, int naz, int *kod) {
  const long E = (long)(nax - 1) * (nay - 1) * (naz - 1);
  const long L = (long)(nax - 1) * (nay - 1);
  memset(kod, 0, sizeof(int) * 6 * E);
  for (long i = 1; i <= L; i++) kod[0 * E + i - 1] = 1;
  for (long i = E - L + 1; i <= E; i++) kod[1 * E + i - 1] = 2;
  for (long i = nax - 1; i <= E; i += nax - 1) kod[3 * E + i - 1] = 4;
  for (long i = 1; i <= E; i += nax - 1) kod[2 * E + i - 1] = 3;
  for (long k = 0; k <= naz - 2; k++)
    for (long i = k * L + 1; i <= k * L + nax - 1; i++) kod[5 * E + i - 1] = 6;
  for (long k = 1; k <= naz - 1; k++)
    for (long i = k * L - nax + 1 + 1; i <= k * L; i++) kod[4 * E + i - 1] = 5;
}

/* build_bc_nodes + mark_face_nodes: OT:1719-1810 (mask_mode 0) and
 * VF:2026-2110 (mask_mode 1).  Faces 1,2,4,5,6 are Dirichlet; face 3 is
 * the Robin face and is skipped. */
void or_build_bc_nodes(int nax, int nay, int naz, const int *iss,
                       const int *kod, int mask_mode, int *bc) {
  const long E = (long)(nax - 1) * (nay - 1) * (naz - 1);
  const long N = (long)nax * nay * naz;
  /* local node lists per face (1-based local ids as in the reference) */
  static const int F1[4] = {1, 2, 3, 4};
  static const int F2[4] = {5, 6, 7, 8};
  static const int F4[4] = {2, 3, 7, 6};
  static const int LO[4] = {1, 2, 6, 5}; /* y-min side nodes */
  static const int HI[4] = {4, 3, 7, 8}; /* y-max side nodes */
  memset(bc, 0, sizeof(int) * N);
  for (long e = 0; e < E; e++) {
    for (int f = 1; f <= 6; f++) {
      if (f == 3) continue;
      if (kod[(long)(f - 1) * E + e] != f) continue;
      const int *loc = 0;
      if (f == 1) loc = F1;
      else if (f == 2) loc = F2;
      else if (f == 4) loc = F4;
      else if (f == 5) loc = (mask_mode == OR_MASK_OT) ? LO : HI;
      else loc = (mask_mode == OR_MASK_OT) ? HI : LO; /* f == 6 */
      for (int a = 0; a < 4; a++) bc[iss[(long)(loc[a] - 1) * E + e] - 1] = 1;
    }
  }
}

/* ------------------------------------------------------------------ */
/* element kernel                                                       */
/* ------------------------------------------------------------------ */

/* shape_hex8DR OT:1398-1474: trilinear N and dN/d(xi,eta,zeta). */
static void shape_hex8(double xi, double eta, double zeta, double n[8],
                       double dn[3][8]) {
  const double xm = 1.0 - xi, xp = 1.0 + xi;
  const double ym = 1.0 - eta, yp = 1.0 + eta;
  const double zm = 1.0 - zeta, zp = 1.0 + zeta;
  n[0] = 0.125 * xm * ym * zm;
  n[1] = 0.125 * xp * ym * zm;
  n[2] = 0.125 * xp * yp * zm;
  n[3] = 0.125 * xm * yp * zm;
  n[4] = 0.125 * xm * ym * zp;
  n[5] = 0.125 * xp * ym * zp;
  n[6] = 0.125 * xp * yp * zp;
  n[7] = 0.125 * xm * yp * zp;
  dn[0][0] = -(0.125 * ym * zm);
  dn[0][1] = 0.125 * ym * zm;
  dn[0][2] = 0.125 * yp * zm;
  dn[0][3] = -(0.125 * yp * zm);
  dn[0][4] = -(0.125 * ym * zp);
  dn[0][5] = 0.125 * ym * zp;
  dn[0][6] = 0.125 * yp * zp;
  dn[0][7] = -(0.125 * yp * zp);
  dn[1][0] = -(0.125 * xm * zm);
  dn[1][1] = -(0.125 * xp * zm);
  dn[1][2] = 0.125 * xp * zm;
  dn[1][3] = 0.125 * xm * zm;
  dn[1][4] = -(0.125 * xm * zp);
  dn[1][5] = -(0.125 * xp * zp);
  dn[1][6] = 0.125 * xp * zp;
  dn[1][7] = 0.125 * xm * zp;
  dn[2][0] = -(0.125 * xm * ym);
  dn[2][1] = -(0.125 * xp * ym);
  dn[2][2] = -(0.125 * xp * yp);
  dn[2][3] = -(0.125 * xm * yp);
  dn[2][4] = 0.125 * xm * ym;
  dn[2][5] = 0.125 * xp * ym;
  dn[2][6] = 0.125 * xp * yp;
  dn[2][7] = 0.125 * xm * yp;
}

/* gauss_point_hex8DR: OT:1567-1716 (variant OT), GP:1-174 (variant GP),
 * VF:1868-2023 (variant VF).  Outputs detJ, N, W = N + tau*(v . grad N)
 * and grad N (the diffusion term uses grad W := grad N in all variants). */
void or_gauss_point(int variant, double xi, double eta, double zeta,
                    const double *xn, const double *yn, const double *zn,
                    const double *lambda, const double *v, double *detj_out,
                    double *n, double *w, double *dnx, double *dny,
                    double *dnz) {
  double dn[3][8];
  shape_hex8(xi, eta, zeta, n, dn);
  double j11 = 0.0, j12 = 0.0, j13 = 0.0, j21 = 0.0, j22 = 0.0, j23 = 0.0,
         j31 = 0.0, j32 = 0.0, j33 = 0.0;
  for (int i = 0; i < 8; i++) {
    j11 = j11 + xn[i] * dn[0][i];
    j12 = j12 + xn[i] * dn[1][i];
    j13 = j13 + xn[i] * dn[2][i];
    j21 = j21 + yn[i] * dn[0][i];
    j22 = j22 + yn[i] * dn[1][i];
    j23 = j23 + yn[i] * dn[2][i];
    j31 = j31 + zn[i] * dn[0][i];
    j32 = j32 + zn[i] * dn[1][i];
    j33 = j33 + zn[i] * dn[2][i];
  }
  const double detj = j11 * (j22 * j33 - j23 * j32) -
                      j12 * (j21 * j33 - j23 * j31) +
                      j13 * (j21 * j32 - j22 * j31);
  const double detji = 1.0 / detj;
  const double i11 = detji * (j22 * j33 - j23 * j32);
  const double i12 = detji * (j13 * j32 - j12 * j33);
  const double i13 = detji * (j12 * j23 - j13 * j22);
  const double i21 = detji * (j23 * j31 - j21 * j33);
  const double i22 = detji * (j11 * j33 - j13 * j31);
  const double i23 = detji * (j13 * j21 - j11 * j23);
  const double i31 = detji * (j21 * j32 - j22 * j31);
  const double i32 = detji * (j12 * j31 - j11 * j32);
  const double i33 = detji * (j11 * j22 - j12 * j21);
  for (int i = 0; i < 8; i++) {
    dnx[i] = i11 * dn[0][i] + i21 * dn[1][i] + i31 * dn[2][i];
    dny[i] = i12 * dn[0][i] + i22 * dn[1][i] + i32 * dn[2][i];
    dnz[i] = i13 * dn[0][i] + i23 * dn[1][i] + i33 * dn[2][i];
  }
  const double eps = 1.0e-14;
  const double vmag = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  double h_stream, lambda_s;
  if (variant == OR_DR_OT) {
    /* OT:1652-1671: axis edge lengths of the (assumed) brick. */
    const double dlx = fabs(xn[1] - xn[0]);
    const double dly = fabs(yn[3] - yn[0]);
    const double dlz = fabs(zn[4] - zn[0]);
    if (vmag > eps)
      h_stream = 2.0 / (fabs(v[0]) / dlx + fabs(v[1]) / dly +
                        fabs(v[2]) / dlz + eps);
    else
      h_stream = 0.0;
    lambda_s = lambda[0];
  } else {
    /* GP / VF:1954-1982: length along the streamline from J^-1 e. */
    double ex = 0.0, ey = 0.0, ez = 0.0;
    if (vmag > eps) {
      ex = v[0] / vmag;
      ey = v[1] / vmag;
      ez = v[2] / vmag;
    }
    const double gx = i11 * ex + i12 * ey + i13 * ez;
    const double gy = i21 * ex + i22 * ey + i23 * ez;
    const double gz = i31 * ex + i32 * ey + i33 * ez;
    const double gnorm = sqrt(gx * gx + gy * gy + gz * gz);
    h_stream = (gnorm > eps) ? 2.0 / gnorm : 0.0;
    if (variant == OR_DR_VF)
      lambda_s = lambda[0] * ex * ex + lambda[1] * ey * ey + lambda[2] * ez * ez;
    else
      lambda_s = lambda[0];
  }
  double pe = 0.0;
  if (vmag > eps && lambda_s > eps) pe = vmag * h_stream / (2.0 * lambda_s);
  double tau = 0.0;
  if (pe > 1.0e-12 && vmag > eps) {
    double beta;
    if (variant == OR_DR_VF) {
      /* VF:1994-2005 */
      if (pe < 1.0e-3)
        beta = pe / 3.0 - (pe * pe * pe) / 45.0 +
               2.0 * ((pe * pe) * (pe * pe) * pe) / 945.0;
      else if (pe > 50.0)
        beta = 1.0 - 1.0 / pe;
      else
        beta = 1.0 / tanh(pe) - 1.0 / pe;
    } else {
      /* OT:1681-1687: coth through exp (NaN once exp overflows). */
      const double epos = exp(pe), eneg = exp(-pe);
      const double coshp = 0.5 * (epos + eneg);
      const double sinhp = 0.5 * (epos - eneg);
      beta = coshp / sinhp - 1.0 / pe;
    }
    tau = 0.5 * h_stream / vmag * beta;
  }
  for (int i = 0; i < 8; i++) {
    const double vdotg = v[0] * dnx[i] + v[1] * dny[i] + v[2] * dnz[i];
    w[i] = n[i] + tau * vdotg;
  }
  *detj_out = detj;
}

/* quad4_3d OT:1199-1261: surface Jacobian |dX/dr x dX/ds| of a 4-node face. */
static double quad4_3d(const double x[4], const double y[4],
                       const double z[4], double r, double s) {
  double dndr[4], dnds[4];
  dndr[0] = -(0.25 * (1.0 - s));
  dndr[1] = 0.25 * (1.0 - s);
  dndr[2] = 0.25 * (1.0 + s);
  dndr[3] = -(0.25 * (1.0 + s));
  dnds[0] = -(0.25 * (1.0 - r));
  dnds[1] = -(0.25 * (1.0 + r));
  dnds[2] = 0.25 * (1.0 + r);
  dnds[3] = 0.25 * (1.0 - r);
  double xr = 0.0, xs = 0.0, yr = 0.0, ys = 0.0, zr = 0.0, zs = 0.0;
  for (int i = 0; i < 4; i++) {
    xr = xr + dndr[i] * x[i];
    xs = xs + dnds[i] * x[i];
    yr = yr + dndr[i] * y[i];
    ys = ys + dnds[i] * y[i];
    zr = zr + dndr[i] * z[i];
    zs = zs + dnds[i] * z[i];
  }
  const double cx = yr * zs - zr * ys;
  const double cy = zr * xs - xr * zs;
  const double cz = xr * ys - yr * xs;
  return sqrt(cx * cx + cy * cy + cz * cz);
}

/* el3d OT:431-610 (outputs hma after the final hma+cma+hmav, cma_n, fmv). */
void or_el3d(int variant, const double *xn, const double *yn,
             const double *zn, double lam, double pdec, const double *v,
             double q, int robin, double alpha, double *H, double *M,
             double *f) {
  const double lambda[3] = {lam, lam, lam};
  double hma[64], cma[64], hmav[64], cman[64], fmv[8];
  double n[8], w[8], dnx[8], dny[8], dnz[8], djac;
  for (int k = 0; k < 64; k++) hma[k] = cma[k] = hmav[k] = cman[k] = 0.0;
  for (int i = 0; i < 8; i++) fmv[i] = 0.0;

  double vol = 0.0;
  for (int g = 0; g < 8; g++) {
    or_gauss_point(variant, GAUSS_C * KSI[g], GAUSS_C * ETA[g],
                   GAUSS_C * ZET[g], xn, yn, zn, lambda, v, &djac, n, w, dnx,
                   dny, dnz);
    vol = vol + djac;
  }
  const double qv = q / vol;

  for (int g = 0; g < 8; g++) {
    or_gauss_point(variant, GAUSS_C * KSI[g], GAUSS_C * ETA[g],
                   GAUSS_C * ZET[g], xn, yn, zn, lambda, v, &djac, n, w, dnx,
                   dny, dnz);
    const double z1 = djac * lambda[0];
    const double z2 = djac * lambda[1];
    const double z3 = djac * lambda[2];
    for (int i = 0; i < 8; i++) fmv[i] = fmv[i] + qv * w[i] * djac;
    for (int i = 0; i < 8; i++)
      for (int j = 0; j < 8; j++) {
        const double hx = dnx[i] * dnx[j], hy = dny[i] * dny[j],
                     hz = dnz[i] * dnz[j];
        const double cg = w[i] * n[j];
        const double hvx = w[i] * dnx[j], hvy = w[i] * dny[j],
                     hvz = w[i] * dnz[j];
        const int k = 8 * i + j;
        hma[k] = hma[k] + hx * z1 + hy * z2 + hz * z3;
        hmav[k] = hmav[k] + (hvx * v[0] + hvy * v[1] + hvz * v[2]) * djac;
        cma[k] = cma[k] + cg * djac * pdec;
        cman[k] = cman[k] + cg * djac;
      }
  }

  if (robin) {
    /* Robin (third-kind) term on face 3 (xi = -1), OT:554-601. */
    double fx[4], fy[4], fz[4];
    for (int a = 0; a < 4; a++) {
      fx[a] = xn[FACE3[a]];
      fy[a] = yn[FACE3[a]];
      fz[a] = zn[FACE3[a]];
    }
    const double gp2[2] = {-GAUSS_C, GAUSS_C};
    for (int g1 = 0; g1 < 2; g1++)
      for (int g2 = 0; g2 < 2; g2++) {
        const double ze2 = gp2[g1], ze3 = gp2[g2];
        const double detjs = quad4_3d(fx, fy, fz, ze2, ze3);
        or_gauss_point(variant, -1.0, ze2, ze3, xn, yn, zn, lambda, v, &djac,
                       n, w, dnx, dny, dnz);
        const double znic = detjs * 1.0 * 1.0 * alpha;
        for (int i = 0; i < 8; i++)
          for (int j = 0; j < 8; j++) {
            const int k = 8 * i + j;
            cma[k] = cma[k] + (w[i] * n[j]) * znic;
          }
      }
  }
  for (int k = 0; k < 64; k++) {
    H[k] = hma[k] + cma[k] + hmav[k];
    M[k] = cman[k];
  }
  for (int i = 0; i < 8; i++) f[i] = fmv[i];
}

/* przest3d OT:649-740 with general coefficients; see the header. */
void or_assemble(int variant, int nnode, int nelem, const double *xx,
                 const double *yy, const double *zz, const int *iss,
                 const int *kod, const double *vel, const double *lam,
                 const double *pdec, const double *q, double robin_alpha,
                 double aH, double aM, double cf, double rM,
                 const double *t_old, double *bb, double *b, double *diag,
                 int nthreads) {
  const long E = nelem;
  double *eb = (b || diag) ? (double *)malloc(sizeof(double) * 16 * E) : 0;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (long e = 0; e < E; e++) {
    double xn[8], yn[8], zn[8], H[64], M[64], f[8], A[64];
    int nd[8];
    for (int s = 0; s < 8; s++) {
      nd[s] = iss[s * E + e] - 1;
      xn[s] = xx[nd[s]];
      yn[s] = yy[nd[s]];
      zn[s] = zz[nd[s]];
    }
    const double v[3] = {vel[e], vel[E + e], vel[2 * E + e]};
    const int robin = kod ? (kod[2 * E + e] == 3) : 0;
    or_el3d(variant, xn, yn, zn, lam[e], pdec ? pdec[e] : 0.0, v,
            q ? q[e] : 0.0, robin, robin_alpha, H, M, f);
    for (int k = 0; k < 64; k++) A[k] = aH * H[k] + aM * M[k];
    if (bb) memcpy(bb + 64 * e, A, sizeof(double) * 64);
    if (eb) {
      for (int i = 0; i < 8; i++) {
        double ft = 0.0;
        if (t_old) {
          /* hma_t = H - rM*M ; fmv_t = hma_t . T_old (ilo_m_v, OT:415-429) */
          for (int k = 0; k < 8; k++)
            ft = ft + (H[8 * i + k] - rM * M[8 * i + k]) * t_old[nd[k]];
        }
        eb[16 * e + i] = cf * f[i] - ft;
        eb[16 * e + 8 + i] = A[8 * i + i];
      }
    }
  }
  if (b) memset(b, 0, sizeof(double) * nnode);
  if (diag) memset(diag, 0, sizeof(double) * nnode);
  if (eb) {
    for (long e = 0; e < E; e++)
      for (int i = 0; i < 8; i++) {
        const int k = iss[i * E + e] - 1;
        if (b) b[k] = b[k] + eb[16 * e + i];
        if (diag) diag[k] = diag[k] + eb[16 * e + 8 + i];
      }
    free(eb);
  }
}

/* ------------------------------------------------------------------ */
/* operator applies                                                     */
/* ------------------------------------------------------------------ */

/* matvec_0 OT:1837-1881 */
void or_matvec0(int nnode, int nelem, const int *iss, const double *bb,
                const int *bc, double *xin, double *xout) {
  const long E = nelem;
  for (long j = 0; j < nnode; j++) xout[j] = 0.0;
  for (long j = 0; j < nnode; j++)
    if (bc[j] == 1) xin[j] = 0.0;
  long ik = 0;
  for (long e = 0; e < E; e++) {
    int nd[8];
    for (int s = 0; s < 8; s++) nd[s] = iss[s * E + e] - 1;
    for (int i = 0; i < 8; i++)
      for (int j = 0; j < 8; j++) {
        xout[nd[i]] = xout[nd[i]] + bb[ik] * xin[nd[j]];
        ik++;
      }
  }
  for (long j = 0; j < nnode; j++)
    if (bc[j] == 1) xout[j] = 0.0;
}

/* mttvec_0 OT:1883-1933 */
void or_mttvec0(int nnode, int nelem, const int *iss, const double *bb,
                const int *bc, double *xin, double *xout) {
  const long E = nelem;
  for (long j = 0; j < nnode; j++) xout[j] = 0.0;
  for (long j = 0; j < nnode; j++)
    if (bc[j] == 1) xin[j] = 0.0;
  for (long e = 0; e < E; e++) {
    int nd[8];
    for (int s = 0; s < 8; s++) nd[s] = iss[s * E + e] - 1;
    const double *b3 = bb + 64 * e;
    for (int i = 0; i < 8; i++)
      for (int j = 0; j < 8; j++)
        xout[nd[i]] = xout[nd[i]] + b3[8 * j + i] * xin[nd[j]];
  }
  for (long j = 0; j < nnode; j++)
    if (bc[j] == 1) xout[j] = 0.0;
}

void or_matvec0_omp(int nnode, int nelem, const int *iss, const double *bb,
                    const int *bc, const int *color_elems,
                    const int *color_offsets, int ncolors, int transpose,
                    double *xin, double *xout, int nthreads) {
  const long E = nelem;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
#endif
  {
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long j = 0; j < nnode; j++) {
      xout[j] = 0.0;
      if (bc[j] == 1) xin[j] = 0.0;
    }
    for (int c = 0; c < ncolors; c++) {
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (long t = color_offsets[c]; t < color_offsets[c + 1]; t++) {
        const long e = color_elems[t];
        int nd[8];
        double xv[8];
        for (int s = 0; s < 8; s++) {
          nd[s] = iss[s * E + e] - 1;
          xv[s] = xin[nd[s]];
        }
        const double *b3 = bb + 64 * e;
        for (int i = 0; i < 8; i++) {
          double acc = xout[nd[i]];
          for (int j = 0; j < 8; j++)
            acc = acc + (transpose ? b3[8 * j + i] : b3[8 * i + j]) * xv[j];
          xout[nd[i]] = acc;
        }
      }
    }
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long j = 0; j < nnode; j++)
      if (bc[j] == 1) xout[j] = 0.0;
  }
}

/* ------------------------------------------------------------------ */
/* Krylov solvers                                                       */
/* ------------------------------------------------------------------ */

static double dnrm2(long n, const double *x) { /* OT:1001-1009 */
  double s = 0.0;
  for (long i = 0; i < n; i++) s = s + x[i] * x[i];
  return sqrt(s);
}

/* dbcg_simple OT:906-984 */
int or_dbcg(int n, int nelem, const double *b, double *x, double tol,
            int itmax, int *iter, double *err, const double *bb,
            const int *iss, const double *diag, const int *bc) {
  double *p = (double *)calloc(6 * (size_t)n, sizeof(double));
  double *pp = p + n, *r = pp + n, *rr = r + n, *z = rr + n, *zz = z + n;
  double ak, akden, bk, bkden = 1.0, bknum, bnrm;
  int status = 1;
  *iter = 0;
  or_matvec0(n, nelem, iss, bb, bc, x, r);
  for (long i = 0; i < n; i++) {
    r[i] = b[i] - r[i];
    rr[i] = r[i];
  }
  for (long i = 0; i < n; i++) z[i] = r[i] / diag[i];
  for (long i = 0; i < n; i++) zz[i] = rr[i] / diag[i];
  bnrm = dnrm2(n, b);
  *err = dnrm2(n, r) / bnrm;
  if (*err <= tol) {
    status = 0;
    goto done;
  }
  for (int k = 1; k <= itmax; k++) {
    *iter = k;
    bknum = 0.0;
    for (long i = 0; i < n; i++) bknum = bknum + z[i] * rr[i];
    if (k == 1) {
      for (long i = 0; i < n; i++) {
        p[i] = z[i];
        pp[i] = zz[i];
      }
    } else {
      bk = bknum / bkden;
      for (long i = 0; i < n; i++) {
        p[i] = z[i] + bk * p[i];
        pp[i] = zz[i] + bk * pp[i];
      }
    }
    bkden = bknum;
    or_matvec0(n, nelem, iss, bb, bc, p, z);
    akden = 0.0;
    for (long i = 0; i < n; i++) akden = akden + z[i] * pp[i];
    ak = bknum / akden;
    for (long i = 0; i < n; i++) {
      x[i] = x[i] + ak * p[i];
      r[i] = r[i] - ak * z[i];
    }
    or_mttvec0(n, nelem, iss, bb, bc, pp, zz);
    for (long i = 0; i < n; i++) rr[i] = rr[i] - ak * zz[i];
    for (long i = 0; i < n; i++) z[i] = r[i] / diag[i];
    for (long i = 0; i < n; i++) zz[i] = rr[i] / diag[i];
    *err = dnrm2(n, r) / bnrm;
    if (*err <= tol) {
      status = 0;
      break;
    }
  }
done:
  free(p);
  return status;
}

static void apply_any(int n, int nelem, const int *iss, const double *bb,
                      const int *bc, const int *ce, const int *co, int nc,
                      int nthreads, double *xin, double *xout) {
  if (ce && co && nc > 0 && nthreads > 1)
    or_matvec0_omp(n, nelem, iss, bb, bc, ce, co, nc, 0, xin, xout, nthreads);
  else
    or_matvec0(n, nelem, iss, bb, bc, xin, xout);
}

static double dot_t(long n, const double *a, const double *b, int nthreads) {
  double s = 0.0;
#ifdef _OPENMP
  if (nthreads > 1) {
#pragma omp parallel for reduction(+ : s) schedule(static) num_threads(nthreads)
    for (long i = 0; i < n; i++) s += a[i] * b[i];
    return s;
  }
#endif
  (void)nthreads;
  for (long i = 0; i < n; i++) s = s + a[i] * b[i];
  return s;
}

/* Jacobi right-preconditioned BiCGStab (van der Vorst 1992). */
int or_bicgstab(int n, int nelem, const double *b, double *x, double tol,
                int itmax, int *iter, double *err, const double *bb,
                const int *iss, const double *diag, const int *bc,
                const int *ce, const int *co, int nc, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  double *buf = (double *)calloc(8 * (size_t)n, sizeof(double));
  double *r = buf, *rh = r + n, *p = rh + n, *v = p + n, *ph = v + n,
         *s = ph + n, *sh = s + n, *t = sh + n;
  int status = 1;
  *iter = 0;
  apply_any(n, nelem, iss, bb, bc, ce, co, nc, nthreads, x, r);
  for (long i = 0; i < n; i++) {
    r[i] = b[i] - r[i];
    rh[i] = r[i];
  }
  const double bnrm = sqrt(dot_t(n, b, b, nthreads));
  *err = sqrt(dot_t(n, r, r, nthreads)) / bnrm;
  if (*err <= tol) {
    free(buf);
    return 0;
  }
  double rho_old = 1.0, alpha = 1.0, omega = 1.0;
  for (int k = 1; k <= itmax; k++) {
    *iter = k;
    const double rho = dot_t(n, rh, r, nthreads);
    if (rho == 0.0 || !isfinite(rho)) {
      status = 2;
      break;
    }
    if (k == 1) {
      for (long i = 0; i < n; i++) p[i] = r[i];
    } else {
      const double beta = (rho / rho_old) * (alpha / omega);
      for (long i = 0; i < n; i++) p[i] = r[i] + beta * (p[i] - omega * v[i]);
    }
    for (long i = 0; i < n; i++) ph[i] = p[i] / diag[i];
    apply_any(n, nelem, iss, bb, bc, ce, co, nc, nthreads, ph, v);
    const double rv = dot_t(n, rh, v, nthreads);
    if (rv == 0.0 || !isfinite(rv)) {
      status = 2;
      break;
    }
    alpha = rho / rv;
    for (long i = 0; i < n; i++) s[i] = r[i] - alpha * v[i];
    const double snrm = sqrt(dot_t(n, s, s, nthreads)) / bnrm;
    if (snrm <= tol) {
      for (long i = 0; i < n; i++) {
        x[i] = x[i] + alpha * ph[i];
        r[i] = s[i];
      }
      *err = snrm;
      status = 0;
      break;
    }
    for (long i = 0; i < n; i++) sh[i] = s[i] / diag[i];
    apply_any(n, nelem, iss, bb, bc, ce, co, nc, nthreads, sh, t);
    const double tt = dot_t(n, t, t, nthreads);
    const double ts = dot_t(n, t, s, nthreads);
    if (tt == 0.0 || !isfinite(tt)) {
      status = 2;
      break;
    }
    omega = ts / tt;
    for (long i = 0; i < n; i++) {
      x[i] = x[i] + alpha * ph[i] + omega * sh[i];
      r[i] = s[i] - omega * t[i];
    }
    rho_old = rho;
    *err = sqrt(dot_t(n, r, r, nthreads)) / bnrm;
    if (*err <= tol) {
      status = 0;
      break;
    }
    if (omega == 0.0) {
      status = 2;
      break;
    }
  }
  free(buf);
  return status;
}

/* ------------------------------------------------------------------ */
/* diagnostics                                                          */
/* ------------------------------------------------------------------ */

static void dd_sums(int nnode, int nelem, const int *iss, const double *bb,
                    double *dg, double *sr) {
  const long E = nelem;
  for (long i = 0; i < nnode; i++) dg[i] = sr[i] = 0.0;
  for (long e = 0; e < E; e++)
    for (int i = 0; i < 8; i++) {
      const int gi = iss[i * E + e] - 1;
      for (int j = 0; j < 8; j++) {
        const int gj = iss[j * E + e] - 1;
        const double a = bb[64 * e + 8 * i + j];
        if (gi == gj)
          dg[gi] = dg[gi] + fabs(a);
        else
          sr[gi] = sr[gi] + fabs(a);
      }
    }
}

/* diagonal_dominance_factor OT:2122-2177: max_i sum_{j!=i}|a_ij| / |a_ii|. */
double or_dominance_factor(int nnode, int nelem, const int *iss,
                           const double *bb) {
  double *dg = (double *)malloc(sizeof(double) * 2 * (size_t)nnode);
  double *sr = dg + nnode;
  dd_sums(nnode, nelem, iss, bb, dg, sr);
  double m = 0.0;
  for (long i = 0; i < nnode; i++)
    if (dg[i] > 0.0) {
      const double ti = sr[i] / dg[i];
      if (ti > m) m = ti;
    }
  free(dg);
  return m;
}

/* is_diagonally_dominant OT:1936-1991 */
int or_is_diag_dominant(int nnode, int nelem, const int *iss,
                        const double *bb) {
  double *dg = (double *)malloc(sizeof(double) * 2 * (size_t)nnode);
  double *sr = dg + nnode;
  dd_sums(nnode, nelem, iss, bb, dg, sr);
  int ok = 1;
  for (long i = 0; i < nnode; i++)
    if (dg[i] <= sr[i]) {
      ok = 0;
      break;
    }
  free(dg);
  return ok;
}

/* integrate_mass_hex8 OT:2181-2285 (abscissa 1/sqrt(3) computed here). */
double or_integrate_mass(int nelem, const int *iss, const double *xx,
                         const double *yy, const double *zz,
                         const double *c) {
  const long E = nelem;
  const double g[2] = {-1.0 / sqrt(3.0), 1.0 / sqrt(3.0)};
  double mass = 0.0;
  for (long e = 0; e < E; e++) {
    double xc[8], yc[8], zc[8], cc[8];
    for (int a = 0; a < 8; a++) {
      const int nd = iss[a * E + e] - 1;
      xc[a] = xx[nd];
      yc[a] = yy[nd];
      zc[a] = zz[nd];
      cc[a] = c[nd];
    }
    for (int ig = 0; ig < 2; ig++)
      for (int jg = 0; jg < 2; jg++)
        for (int kg = 0; kg < 2; kg++) {
          double n[8], dn[3][8];
          shape_hex8(g[ig], g[jg], g[kg], n, dn);
          double j11 = 0.0, j12 = 0.0, j13 = 0.0, j21 = 0.0, j22 = 0.0,
                 j23 = 0.0, j31 = 0.0, j32 = 0.0, j33 = 0.0;
          for (int a = 0; a < 8; a++) {
            j11 = j11 + dn[0][a] * xc[a];
            j12 = j12 + dn[1][a] * xc[a];
            j13 = j13 + dn[2][a] * xc[a];
            j21 = j21 + dn[0][a] * yc[a];
            j22 = j22 + dn[1][a] * yc[a];
            j23 = j23 + dn[2][a] * yc[a];
            j31 = j31 + dn[0][a] * zc[a];
            j32 = j32 + dn[1][a] * zc[a];
            j33 = j33 + dn[2][a] * zc[a];
          }
          const double detj = j11 * (j22 * j33 - j23 * j32) -
                              j12 * (j21 * j33 - j23 * j31) +
                              j13 * (j21 * j32 - j22 * j31);
          double cv = 0.0;
          for (int a = 0; a < 8; a++) cv = cv + n[a] * cc[a];
          mass = mass + cv * detj * 1.0;
        }
  }
  return mass;
}

/* ------------------------------------------------------------------ */
/* colouring                                                            */
/* ------------------------------------------------------------------ */

/* CC:50-74: colour = (i&1) + 2(j&1) + 4(k&1), e = i + (nax-1)j + ... */
void or_parity_colors(int nax, int nay, int naz, int *color) {
  for (long k = 0; k < naz - 1; k++)
    for (long j = 0; j < nay - 1; j++)
      for (long i = 0; i < nax - 1; i++) {
        const long e = i + (long)(nax - 1) * j + (long)(nax - 1) * (nay - 1) * k;
        color[e] = (int)((i & 1) + 2 * (j & 1) + 4 * (k & 1));
      }
}

/* First fit in element index order; per-node bitmask of colours in use. */
int or_greedy_colors(int nnode, int nelem, const int *iss, int *color) {
  const long E = nelem;
  uint32_t *used = (uint32_t *)calloc((size_t)nnode, sizeof(uint32_t));
  int ncol = 0;
  for (long e = 0; e < E; e++) {
    uint32_t m = 0;
    for (int s = 0; s < 8; s++) m |= used[iss[s * E + e] - 1];
    if (m == 0xffffffffu) {
      free(used);
      return -1;
    }
    int c = 0;
    while (m & (1u << c)) c++;
    color[e] = c;
    if (c + 1 > ncol) ncol = c + 1;
    for (int s = 0; s < 8; s++) used[iss[s * E + e] - 1] |= (1u << c);
  }
  free(used);
  return ncol;
}

/* CC:82-106: stable compaction of the element ids of each colour. */
void or_color_lists(int nelem, const int *color, int ncolors,
                    int *color_elems, int *color_offsets) {
  int *cursor = (int *)calloc((size_t)ncolors + 1, sizeof(int));
  for (int c = 0; c <= ncolors; c++) color_offsets[c] = 0;
  for (long e = 0; e < nelem; e++) color_offsets[color[e] + 1]++;
  for (int c = 0; c < ncolors; c++)
    color_offsets[c + 1] += color_offsets[c];
  for (int c = 0; c < ncolors; c++) cursor[c] = color_offsets[c];
  for (long e = 0; e < nelem; e++) color_elems[cursor[color[e]]++] = (int)e;
  free(cursor);
}
