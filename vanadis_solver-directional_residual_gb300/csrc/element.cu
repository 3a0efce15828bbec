// element.cu -- per-element DR recompute kernels.
//
// The build and apply kernels map one element onto 8 consecutive lanes;
// lane q evaluates Gauss point q (the reference's point order: the
// node-sign pattern of par_3d times 0.577350269189626) so the geometry,
// Jacobian inverse and DR weight of the 8 points are computed in parallel
// in registers.  What differs is what is done with them:
//
//   elem_build_df_kernel<SPLIT>  (default) A_e = aH H + aM M, row i kept by
//                                lane i, in double-float on the FP32 pipe,
//                                written to the double-float store, with the
//                                Jacobi diagonal, b += cf f - (H - rM M) T_old
//                                and, for the time loop, M and F = sum f_e
//                                (el3d + sklad_wd + diag assembly + przest3d,
//                                vanadis_full_DR_OpenMP_timing.for:431-610,
//                                676-740, 880-904); elem_dr_scalars_kernel
//                                forms its per-element velocity scalars
//   elem_build_kernel<T>         the same in plain FP64 (the range fallback)
//                                or FP32 (the recomputed FP32 operator)
//   mf_apply_kernel<T,TRANS>     y += C x or C^T x without forming C: lane q
//                                forms its point's contribution to all 8
//                                outputs, then a 3-step shuffle reduce-scatter
//                                leaves output i in lane i (matrix-free apply)
//   mass_weights_kernel,         int c dOmega (integrate_mass_hex8 :2181-2285)
//   mass_dot_kernel, mass_kernel from per-element weights formed once, or
//                                directly
//
// with H = int lambda gradN.gradN + int W (v.gradN) + P int W N
//          + alpha int_{face 3} W N,  M = int W N,  f = (Q/vol) int W.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "dfloat.cuh"
#include "dr_device.cuh"
#include "vdr_internal.h"

namespace vdr {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename T>
struct Src;
template <>
struct Src<double> {
  static __device__ __forceinline__ const double *vel(const OpArgs &a) { return a.f.vel; }
  static __device__ __forceinline__ const double *lam(const OpArgs &a) { return a.f.lam; }
  static __device__ __forceinline__ const double *pdec(const OpArgs &a) { return a.f.pdec; }
};
template <>
struct Src<float> {
  static __device__ __forceinline__ const float *vel(const OpArgs &a) { return a.vel32; }
  static __device__ __forceinline__ const float *lam(const OpArgs &a) { return a.lam32; }
  static __device__ __forceinline__ const float *pdec(const OpArgs &a) { return a.pdec32; }
};

template <typename T>
struct Elem {
  T xe[8], ye[8], ze[8];
  int c[8];  // connectivity entries (node | MASK_BIT)
  T vx, vy, vz, lam, pdec;
  bool robin;
};

// FP64 kernels use the node coordinates as stored.  FP32 kernels use them
// relative to local node 1, formed in FP64 and then rounded: the Jacobian,
// streamline length and face Jacobian depend only on coordinate
// differences, and rounding absolute coordinates (~1) to FP32 would cost
// ~1e-5 relative accuracy on an element of size 1/256.
template <typename T>
__device__ __forceinline__ void load_coords(const OpArgs &a, long p, Elem<T> &e) {
#pragma unroll
  for (int s = 0; s < 8; s++) {
    e.c[s] = __ldg(a.conn + (size_t)s * a.E + p);
    const int n = e.c[s] & NODE_BITS;
    e.xe[s] = __ldg(a.xx + n);
    e.ye[s] = __ldg(a.yy + n);
    e.ze[s] = __ldg(a.zz + n);
  }
}
template <>
__device__ __forceinline__ void load_coords<float>(const OpArgs &a, long p,
                                                   Elem<float> &e) {
  double x0 = 0.0, y0 = 0.0, z0 = 0.0;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    e.c[s] = __ldg(a.conn + (size_t)s * a.E + p);
    const int n = e.c[s] & NODE_BITS;
    const double x = __ldg(a.xx + n), y = __ldg(a.yy + n), z = __ldg(a.zz + n);
    if (s == 0) {
      x0 = x;
      y0 = y;
      z0 = z;
    }
    e.xe[s] = (float)(x - x0);
    e.ye[s] = (float)(y - y0);
    e.ze[s] = (float)(z - z0);
  }
}

template <typename T>
__device__ __forceinline__ void load_elem(const OpArgs &a, long p, Elem<T> &e) {
  load_coords<T>(a, p, e);
  const T *V = Src<T>::vel(a);
  e.vx = __ldg(V + p);
  e.vy = __ldg(V + a.E + p);
  e.vz = __ldg(V + 2 * (size_t)a.E + p);
  e.lam = __ldg(Src<T>::lam(a) + p);
  const T *P = Src<T>::pdec(a);
  e.pdec = P ? __ldg(P + p) : T(0);
  e.robin = a.f.robin ? (__ldg(a.f.robin + p) != 0) : false;
}

template <typename T>
__device__ __forceinline__ T gauss_coord(int q, int axis) {
  const T c = T(VDR_GAUSS_C);
  const float sg = axis == 0 ? node_sx(q) : (axis == 1 ? node_sy(q) : node_sz(q));
  return sg > 0 ? c : -c;
}

// Sum over the 8 lanes of one element (butterfly, same order in all lanes).
template <typename T>
__device__ __forceinline__ T group8_sum(T v) {
  v += __shfl_xor_sync(FULL, v, 1);
  v += __shfl_xor_sync(FULL, v, 2);
  v += __shfl_xor_sync(FULL, v, 4);
  return v;
}

// Reduce-scatter over the 8 lanes of one element: lane t returns
// sum over lanes of v[t].
template <typename T>
__device__ __forceinline__ T group8_reduce_scatter(const T (&v)[8], int lane8) {
  const bool b2 = lane8 & 4, b1 = lane8 & 2, b0 = lane8 & 1;
  T h[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const T send = b2 ? v[k] : v[k + 4];
    const T keep = b2 ? v[k + 4] : v[k];
    h[k] = keep + __shfl_xor_sync(FULL, send, 4);
  }
  T g[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const T send = b1 ? h[k] : h[k + 2];
    const T keep = b1 ? h[k + 2] : h[k];
    g[k] = keep + __shfl_xor_sync(FULL, send, 2);
  }
  const T send = b0 ? g[0] : g[1];
  const T keep = b0 ? g[1] : g[0];
  return keep + __shfl_xor_sync(FULL, send, 1);
}

constexpr int ROWS_EPB = 8;  // elements per 64-thread block

template <typename T>
struct BuildSmem {
  T g[ROWS_EPB][8][6][8];    // per element, per Gauss point q, per node j:
                             // dNj/dx, dNj/dy, dNj/dz, v.gradNj + P*Nj, Nj, Wj
  T d[ROWS_EPB][8][2];       // detJ, lambda*detJ
  T fnw[ROWS_EPB][4][2][8];  // face-3 points: N, W
  T fd[ROWS_EPB][4];         // alpha*detJs
  T tab[12][4][8];           // shape N, dN/dxi, dN/deta, dN/dzeta at the 8
                             // volume points and the 4 face-3 points
};

// Fills the shape tables of the 12 evaluation points (same for every
// element) once per block.
template <typename T>
__device__ __forceinline__ void fill_shape_tables(T (&tab)[12][4][8]) {
  for (int t = threadIdx.x; t < 12; t += blockDim.x) {
    T xi, eta, zeta;
    if (t < 8) {
      xi = gauss_coord<T>(t, 0);
      eta = gauss_coord<T>(t, 1);
      zeta = gauss_coord<T>(t, 2);
    } else {
      const T gc = T(VDR_GAUSS_C);
      xi = T(-1);
      eta = ((t - 8) & 2) ? gc : -gc;
      zeta = ((t - 8) & 1) ? gc : -gc;
    }
    shape_at<T>(xi, eta, zeta, tab[t][0], tab[t][1], tab[t][2], tab[t][3]);
  }
  __syncthreads();
}

// One pass over the elements computing, per element, the rows of
// H = int lambda gradN.gradN + int W (v.gradN + P N) + alpha int_face3 W N
// and M = int W N (lane i keeps row i), then any of
//   A_e = aH*H + aM*M  -> element-matrix store (FP64 pairs and/or FP32)
//   diag += diag(A_e)
//   b    += cf*f_e - (H - rM*M) . T_old|_e      (f = (Q/vol) int W)
// so that the operator build and the right-hand side share the Gauss-point
// work (przest3d's per-element loop, vanadis_full_DR_OpenMP_timing.for:
// 676-740, in one kernel).
template <typename T>
__global__ void __launch_bounds__(64) elem_build_kernel(OpArgs a, BuildArgs ba) {
  __shared__ BuildSmem<T> sm;
  fill_shape_tables<T>(sm.tab);
  const int lane8 = threadIdx.x & 7;
  const int le = threadIdx.x >> 3;
  const long E = a.E;
  const T aH = T(ba.aH), aM = T(ba.aM), rM = T(ba.rM);
  for (long base = (long)blockIdx.x * ROWS_EPB; base < E;
       base += (long)gridDim.x * ROWS_EPB) {
    const long pe = base + le;
    const bool valid = pe < E;
    const long p = valid ? pe : E - 1;
    Elem<T> el;
    load_elem<T>(a, p, el);
    GPData<T> o;
    gp_core<T>(a.variant, sm.tab[lane8][0], sm.tab[lane8][1], sm.tab[lane8][2],
               sm.tab[lane8][3], el.xe, el.ye, el.ze, el.lam, el.vx, el.vy,
               el.vz, o);
    const T vol = group8_sum<T>(o.detj);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      sm.g[le][lane8][0][j] = o.gx[j];
      sm.g[le][lane8][1][j] = o.gy[j];
      sm.g[le][lane8][2][j] = o.gz[j];
      sm.g[le][lane8][3][j] =
          (el.vx * o.gx[j] + el.vy * o.gy[j] + el.vz * o.gz[j]) + el.pdec * o.n[j];
      sm.g[le][lane8][4][j] = o.n[j];
      sm.g[le][lane8][5][j] = o.w[j];
    }
    sm.d[le][lane8][0] = o.detj;
    sm.d[le][lane8][1] = el.lam * o.detj;
    if (el.robin && lane8 < 4) {
      const T gc = T(VDR_GAUSS_C);
      const T r = (lane8 & 2) ? gc : -gc;
      const T s = (lane8 & 1) ? gc : -gc;
      const T djs = face3_detjs<T>(el.xe, el.ye, el.ze, r, s);
      gp_core<T>(a.variant, sm.tab[8 + lane8][0], sm.tab[8 + lane8][1],
                 sm.tab[8 + lane8][2], sm.tab[8 + lane8][3], el.xe, el.ye,
                 el.ze, el.lam, el.vx, el.vy, el.vz, o);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        sm.fnw[le][lane8][0][j] = o.n[j];
        sm.fnw[le][lane8][1][j] = o.w[j];
      }
      sm.fd[le][lane8] = T(a.f.robin_alpha) * djs;
    }
    __syncwarp();
    const int i = lane8;
    T accH[8], accM[8];
#pragma unroll
    for (int j = 0; j < 8; j++) accH[j] = accM[j] = T(0);
    T fw = T(0);
#pragma unroll 2
    for (int q = 0; q < 8; q++) {
      const T dj = sm.d[le][q][0];
      const T dl = sm.d[le][q][1];
      const T gxi = sm.g[le][q][0][i], gyi = sm.g[le][q][1][i],
              gzi = sm.g[le][q][2][i];
      const T wd = sm.g[le][q][5][i] * dj;
      fw += wd;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const T gg = gxi * sm.g[le][q][0][j] + gyi * sm.g[le][q][1][j] +
                     gzi * sm.g[le][q][2][j];
        accH[j] += dl * gg + wd * sm.g[le][q][3][j];
        accM[j] += wd * sm.g[le][q][4][j];
      }
    }
    if (el.robin) {
#pragma unroll
      for (int f = 0; f < 4; f++) {
        const T aw = sm.fd[le][f] * sm.fnw[le][f][1][i];
#pragma unroll
        for (int j = 0; j < 8; j++) accH[j] += aw * sm.fnw[le][f][0][j];
      }
    }
    __syncwarp();
    if (!valid) continue;
    const int ci = el.c[i];
    if (ba.A64 || ba.A32 || ba.Ahi || ba.diag) {
      T row[8];
#pragma unroll
      for (int j = 0; j < 8; j++) row[j] = aH * accH[j] + aM * accM[j];
      if (ba.A64) {
#pragma unroll
        for (int jj = 0; jj < 4; jj++)
          ba.A64[(size_t)(4 * i + jj) * E + p] =
              make_double2((double)row[2 * jj], (double)row[2 * jj + 1]);
      }
      if (ba.A32) {
#pragma unroll
        for (int h = 0; h < 2; h++)
          ba.A32[(size_t)(2 * i + h) * E + p] =
              make_float4((float)row[4 * h], (float)row[4 * h + 1],
                          (float)row[4 * h + 2], (float)row[4 * h + 3]);
      }
      if (ba.Ahi) {
        // The pair store holds nonzero entries in [2^-100, 2^120]; anything
        // else sends the operator to the FP64 store.
        bool bad = false;
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int ej = df_exp((double)row[j]);
          if (ej != 0 && (ej < 1023 - 100 || ej > 1023 + 120)) bad = true;
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
          float4 vh, vl;
          df_split((double)row[4 * h], vh.x, vl.x, bad);
          df_split((double)row[4 * h + 1], vh.y, vl.y, bad);
          df_split((double)row[4 * h + 2], vh.z, vl.z, bad);
          df_split((double)row[4 * h + 3], vh.w, vl.w, bad);
          ba.Ahi[(size_t)(2 * i + h) * E + p] = vh;
          ba.Alo[(size_t)(2 * i + h) * E + p] = vl;
        }
        if (bad) atomicOr(ba.bad, 1);
      }
      if (ba.diag && ci >= 0) atomicAdd(ba.diag + ci, (double)row[i]);
    }
    if (ba.phi) ba.phi[(size_t)i * E + p] = (double)fw / (double)vol;
    if (ba.b && ci >= 0) {
      const double qe = a.f.q ? __ldg(a.f.q + p) : 0.0;
      double val = ba.cf * ((qe / (double)vol) * (double)fw);
      if (ba.told) {
        double ft = 0.0;
#pragma unroll
        for (int j = 0; j < 8; j++)
          ft += (double)(accH[j] - rM * accM[j]) *
                __ldg(ba.told + (el.c[j] & NODE_BITS));
        val -= ft;
      }
      atomicAdd(ba.b + ci, val);
    }
  }
}

// Per-element DR scalars of the double-float build, one thread per element,
// in FP64 with the operations of dr_tau.  GP and VF variants:
// drs[0..2][p] = e = v/|v|, drs[3][p] = kpe = |v|/(2 lambda_s) and
// drs[4][p] = khalf = 0.5/|v|, the last two zero where Pe is zero at every
// point (|v| or lambda_s <= 1e-14), so that a point with streamline length h
// has Pe = h kpe and tau = h khalf beta(Pe).  OT, whose tau does not depend
// on the point: drs[0][p] = tau.
__global__ void __launch_bounds__(256) elem_dr_scalars_kernel(OpArgs a,
                                                              double *__restrict__ drs) {
  const long E = a.E;
  const double eps = 1.0e-14;
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < E;
       p += (long)gridDim.x * blockDim.x) {
    const double vx = __ldg(a.f.vel + p), vy = __ldg(a.f.vel + E + p),
                 vz = __ldg(a.f.vel + 2 * E + p);
    const double lam = __ldg(a.f.lam + p);
    const double vmag = sqrt(vx * vx + vy * vy + vz * vz);
    if (a.variant == DR_OT) {
      const int n0 = __ldg(a.conn + p) & NODE_BITS;
      const int n1 = __ldg(a.conn + (size_t)1 * E + p) & NODE_BITS;
      const int n3 = __ldg(a.conn + (size_t)3 * E + p) & NODE_BITS;
      const int n4 = __ldg(a.conn + (size_t)4 * E + p) & NODE_BITS;
      const double h = dr_h_axes<double>(
          vx, vy, vz, vmag, fabs(__ldg(a.xx + n1) - __ldg(a.xx + n0)),
          fabs(__ldg(a.yy + n3) - __ldg(a.yy + n0)),
          fabs(__ldg(a.zz + n4) - __ldg(a.zz + n0)));
      drs[p] = dr_tau_from<double>(DR_OT, h, vmag, lam);
    } else {
      double ex = 0.0, ey = 0.0, ez = 0.0, iv = 0.0;
      if (vmag > eps) {
        iv = 1.0 / vmag;
        ex = vx * iv;
        ey = vy * iv;
        ez = vz * iv;
      }
      const double lams =
          (a.variant == DR_VF) ? (lam * ex * ex + lam * ey * ey + lam * ez * ez) : lam;
      const bool on = vmag > eps && lams > eps;
      drs[p] = ex;
      drs[E + p] = ey;
      drs[2 * E + p] = ez;
      drs[3 * E + p] = on ? vmag / (2.0 * lams) : 0.0;
      drs[4 * E + p] = on ? 0.5 * iv : 0.0;
    }
  }
}

// The FP64-accurate element build with its arithmetic moved to the FP32
// pipe (on GB300 the FP64 pipe runs at 1/58 of the FP32 rate and is the
// scarce unit).  Per element, on 8 lanes:
//   lane k = node k: connectivity, coordinates relative to local node 1
//     (differences formed in FP64, then split into pairs) and, for the
//     right-hand side, T_old scaled by a power of two so that the element's
//     largest |T_old| lies in [1, 2);
//   lane q = Gauss point q: Jacobian, cofactors, 1/detJ, inverse, gradients
//     and W in double-float; |J^-1 e| in double-float; only sqrt, the
//     Peclet number and beta(Pe) (tanh) are FP64, with the element's
//     velocity scalars from elem_dr_scalars_kernel;
//   lane i = row i: the rows accumulated in double-float (exact FP32
//     two-products + TwoSum), then A_e, diag(A_e) and b += cf f or, with
//     T_old, b += cf f - (H - rM M) T_old.  SPLIT (T_old given) keeps H and
//     M apart; otherwise aH and aM are folded into the point weights and
//     A_e = aH H + aM M is accumulated directly (4 pair products per point
//     and node instead of 5, one accumulator row instead of two).
// Any value outside the pairs' safe window sets bit 2 of the flag and the
// host redoes the build with FP64 rows (elem_build_kernel<double>).
// The shape tables of the double-float kernels: N and its reference
// derivatives at the 8 Gauss points and, when ftab is given, N at the 4
// face-3 points; once per block, ending with __syncthreads.
__device__ __forceinline__ void fill_df_tables(Df2 (&tab)[8][4][8], Df2 (*ftab)[8]) {
  const int npts = ftab ? 12 : 8;
  for (int t = threadIdx.x; t < npts; t += blockDim.x) {
    double xi, eta, zeta;
    if (t < 8) {
      xi = gauss_coord<double>(t, 0);
      eta = gauss_coord<double>(t, 1);
      zeta = gauss_coord<double>(t, 2);
    } else {
      const double gc = VDR_GAUSS_C;
      xi = -1.0;
      eta = ((t - 8) & 2) ? gc : -gc;
      zeta = ((t - 8) & 1) ? gc : -gc;
    }
    double n[8], d0[8], d1[8], d2[8];
    shape_at<double>(xi, eta, zeta, n, d0, d1, d2);
    if (t >= 8) {
#pragma unroll
      for (int i = 0; i < 8; i++) ftab[t - 8][i] = df_from_double(n[i]);
      continue;
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
      tab[t][0][i] = df_from_double(n[i]);
      tab[t][1][i] = df_from_double(d0[i]);
      tab[t][2][i] = df_from_double(d1[i]);
      tab[t][3][i] = df_from_double(d2[i]);
    }
  }
  __syncthreads();
}

// One Gauss point in double-float: J from the element's node coordinates
// relative to local node 1 (rel[3k..3k+2], node 1 itself at the origin) and
// the reference derivatives t0..t2 of the 8 shape functions at the point;
// returns detJ as a pair, detj as FP64 and di[3a+b] = (J^-1)_{ab} =
// d xi_a / d x_b.  A detJ outside 2^-60..2^60 (zero, inf and NaN included)
// sets range_bad.
__device__ __forceinline__ Df2 df_inverse_jacobian(const Df2 *rel, const Df2 *t0,
                                                   const Df2 *t1, const Df2 *t2,
                                                   Df2 (&di)[9], double &detj,
                                                   bool &range_bad) {
  DfAcc J[9];
#pragma unroll
  for (int k = 0; k < 9; k++) J[k] = DfAcc{0.0f, 0.0f};
#pragma unroll 1
  for (int k = 1; k < 8; k++) {  // local node 1 is the origin
    const Df2 rx = rel[3 * k], ry = rel[3 * k + 1], rz = rel[3 * k + 2];
    df_acc(J[0], rx, t0[k]);
    df_acc(J[1], rx, t1[k]);
    df_acc(J[2], rx, t2[k]);
    df_acc(J[3], ry, t0[k]);
    df_acc(J[4], ry, t1[k]);
    df_acc(J[5], ry, t2[k]);
    df_acc(J[6], rz, t0[k]);
    df_acc(J[7], rz, t1[k]);
    df_acc(J[8], rz, t2[k]);
  }
  const Df2 j11 = df_norm(J[0]), j12 = df_norm(J[1]), j13 = df_norm(J[2]);
  const Df2 j21 = df_norm(J[3]), j22 = df_norm(J[4]), j23 = df_norm(J[5]);
  const Df2 j31 = df_norm(J[6]), j32 = df_norm(J[7]), j33 = df_norm(J[8]);
  const Df2 c11 = df_sub(df_mul(j22, j33), df_mul(j23, j32));
  const Df2 c12 = df_sub(df_mul(j21, j33), df_mul(j23, j31));
  const Df2 c13 = df_sub(df_mul(j21, j32), df_mul(j22, j31));
  const Df2 detp =
      df_add(df_sub(df_mul(j11, c11), df_mul(j12, c12)), df_mul(j13, c13));
  detj = df_to_double(detp.h, detp.l);
  {
    const int ed = df_exp(detj);  // zero, subnormal, inf, NaN included
    if (ed < 1023 - 60 || ed > 1023 + 60) range_bad = true;
  }
  const Df2 r = df_rcp(detp);
  di[0] = df_mul(r, c11);
  di[1] = df_mul(r, df_sub(df_mul(j13, j32), df_mul(j12, j33)));
  di[2] = df_mul(r, df_sub(df_mul(j12, j23), df_mul(j13, j22)));
  di[3] = df_neg(df_mul(r, c12));
  di[4] = df_mul(r, df_sub(df_mul(j11, j33), df_mul(j13, j31)));
  di[5] = df_mul(r, df_sub(df_mul(j13, j21), df_mul(j11, j23)));
  di[6] = df_mul(r, c13);
  di[7] = df_mul(r, df_sub(df_mul(j12, j31), df_mul(j11, j32)));
  di[8] = df_mul(r, df_sub(df_mul(j11, j22), df_mul(j12, j21)));
  return detp;
}

// coth x - 1/x (beta of the VF variant, beta_safe) in double-float on the
// FP32 pipe for a pair x > 0: below 1/2 the Taylor series of coth x - 1/x,
// sum_n 2^2n B_2n x^(2n-1) / (2n)! (the Bernoulli-number expansion of coth,
// ten terms: truncation below 2^-50 relative at x = 1/2); from 1/2 to 44,
// 1 - 1/x + 2u/(1 - u) with u = e^(-2x): 2x = k ln 2 + r (Cody-Waite
// reduction, ln 2 in three parts, the first of 16 bits so that k ln2_1 is
// exact), e^(-r) from the degree-7 Taylor polynomial of e^s at s = -r/8
// squared three times, then scaled by 2^-k; above 44 (u < 2^-126) 1 - 1/x.
// Measured against the exact function: relative error ~1e-15 typically,
// 1.2e-13 at most (just above 1/2, where 1 - 1/x and 2u/(1 - u) cancel).
__device__ __constant__ float COTH_SERIES[10][2] = {
    {0x1.555556p-2f, -0x1.555556p-27f},  {-0x1.6c16c2p-6f, 0x1.27d27ep-31f},
    {0x1.1566acp-9f, -0x1.ff754cp-36f},  {-0x1.bbd77ap-13f, 0x1.99621ep-38f},
    {0x1.66a8f2p-16f, 0x1.7ee1d8p-41f},  {-0x1.22805ep-19f, 0x1.377b30p-44f},
    {0x1.d6db2cp-23f, 0x1.382458p-49f},  {-0x1.7da4e2p-26f, 0x1.0cd548p-55f},
    {0x1.355872p-29f, -0x1.4d68b2p-56f}, {-0x1.f57d96p-33f, -0x1.19559ep-58f}};
__device__ __constant__ float EXP_TAYLOR[8][2] = {  // 1/n!, n = 0..7
    {1.0f, 0.0f},
    {1.0f, 0.0f},
    {0.5f, 0.0f},
    {0x1.555556p-3f, -0x1.555556p-28f},
    {0x1.555556p-5f, -0x1.555556p-30f},
    {0x1.111112p-7f, -0x1.dddddep-32f},
    {0x1.6c16c2p-10f, -0x1.27d27ep-35f},
    {0x1.a01a02p-13f, -0x1.7f97fap-39f}};

__device__ __forceinline__ Df2 df_beta_vf(Df2 x) {
  const Df2 one{1.0f, 0.0f};
  if (x.h < 0.5f) {
    const Df2 y = df_mul(x, x);
    Df2 p{COTH_SERIES[9][0], COTH_SERIES[9][1]};
#pragma unroll
    for (int n = 8; n >= 0; n--) p = df_add(df_mul(p, y), Df2{COTH_SERIES[n][0], COTH_SERIES[n][1]});
    return df_mul(p, x);
  }
  const Df2 base = df_sub(one, df_rcp(x));
  if (x.h > 44.0f) return base;
  // 2x = k ln2 + r, |r| <= ln2 / 2
  const Df2 y{2.0f * x.h, 2.0f * x.l};
  const float k = rintf(y.h * 0x1.715476p+0f);
  const float t1 = __fmaf_rn(-k, 0x1.62e4p-1f, y.h);  // exact
  const float p2 = __fmul_rn(k, 0x1.7f7d1cp-20f);
  const float e2 = __fmaf_rn(k, 0x1.7f7d1cp-20f, -p2);
  Df2 r = df_add(Df2{t1, 0.0f}, Df2{-p2, -e2});
  r = df_add(r, Df2{__fmaf_rn(-k, 0x1.ef357ap-45f, y.l), 0.0f});
  // e^(-r) = (e^s)^8
  const Df2 sx{-0.125f * r.h, -0.125f * r.l};
  Df2 e{EXP_TAYLOR[7][0], EXP_TAYLOR[7][1]};
#pragma unroll
  for (int n = 6; n >= 0; n--) e = df_add(df_mul(e, sx), Df2{EXP_TAYLOR[n][0], EXP_TAYLOR[n][1]});
  e = df_mul(e, e);
  e = df_mul(e, e);
  e = df_mul(e, e);
  const int ki = (int)k;
  const float sc = ki < 127 ? __int_as_float((127 - ki) << 23) : 0.0f;  // 2^-k
  const Df2 u{e.h * sc, e.l * sc};
  const Df2 t = df_mul(Df2{2.0f * u.h, 2.0f * u.l}, df_rcp(df_sub(one, u)));
  return df_add(base, t);
}

__global__ void beta_vf_kernel(int n, const double *__restrict__ pe, double *__restrict__ beta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Df2 b = df_beta_vf(df_from_double(pe[i]));
  beta[i] = df_to_double(b.h, b.l);
}

// The streamline parameter tau at one Gauss point of the double-float
// builds as a pair, di = J^-1 at the point: OT from the per-element value;
// GP and VF from h = 2/|J^-1 e| (zero for |J^-1 e| <= 1e-14), Pe = h kpe and
// tau = h khalf beta(Pe) with the element's scalars of
// elem_dr_scalars_kernel, beta(Pe) in double-float for VF (df_beta_vf) and
// in FP64 for GP (beta_exp, whose exp overflow the variant keeps).
__device__ __forceinline__ Df2 df_point_tau(const OpArgs &a, const double *drs, long p,
                                            const Df2 (&di)[9], bool &range_bad) {
  const long E = a.E;
  if (a.variant == DR_OT) return df_from_double_chk(__ldg(drs + p), range_bad);
  const Df2 exd = df_from_double(__ldg(drs + p));
  const Df2 eyd = df_from_double(__ldg(drs + E + p));
  const Df2 ezd = df_from_double(__ldg(drs + 2 * E + p));
  DfAcc gxa{0.0f, 0.0f}, gya{0.0f, 0.0f}, gza{0.0f, 0.0f};
  df_acc(gxa, di[0], exd);
  df_acc(gxa, di[1], eyd);
  df_acc(gxa, di[2], ezd);
  df_acc(gya, di[3], exd);
  df_acc(gya, di[4], eyd);
  df_acc(gya, di[5], ezd);
  df_acc(gza, di[6], exd);
  df_acc(gza, di[7], eyd);
  df_acc(gza, di[8], ezd);
  const Df2 gx = df_norm(gxa), gy = df_norm(gya), gz = df_norm(gza);
  DfAcc n2{0.0f, 0.0f};
  df_acc(n2, gx, gx);
  df_acc(n2, gy, gy);
  df_acc(n2, gz, gz);
  const double gn2 = df_to_double(n2.s, n2.c);
  const double h = (gn2 > 1.0e-28) ? 2.0 * rsqrt(gn2) : 0.0;
  const double pe = h * __ldg(drs + 3 * E + p);
  if (!(pe > 1.0e-12)) return Df2{0.0f, 0.0f};
  const double hk = h * __ldg(drs + 4 * E + p);
  if (a.variant == DR_VF)
    return df_mul(df_from_double_chk(hk, range_bad), df_beta_vf(df_from_double(fmin(pe, 1.0e30))));
  return df_from_double_chk(hk * beta_exp(pe), range_bad);
}

// Lane i's output of the double-float builds, from its accumulated rows:
// accH = A_e row i (!SPLIT) or H row i (SPLIT, with accM = M row i),
// fw = int W_i dOmega, qe = the element's source Q, vol = the element
// volume.  Writes the element-matrix
// store (double-float pairs, or FP64 rows), diag += A_ii, the M store, phi,
// f and b += cf f_i - ((H - rM M) T_old)_i as the BuildArgs ask; told is the
// element's T_old at the nodes scaled by 2^-tshift.
template <bool SPLIT>
__device__ __forceinline__ void df_rows_out(const OpArgs &a, const BuildArgs &ba, long p,
                                            int i, int ci, DfAcc (&accH)[8],
                                            DfAcc (&accM)[SPLIT ? 8 : 1], const DfAcc &fw,
                                            double qe, double vol, Df2 aHd, Df2 aMd, Df2 nrMd,
                                            const Df2 *told, int tshift) {
  const long E = a.E;
  if (ba.Ahi && !ba.A64) {
    // double-float store: A_e row = aH H + aM M formed in double-float,
    // stored as its (hi, lo) pair; the store window is checked on hi
    // (FP32 biased exponent 27..247 = FP64 exponent -100..120)
    Df2 rowd[8];
    bool bad = false;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if constexpr (SPLIT) {
        DfAcc acc{0.0f, 0.0f};
        df_acc(acc, aHd, df_norm(accH[j]));
        df_acc(acc, aMd, df_norm(accM[j % (SPLIT ? 8 : 1)]));
        rowd[j] = df_norm(acc);
      } else {
        rowd[j] = df_norm(accH[j]);
      }
      const unsigned eb = (__float_as_uint(rowd[j].h) >> 23) & 0xffu;
      if (rowd[j].h != 0.0f && (eb < 27u || eb > 247u)) bad = true;
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
      ba.Ahi[(size_t)(2 * i + h) * E + p] =
          make_float4(rowd[4 * h].h, rowd[4 * h + 1].h, rowd[4 * h + 2].h, rowd[4 * h + 3].h);
      ba.Alo[(size_t)(2 * i + h) * E + p] =
          make_float4(rowd[4 * h].l, rowd[4 * h + 1].l, rowd[4 * h + 2].l, rowd[4 * h + 3].l);
    }
    if (bad) atomicOr(ba.bad, 1);  // store window (bit 1)
    if (ba.diag && ci >= 0) atomicAdd(ba.diag + ci, df_to_double(rowd[i].h, rowd[i].l));
  }
  if (!ba.Ahi && (ba.A64 || ba.diag)) {
    double row[8];
#pragma unroll
    for (int j = 0; j < 8; j++)
      row[j] = SPLIT ? ba.aH * df_to_double(accH[j].s, accH[j].c) +
                           ba.aM * df_to_double(accM[j % (SPLIT ? 8 : 1)].s,
                                                accM[j % (SPLIT ? 8 : 1)].c)
                     : df_to_double(accH[j].s, accH[j].c);
    if (ba.A64) {
#pragma unroll
      for (int jj = 0; jj < 4; jj++)
        ba.A64[(size_t)(4 * i + jj) * E + p] = make_double2(row[2 * jj], row[2 * jj + 1]);
    }
    if (ba.diag && ci >= 0) atomicAdd(ba.diag + ci, row[i]);
  }
  if constexpr (SPLIT) {
    if (ba.Mhi) {
      // M row as its own double-float store (window as for A: bit 3)
      Df2 rowm[8];
      bool badm = false;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        rowm[j] = df_norm(accM[j % (SPLIT ? 8 : 1)]);
        const unsigned eb = (__float_as_uint(rowm[j].h) >> 23) & 0xffu;
        if (rowm[j].h != 0.0f && (eb < 27u || eb > 247u)) badm = true;
      }
#pragma unroll
      for (int h = 0; h < 2; h++) {
        ba.Mhi[(size_t)(2 * i + h) * E + p] =
            make_float4(rowm[4 * h].h, rowm[4 * h + 1].h, rowm[4 * h + 2].h, rowm[4 * h + 3].h);
        ba.Mlo[(size_t)(2 * i + h) * E + p] =
            make_float4(rowm[4 * h].l, rowm[4 * h + 1].l, rowm[4 * h + 2].l, rowm[4 * h + 3].l);
      }
      if (badm) atomicOr(ba.bad, 4);
    }
  }
  const double fwd = df_to_double(fw.s, fw.c);
  if (ba.phi) ba.phi[(size_t)i * E + p] = fwd / vol;
  if (ba.f && ci >= 0) atomicAdd(ba.f + ci, (qe / vol) * fwd);
  if (ba.b && ci >= 0) {
    double val = ba.cf * ((qe / vol) * fwd);
    if (SPLIT && ba.told) {
      // (H - rM M) T_old in double-float on the scaled T_old, scaled back
      DfAcc ft{0.0f, 0.0f};
#pragma unroll
      for (int j = 0; j < 8; j++) {
        DfAcc rowj = accH[j];
        df_acc(rowj, nrMd, df_norm(accM[j % (SPLIT ? 8 : 1)]));
        df_acc(ft, df_norm(rowj), told[j]);
      }
      double f = df_to_double(ft.s, ft.c);
      if (!df_scale(f, tshift)) f = ldexp(f, tshift);
      val -= f;
    }
    atomicAdd(ba.b + ci, val);
  }
}

struct BuildSmemDF {
  Df2 g[ROWS_EPB][8][5][8];  // per element, point q, node j: dNj/dx, dNj/dy,
                             // dNj/dz, v.gradNj + P Nj, Wj
  Df2 d[ROWS_EPB][8][2];     // detJ, lambda*detJ
  Df2 fw[ROWS_EPB][4][8];    // face-3 points: W
  Df2 fd[ROWS_EPB][4];       // alpha*detJs
  Df2 rel[ROWS_EPB][24];     // node k's (x, y, z) - node 1's at [3k..3k+2]
  Df2 told[ROWS_EPB][8];     // T_old at the nodes times 2^-shift
  Df2 tab[8][4][8];          // N, dN/dxi, dN/deta, dN/dzeta at the 8 points
  Df2 ftab[4][8];            // N at the 4 face-3 points
};

template <bool SPLIT>
__global__ void __launch_bounds__(64, 8) elem_build_df_kernel(OpArgs a, BuildArgs ba) {
  __shared__ BuildSmemDF sm;
  fill_df_tables(sm.tab, sm.ftab);
  const int lane8 = threadIdx.x & 7;
  const int le = threadIdx.x >> 3;
  const long E = a.E;
  bool range_bad = false;  // a quantity the pairs cannot hold safely
  const Df2 aHd = df_from_double_chk(ba.aH, range_bad);
  const Df2 aMd = df_from_double_chk(ba.aM, range_bad);
  const Df2 nrMd = df_neg(df_from_double_chk(SPLIT ? ba.rM : 0.0, range_bad));
  const bool need_rows = SPLIT || ba.Ahi || ba.A64 || ba.diag;
  const double *V = a.f.vel;
  for (long base = (long)blockIdx.x * ROWS_EPB; base < E;
       base += (long)gridDim.x * ROWS_EPB) {
    const long pe = base + le;
    const bool valid = pe < E;
    const long p = valid ? pe : E - 1;
    __syncwarp();  // the previous element's shared data has been read
    // ---- lane k = node k
    const int ck = __ldg(a.conn + (size_t)lane8 * E + p);
    const int nk = ck & NODE_BITS;
    const double xk = __ldg(a.xx + nk), yk = __ldg(a.yy + nk), zk = __ldg(a.zz + nk);
    const double x0 = __shfl_sync(FULL, xk, 0, 8);
    const double y0 = __shfl_sync(FULL, yk, 0, 8);
    const double z0 = __shfl_sync(FULL, zk, 0, 8);
    sm.rel[le][3 * lane8] = df_from_double_chk(xk - x0, range_bad);
    sm.rel[le][3 * lane8 + 1] = df_from_double_chk(yk - y0, range_bad);
    sm.rel[le][3 * lane8 + 2] = df_from_double_chk(zk - z0, range_bad);
    int tshift = 0;
    if (SPLIT && ba.told) {
      const double tk = __ldg(ba.told + nk);
      int em = df_exp(tk);
      em = max(em, __shfl_xor_sync(FULL, em, 1));
      em = max(em, __shfl_xor_sync(FULL, em, 2));
      em = max(em, __shfl_xor_sync(FULL, em, 4));
      if (em == 0 && tk != 0.0) range_bad = true;  // all subnormal
      tshift = em - 1023;
      Df2 t;
      df_split(tk, t.h, t.l, range_bad, tshift);  // inf/NaN: bad
      sm.told[le][lane8] = t;
    }
    const double vx = __ldg(V + p), vy = __ldg(V + E + p), vz = __ldg(V + 2 * E + p);
    const double lam = __ldg(a.f.lam + p);
    const double pdec = a.f.pdec ? __ldg(a.f.pdec + p) : 0.0;
    const bool robin = a.f.robin ? (__ldg(a.f.robin + p) != 0) : false;
    __syncwarp();
    // ---- lane q = Gauss point q
    const Df2 *tn = sm.tab[lane8][0], *t0 = sm.tab[lane8][1],
              *t1 = sm.tab[lane8][2], *t2 = sm.tab[lane8][3];
    Df2 di[9];
    double detj;
    const Df2 detp = df_inverse_jacobian(sm.rel[le], t0, t1, t2, di, detj, range_bad);
    const Df2 di11 = di[0], di12 = di[1], di13 = di[2];
    const Df2 di21 = di[3], di22 = di[4], di23 = di[5];
    const Df2 di31 = di[6], di32 = di[7], di33 = di[8];
    const Df2 taud = df_point_tau(a, ba.drs, p, di, range_bad);
    const Df2 vxd = df_from_double_chk(vx, range_bad);
    const Df2 vyd = df_from_double_chk(vy, range_bad);
    const Df2 vzd = df_from_double_chk(vz, range_bad);
    const Df2 pd = df_from_double_chk(pdec, range_bad);
#pragma unroll 2
    for (int j = 0; j < 8; j++) {
      DfAcc ax{0.0f, 0.0f}, ay{0.0f, 0.0f}, az{0.0f, 0.0f};
      df_acc(ax, di11, t0[j]);
      df_acc(ax, di21, t1[j]);
      df_acc(ax, di31, t2[j]);
      df_acc(ay, di12, t0[j]);
      df_acc(ay, di22, t1[j]);
      df_acc(ay, di32, t2[j]);
      df_acc(az, di13, t0[j]);
      df_acc(az, di23, t1[j]);
      df_acc(az, di33, t2[j]);
      const Df2 gx = df_norm(ax), gy = df_norm(ay), gz = df_norm(az);
      DfAcc av{0.0f, 0.0f};
      df_acc(av, vxd, gx);
      df_acc(av, vyd, gy);
      df_acc(av, vzd, gz);
      const Df2 vg = df_norm(av);
      DfAcc aw{0.0f, 0.0f}, aa = av;
      df_acc_add(aw, tn[j]);
      df_acc(aw, taud, vg);
      df_acc(aa, pd, tn[j]);
      sm.g[le][lane8][0][j] = gx;
      sm.g[le][lane8][1][j] = gy;
      sm.g[le][lane8][2][j] = gz;
      if constexpr (SPLIT) {
        sm.g[le][lane8][3][j] = df_norm(aa);
      } else {  // aH (v.gradN_j + P N_j) + aM N_j
        DfAcc bw{0.0f, 0.0f};
        df_acc(bw, aHd, df_norm(aa));
        df_acc(bw, aMd, tn[j]);
        sm.g[le][lane8][3][j] = df_norm(bw);
      }
      sm.g[le][lane8][4][j] = df_norm(aw);
    }
    const double vol = group8_sum<double>(detj);
    sm.d[le][lane8][0] = detp;
    {
      const Df2 lamd = df_from_double_chk(lam, range_bad);
      sm.d[le][lane8][1] = df_mul(SPLIT ? lamd : df_mul(aHd, lamd), detp);
    }
    if (robin && lane8 < 4) {
      // face-3 point lane8 (Robin term) in FP64 from the element's
      // coordinates relative to local node 1
      double xe[8], ye[8], ze[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int n = __ldg(a.conn + (size_t)k * E + p) & NODE_BITS;
        xe[k] = __ldg(a.xx + n) - x0;
        ye[k] = __ldg(a.yy + n) - y0;
        ze[k] = __ldg(a.zz + n) - z0;
      }
      const double gc = VDR_GAUSS_C;
      const double rr = (lane8 & 2) ? gc : -gc;
      const double ss = (lane8 & 1) ? gc : -gc;
      const double djs = face3_detjs<double>(xe, ye, ze, rr, ss);
      double n[8], d0[8], d1[8], d2[8];
      shape_at<double>(-1.0, rr, ss, n, d0, d1, d2);
      GPData<double> o;
      gp_core<double>(a.variant, n, d0, d1, d2, xe, ye, ze, lam, vx, vy, vz, o);
#pragma unroll
      for (int j = 0; j < 8; j++) sm.fw[le][lane8][j] = df_from_double_chk(o.w[j], range_bad);
      sm.fd[le][lane8] = df_from_double_chk(a.f.robin_alpha * djs, range_bad);
    }
    __syncwarp();
    // ---- lane i = row i
    const int i = lane8;
    // accH: H (SPLIT) or A_e; accM: M (SPLIT only)
    DfAcc accH[8], accM[SPLIT ? 8 : 1];
#pragma unroll
    for (int j = 0; j < 8; j++) accH[j] = DfAcc{0.0f, 0.0f};
#pragma unroll
    for (int j = 0; j < (SPLIT ? 8 : 1); j++) accM[j] = DfAcc{0.0f, 0.0f};
    DfAcc fw{0.0f, 0.0f};
#pragma unroll 1
    for (int q = 0; q < 8; q++) {
      const Df2 dj = sm.d[le][q][0];
      const Df2 wd = df_mul(sm.g[le][q][4][i], dj);
      df_acc_add(fw, wd);
      if (!need_rows) continue;
      const Df2 dl = sm.d[le][q][1];
      const Df2 dgx = df_mul(dl, sm.g[le][q][0][i]);
      const Df2 dgy = df_mul(dl, sm.g[le][q][1][i]);
      const Df2 dgz = df_mul(dl, sm.g[le][q][2][i]);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        df_acc(accH[j], dgx, sm.g[le][q][0][j]);
        df_acc(accH[j], dgy, sm.g[le][q][1][j]);
        df_acc(accH[j], dgz, sm.g[le][q][2][j]);
        df_acc(accH[j], wd, sm.g[le][q][3][j]);
        if constexpr (SPLIT) df_acc(accM[j], wd, sm.tab[q][0][j]);
      }
    }
    if (robin && need_rows) {
#pragma unroll
      for (int f = 0; f < 4; f++) {
        Df2 aw = df_mul(sm.fd[le][f], sm.fw[le][f][i]);
        if constexpr (!SPLIT) aw = df_mul(aHd, aw);
#pragma unroll
        for (int j = 0; j < 8; j++) df_acc(accH[j], aw, sm.ftab[f][j]);
      }
    }
    if (!valid) continue;
    const double qe = (a.f.q && (ba.f || ba.b)) ? __ldg(a.f.q + p) : 0.0;
    df_rows_out<SPLIT>(a, ba, p, i, ck, accH, accM, fw, qe, vol, aHd, aMd, nrMd, sm.told[le],
                       tshift);
  }
  // Any out-of-window value: the host redoes this build with the FP64 rows
  // (bit 2 of the flag).
  if (range_bad) atomicOr(ba.bad, 2);
}

// ---- geometric factors of the double-float build, once per mesh
struct GeoSmem {
  Df2 g[ROWS_EPB][8][3][8];  // per element, point q, node j: dNj/dx, dNj/dy, dNj/dz
  Df2 dj[ROWS_EPB][8];       // detJ at point q
  Df2 rel[ROWS_EPB][24];     // node k's (x, y, z) - node 1's at [3k..3k+2]
  Df2 tab[8][4][8];          // N, dN/dxi, dN/deta, dN/dzeta at the 8 points
};

// Per element on 8 lanes: lane q forms J^-1 and detJ at Gauss point q
// (the same double-float evaluation as elem_build_df_kernel) and the
// physical gradients of the 8 shape functions there; lane i then forms
// K_ij = sum_q detJ_q gradN_i . gradN_j for j >= i.
__global__ void __launch_bounds__(64) geo_factors_kernel(OpArgs a, GeoFactors g, int *bad) {
  __shared__ GeoSmem sm;
  fill_df_tables(sm.tab, nullptr);
  const int lane8 = threadIdx.x & 7;
  const int le = threadIdx.x >> 3;
  const long E = a.E;
  bool range_bad = false;
  for (long base = (long)blockIdx.x * ROWS_EPB; base < E;
       base += (long)gridDim.x * ROWS_EPB) {
    const long pe = base + le;
    const bool valid = pe < E;
    const long p = valid ? pe : E - 1;
    __syncwarp();  // the previous element's shared data has been read
    // ---- lane k = node k
    const int nk = __ldg(a.conn + (size_t)lane8 * E + p) & NODE_BITS;
    const double xk = __ldg(a.xx + nk), yk = __ldg(a.yy + nk), zk = __ldg(a.zz + nk);
    const double x0 = __shfl_sync(FULL, xk, 0, 8);
    const double y0 = __shfl_sync(FULL, yk, 0, 8);
    const double z0 = __shfl_sync(FULL, zk, 0, 8);
    sm.rel[le][3 * lane8] = df_from_double_chk(xk - x0, range_bad);
    sm.rel[le][3 * lane8 + 1] = df_from_double_chk(yk - y0, range_bad);
    sm.rel[le][3 * lane8 + 2] = df_from_double_chk(zk - z0, range_bad);
    __syncwarp();
    // ---- lane q = Gauss point q
    const int q = lane8;
    const Df2 *t0 = sm.tab[q][1], *t1 = sm.tab[q][2], *t2 = sm.tab[q][3];
    Df2 di[9];
    double detj;
    const Df2 detp = df_inverse_jacobian(sm.rel[le], t0, t1, t2, di, detj, range_bad);
    if (valid) {
#pragma unroll
      for (int k = 0; k < 9; k++) g.Ji[(size_t)(9 * q + k) * E + p] = make_float2(di[k].h, di[k].l);
      g.Dj[(size_t)q * E + p] = make_float2(detp.h, detp.l);
    }
#pragma unroll 2
    for (int j = 0; j < 8; j++) {
      DfAcc ax{0.0f, 0.0f}, ay{0.0f, 0.0f}, az{0.0f, 0.0f};
      df_acc(ax, di[0], t0[j]);
      df_acc(ax, di[3], t1[j]);
      df_acc(ax, di[6], t2[j]);
      df_acc(ay, di[1], t0[j]);
      df_acc(ay, di[4], t1[j]);
      df_acc(ay, di[7], t2[j]);
      df_acc(az, di[2], t0[j]);
      df_acc(az, di[5], t1[j]);
      df_acc(az, di[8], t2[j]);
      sm.g[le][q][0][j] = df_norm(ax);
      sm.g[le][q][1][j] = df_norm(ay);
      sm.g[le][q][2][j] = df_norm(az);
    }
    sm.dj[le][q] = detp;
    __syncwarp();
    // ---- lane i = row i of K (the upper triangle is stored)
    const int i = lane8;
    DfAcc acc[8];
#pragma unroll
    for (int j = 0; j < 8; j++) acc[j] = DfAcc{0.0f, 0.0f};
#pragma unroll 1
    for (int r = 0; r < 8; r++) {
      const Df2 dj = sm.dj[le][r];
      const Df2 dgx = df_mul(dj, sm.g[le][r][0][i]);
      const Df2 dgy = df_mul(dj, sm.g[le][r][1][i]);
      const Df2 dgz = df_mul(dj, sm.g[le][r][2][i]);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        df_acc(acc[j], dgx, sm.g[le][r][0][j]);
        df_acc(acc[j], dgy, sm.g[le][r][1][j]);
        df_acc(acc[j], dgz, sm.g[le][r][2][j]);
      }
    }
    if (!valid) continue;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if (j < i) continue;
      const Df2 k = df_norm(acc[j]);
      g.K[(size_t)(i * (15 - i) / 2 + j) * E + p] = make_float2(k.h, k.l);
    }
  }
  if (range_bad) atomicOr(bad, 2);
}

__device__ __forceinline__ Df2 ld_pair(const float2 *p) {
  const float2 v = __ldg(p);
  return Df2{v.x, v.y};
}

// Per-element scalars of the geometric-factor build as double-float pairs,
// one thread per element in FP64 (the operations of elem_dr_scalars_kernel):
// sc[k E + p] for k = 0..2 velocity, 3 lambda, 4 decay rate; OT: 5 tau; GP
// and VF: 5..7 e = v/|v|, 8 kpe = |v|/(2 lambda_s), 9 khalf = 0.5/|v| (kpe
// and khalf zero where Pe is zero at every point).  A value outside the
// pairs' safe window sets bit 2 of *bad (the source stays FP64: its
// Gaussian tails reach far below that window).
__global__ void __launch_bounds__(256) elem_geo_scalars_kernel(OpArgs a, float2 *__restrict__ sc,
                                                               int *bad) {
  const long E = a.E;
  const double eps = 1.0e-14;
  bool range_bad = false;
  auto put = [&](int k, long p, double v, bool chk) {
    const Df2 d = chk ? df_from_double_chk(v, range_bad) : df_from_double(v);
    sc[(size_t)k * E + p] = make_float2(d.h, d.l);
  };
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < E;
       p += (long)gridDim.x * blockDim.x) {
    const double vx = __ldg(a.f.vel + p), vy = __ldg(a.f.vel + E + p),
                 vz = __ldg(a.f.vel + 2 * E + p);
    const double lam = __ldg(a.f.lam + p);
    put(0, p, vx, true);
    put(1, p, vy, true);
    put(2, p, vz, true);
    put(3, p, lam, true);
    put(4, p, a.f.pdec ? __ldg(a.f.pdec + p) : 0.0, true);
    const double vmag = sqrt(vx * vx + vy * vy + vz * vz);
    if (a.variant == DR_OT) {
      const int n0 = __ldg(a.conn + p) & NODE_BITS;
      const int n1 = __ldg(a.conn + (size_t)1 * E + p) & NODE_BITS;
      const int n3 = __ldg(a.conn + (size_t)3 * E + p) & NODE_BITS;
      const int n4 = __ldg(a.conn + (size_t)4 * E + p) & NODE_BITS;
      const double h = dr_h_axes<double>(
          vx, vy, vz, vmag, fabs(__ldg(a.xx + n1) - __ldg(a.xx + n0)),
          fabs(__ldg(a.yy + n3) - __ldg(a.yy + n0)),
          fabs(__ldg(a.zz + n4) - __ldg(a.zz + n0)));
      put(5, p, dr_tau_from<double>(DR_OT, h, vmag, lam), true);
    } else {
      double ex = 0.0, ey = 0.0, ez = 0.0, iv = 0.0;
      if (vmag > eps) {
        iv = 1.0 / vmag;
        ex = vx * iv;
        ey = vy * iv;
        ez = vz * iv;
      }
      const double lams =
          (a.variant == DR_VF) ? (lam * ex * ex + lam * ey * ey + lam * ez * ez) : lam;
      const bool on = vmag > eps && lams > eps;
      put(5, p, ex, false);
      put(6, p, ey, false);
      put(7, p, ez, false);
      put(8, p, on ? vmag / (2.0 * lams) : 0.0, true);
      put(9, p, on ? 0.5 * iv : 0.0, true);
    }
  }
  if (range_bad) atomicOr(bad, 2);
}

// 1/sqrt(a) for a positive normal pair: the FP32 estimate refined once in
// FP32 and once in double-float (Newton's y (3 - a y^2) / 2 with the
// residual 1 - a y^2 formed from the exact square of y); relative error
// ~2^-47.
__device__ __forceinline__ Df2 df_rsqrt(Df2 a) {
  float y = rsqrtf(a.h);
  y = __fmul_rn(y, __fmaf_rn(-0.5f * a.h * y, y, 1.5f));
  const float p = __fmul_rn(y, y);
  const Df2 r = df_sub(Df2{1.0f, 0.0f}, df_mul(a, Df2{p, __fmaf_rn(y, y, -p)}));
  const float c = __fmul_rn(0.5f * y, r.h);
  const float s = __fadd_rn(y, c);
  return Df2{s, __fsub_rn(c, __fsub_rn(s, y))};
}

// tau at one Gauss point from the pair scalars of elem_geo_scalars_kernel,
// di = J^-1 at the point: as df_point_tau with h = 2/|J^-1 e|, Pe = h kpe
// and h khalf in double-float.
__device__ __forceinline__ Df2 df_point_tau_pairs(int variant, const float2 *sc, long E,
                                                  long p, const Df2 (&di)[9],
                                                  bool &range_bad) {
  const Df2 zero{0.0f, 0.0f};
  if (variant == DR_OT) return ld_pair(sc + 5 * E + p);
  const Df2 ex = ld_pair(sc + 5 * E + p), ey = ld_pair(sc + 6 * E + p),
            ez = ld_pair(sc + 7 * E + p);
  DfAcc gxa{0.0f, 0.0f}, gya{0.0f, 0.0f}, gza{0.0f, 0.0f};
  df_acc(gxa, di[0], ex);
  df_acc(gxa, di[1], ey);
  df_acc(gxa, di[2], ez);
  df_acc(gya, di[3], ex);
  df_acc(gya, di[4], ey);
  df_acc(gya, di[5], ez);
  df_acc(gza, di[6], ex);
  df_acc(gza, di[7], ey);
  df_acc(gza, di[8], ez);
  const Df2 gx = df_norm(gxa), gy = df_norm(gya), gz = df_norm(gza);
  DfAcc n2{0.0f, 0.0f};
  df_acc(n2, gx, gx);
  df_acc(n2, gy, gy);
  df_acc(n2, gz, gz);
  const Df2 g2 = df_norm(n2);
  if (!(g2.h > 1.0e-28f)) return zero;  // h = 0
  const Df2 rs = df_rsqrt(g2);
  const Df2 h{2.0f * rs.h, 2.0f * rs.l};
  Df2 pe = df_mul(h, ld_pair(sc + 8 * E + p));
  if (!(pe.h > 1.0e-12f)) return zero;
  const Df2 hk = df_mul(h, ld_pair(sc + 9 * E + p));
  if (variant == DR_VF) {
    if (!(pe.h < 1.0e30f)) pe = Df2{1.0e30f, 0.0f};  // beta = 1 - 1/Pe there
    return df_mul(hk, df_beta_vf(pe));
  }
  return df_from_double_chk(df_to_double(hk.h, hk.l) * beta_exp(df_to_double(pe.h, pe.l)),
                            range_bad);
}

struct GeoBuildSmem {
  // per element, point q, node j: detJ W_j and c_j (SPLIT: v.gradN_j + P N_j;
  // otherwise aH v.gradN_j + (aH P + aM) N_j), read by the row lanes two
  // nodes per 16-byte load
  __align__(16) Df2 dw[ROWS_EPB][8][8];
  __align__(16) Df2 c[ROWS_EPB][8][8];
  __align__(16) Df2 told[ROWS_EPB][8];  // T_old at the nodes times 2^-shift
  __align__(16) float4 qt[8][8][2];     // point q, node j: (N, dN/dxi), (dN/deta, dN/dzeta)
  __align__(16) Df2 nt[8][8];           // N_j at point q
};

// Two consecutive pairs (16-byte aligned) from shared memory.
__device__ __forceinline__ void lds_pairs(const Df2 *p, Df2 &a, Df2 &b) {
  const float4 v = *reinterpret_cast<const float4 *>(p);
  a = Df2{v.x, v.y};
  b = Df2{v.z, v.w};
}
__device__ __forceinline__ void sts_pairs(Df2 *p, Df2 a, Df2 b) {
  *reinterpret_cast<float4 *>(p) = make_float4(a.h, a.l, b.h, b.l);
}

// The double-float build from the mesh's geometric factors.  With
// a_j = v . gradN_j = (J^-1 v) . dN_j/dxi and W_j = N_j + tau a_j at each
// Gauss point,
//   H_ij = lambda K_ij + sum_q detJ W_i (a_j + P N_j),
//   M_ij = sum_q detJ W_i N_j
// (el3d's hma + hmav + cma and cman, vanadis_full_DR_OpenMP_timing.for:
// 431-610, the diffusion term's geometry K formed once per mesh); no Robin
// term (elements with a nonzero Robin coefficient take elem_build_df_kernel).
// Per element on 8 lanes: lane q forms point q's tau, J^-1 v and, per node,
// a_j and W_j (4 pair products); lane i accumulates row i, 1 + 8 pair
// products per entry (SPLIT: H and M apart, 1 + 16), then writes as
// elem_build_df_kernel does.  A value outside the pairs' safe window sets
// bit 2 of the flag (the host redoes the build with FP64 rows).
template <bool SPLIT>
__global__ void __launch_bounds__(64, SPLIT ? 12 : 16) elem_build_geo_kernel(OpArgs a, BuildArgs ba) {
  __shared__ GeoBuildSmem sm;
  if (threadIdx.x < 8) {
    const int t = threadIdx.x;
    double n[8], d0[8], d1[8], d2[8];
    shape_at<double>(gauss_coord<double>(t, 0), gauss_coord<double>(t, 1),
                     gauss_coord<double>(t, 2), n, d0, d1, d2);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const Df2 N = df_from_double(n[j]), a0 = df_from_double(d0[j]);
      const Df2 a1 = df_from_double(d1[j]), a2 = df_from_double(d2[j]);
      sm.qt[t][j][0] = make_float4(N.h, N.l, a0.h, a0.l);
      sm.qt[t][j][1] = make_float4(a1.h, a1.l, a2.h, a2.l);
      sm.nt[t][j] = N;
    }
  }
  __syncthreads();
  const int lane8 = threadIdx.x & 7;
  const int le = threadIdx.x >> 3;
  const long E = a.E;
  bool range_bad = false;
  const Df2 aHd = df_from_double_chk(ba.aH, range_bad);
  const Df2 aMd = df_from_double_chk(ba.aM, range_bad);
  const Df2 nrMd = df_neg(df_from_double_chk(SPLIT ? ba.rM : 0.0, range_bad));
  const bool need_rows = SPLIT || ba.Ahi || ba.A64 || ba.diag;
  const float2 *sc = ba.gsc;
  for (long base = (long)blockIdx.x * ROWS_EPB; base < E;
       base += (long)gridDim.x * ROWS_EPB) {
    const long pe = base + le;
    const bool valid = pe < E;
    const long p = valid ? pe : E - 1;
    __syncwarp();  // the previous element's shared data has been read
    // ---- lane k = node k
    const int ck = __ldg(a.conn + (size_t)lane8 * E + p);
    int tshift = 0;
    if (SPLIT && ba.told) {
      const double tk = __ldg(ba.told + (ck & NODE_BITS));
      int em = df_exp(tk);
      em = max(em, __shfl_xor_sync(FULL, em, 1));
      em = max(em, __shfl_xor_sync(FULL, em, 2));
      em = max(em, __shfl_xor_sync(FULL, em, 4));
      if (em == 0 && tk != 0.0) range_bad = true;  // all subnormal
      tshift = em - 1023;
      Df2 t;
      df_split(tk, t.h, t.l, range_bad, tshift);  // inf/NaN: bad
      sm.told[le][lane8] = t;
    }
    const Df2 vxd = ld_pair(sc + p), vyd = ld_pair(sc + E + p), vzd = ld_pair(sc + 2 * E + p);
    const Df2 pd = ld_pair(sc + 4 * E + p);
    // ---- lane q = Gauss point q
    const int q = lane8;
    Df2 di[9];
#pragma unroll
    for (int k = 0; k < 9; k++) di[k] = ld_pair(ba.gJi + (size_t)(9 * q + k) * E + p);
    const Df2 djq = ld_pair(ba.gDj + (size_t)q * E + p);
    const Df2 taud = df_point_tau_pairs(a.variant, sc, E, p, di, range_bad);
    Df2 w[3];  // J^-1 v
#pragma unroll
    for (int r = 0; r < 3; r++) {
      DfAcc acc{0.0f, 0.0f};
      df_acc(acc, di[3 * r], vxd);
      df_acc(acc, di[3 * r + 1], vyd);
      df_acc(acc, di[3 * r + 2], vzd);
      w[r] = df_norm(acc);
    }
    const Df2 cm = SPLIT ? pd : df_add(df_mul(aHd, pd), aMd);
#pragma unroll 1
    for (int j = 0; j < 8; j += 2) {
      Df2 dwv[2], cv[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const float4 u0 = sm.qt[q][j + h][0], u1 = sm.qt[q][j + h][1];
        const Df2 N{u0.x, u0.y};
        DfAcc aa{0.0f, 0.0f};
        df_acc(aa, w[0], Df2{u0.z, u0.w});
        df_acc(aa, w[1], Df2{u1.x, u1.y});
        df_acc(aa, w[2], Df2{u1.z, u1.w});
        const Df2 av = df_norm(aa);
        DfAcc aw{0.0f, 0.0f};
        df_acc_add(aw, N);
        df_acc(aw, taud, av);
        dwv[h] = df_mul(djq, df_norm(aw));
        DfAcc ac{0.0f, 0.0f};
        if constexpr (SPLIT)
          df_acc_add(ac, av);
        else
          df_acc(ac, aHd, av);
        df_acc(ac, cm, N);
        cv[h] = df_norm(ac);
      }
      sts_pairs(&sm.dw[le][q][j], dwv[0], dwv[1]);
      sts_pairs(&sm.c[le][q][j], cv[0], cv[1]);
    }
    // element volume as a pair (the same sum in every lane: TwoSum is exact
    // in either order)
    Df2 vol = djq;
#pragma unroll
    for (int m = 1; m < 8; m <<= 1)
      vol = df_add(vol, Df2{__shfl_xor_sync(FULL, vol.h, m), __shfl_xor_sync(FULL, vol.l, m)});
    __syncwarp();
    // ---- lane i = row i
    const int i = lane8;
    DfAcc accH[8], accM[SPLIT ? 8 : 1];
#pragma unroll
    for (int j = 0; j < 8; j++) accH[j] = DfAcc{0.0f, 0.0f};
#pragma unroll
    for (int j = 0; j < (SPLIT ? 8 : 1); j++) accM[j] = DfAcc{0.0f, 0.0f};
    DfAcc fw{0.0f, 0.0f};
    if (need_rows) {
      const Df2 lamd = ld_pair(sc + 3 * E + p);
      const Df2 lk = SPLIT ? lamd : df_mul(aHd, lamd);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int t = (j >= i) ? i * (15 - i) / 2 + j : j * (15 - j) / 2 + i;
        df_acc(accH[j], lk, ld_pair(ba.gK + (size_t)t * E + p));
      }
    }
#pragma unroll 1
    for (int r = 0; r < 8; r++) {
      const Df2 dwi = sm.dw[le][r][i];
      df_acc_add(fw, dwi);
      if (!need_rows) continue;
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        Df2 c0, c1;
        lds_pairs(&sm.c[le][r][j], c0, c1);
        df_acc(accH[j], dwi, c0);
        df_acc(accH[j + 1], dwi, c1);
        if constexpr (SPLIT) {
          Df2 n0, n1;
          lds_pairs(&sm.nt[r][j], n0, n1);
          df_acc(accM[j], dwi, n0);
          df_acc(accM[j + 1], dwi, n1);
        }
      }
    }
    if (!valid) continue;
    const double qe = (a.f.q && (ba.f || ba.b)) ? __ldg(a.f.q + p) : 0.0;
    df_rows_out<SPLIT>(a, ba, p, i, ck, accH, accM, fw, qe, df_to_double(vol.h, vol.l), aHd,
                       aMd, nrMd, sm.told[le],
                       tshift);
  }
  if (range_bad) atomicOr(ba.bad, 2);
}

template <typename T, bool TRANS>
__global__ void __launch_bounds__(256) mf_apply_kernel(
    OpArgs a, T c1, T c2, const double *__restrict__ x, double *__restrict__ y,
    const int *skip, const int *skip2) {
  if (skip && *(volatile const int *)skip) return;
  if (skip2 && *(volatile const int *)skip2) return;
  const int lane8 = threadIdx.x & 7;
  const long E = a.E;
  const long groups_per_block = blockDim.x >> 3;
  for (long base = (long)blockIdx.x * groups_per_block; base < E;
       base += (long)gridDim.x * groups_per_block) {
    const long pe = base + (threadIdx.x >> 3);
    const bool valid = pe < E;
    const long p = valid ? pe : E - 1;
    Elem<T> el;
    load_elem<T>(a, p, el);
    T xv[8];
#pragma unroll
    for (int j = 0; j < 8; j++)
      xv[j] = el.c[j] < 0 ? T(0) : (T)__ldg(x + el.c[j]);
    GPData<T> o;
    gp_eval<T>(a.variant, gauss_coord<T>(lane8, 0), gauss_coord<T>(lane8, 1),
               gauss_coord<T>(lane8, 2), el.xe, el.ye, el.ze, el.lam, el.vx,
               el.vy, el.vz, o);
    const T cm = c1 * el.pdec + c2;
    const T dl = c1 * el.lam * o.detj;
    T con[8];
    if (!TRANS) {
      T u = 0, gu = 0, hu = 0, ku = 0;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        u += o.n[j] * xv[j];
        gu += o.gx[j] * xv[j];
        hu += o.gy[j] * xv[j];
        ku += o.gz[j] * xv[j];
      }
      const T t = o.detj * (c1 * (el.vx * gu + el.vy * hu + el.vz * ku) + cm * u);
#pragma unroll
      for (int i = 0; i < 8; i++)
        con[i] = dl * (o.gx[i] * gu + o.gy[i] * hu + o.gz[i] * ku) + o.w[i] * t;
    } else {
      T ws = 0, gu = 0, hu = 0, ku = 0;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        ws += o.w[i] * xv[i];
        gu += o.gx[i] * xv[i];
        hu += o.gy[i] * xv[i];
        ku += o.gz[i] * xv[i];
      }
      const T dw = o.detj * ws;
#pragma unroll
      for (int j = 0; j < 8; j++)
        con[j] = dl * (o.gx[j] * gu + o.gy[j] * hu + o.gz[j] * ku) +
                 dw * (c1 * (el.vx * o.gx[j] + el.vy * o.gy[j] + el.vz * o.gz[j]) +
                       cm * o.n[j]);
    }
    if (el.robin && lane8 < 4) {
      const T gc = T(VDR_GAUSS_C);
      const T r = (lane8 & 2) ? gc : -gc;
      const T s = (lane8 & 1) ? gc : -gc;
      const T ca = c1 * T(a.f.robin_alpha) * face3_detjs<T>(el.xe, el.ye, el.ze, r, s);
      gp_eval<T>(a.variant, T(-1), r, s, el.xe, el.ye, el.ze, el.lam, el.vx,
                 el.vy, el.vz, o);
      if (!TRANS) {
        T uf = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) uf += o.n[j] * xv[j];
#pragma unroll
        for (int i = 0; i < 8; i++) con[i] += ca * o.w[i] * uf;
      } else {
        T wf = 0;
#pragma unroll
        for (int i = 0; i < 8; i++) wf += o.w[i] * xv[i];
#pragma unroll
        for (int j = 0; j < 8; j++) con[j] += ca * o.n[j] * wf;
      }
    }
    const T mine = group8_reduce_scatter<T>(con, lane8);
    const int cme = el.c[lane8];
    if (valid && cme >= 0) atomicAdd(y + cme, (double)mine);
  }
}

// integrate_mass_hex8's per-element weights w_s = sum_q N_s(q) detJ_q
// (2x2x2 Gauss, abscissa 1/sqrt(3), FP64), stored [8][E]: the geometry of a
// handle is fixed, so they are formed once and every later integral is
// sum_e sum_s w_s c_s (mass_dot_kernel).
__global__ void __launch_bounds__(256) mass_weights_kernel(
    const int *__restrict__ conn, int E, const double *__restrict__ xx,
    const double *__restrict__ yy, const double *__restrict__ zz,
    double *__restrict__ w) {
  const double g = 1.0 / sqrt(3.0);
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < E;
       p += (long)gridDim.x * blockDim.x) {
    double xe[8], ye[8], ze[8], ws[8];
#pragma unroll
    for (int s = 0; s < 8; s++) {
      const int n = __ldg(conn + (size_t)s * E + p) & NODE_BITS;
      xe[s] = __ldg(xx + n);
      ye[s] = __ldg(yy + n);
      ze[s] = __ldg(zz + n);
      ws[s] = 0.0;
    }
#pragma unroll 1
    for (int q = 0; q < 8; q++) {
      const double xi = ((q >> 2) & 1) ? g : -g;
      const double eta = ((q >> 1) & 1) ? g : -g;
      const double zeta = (q & 1) ? g : -g;
      double n[8], d0[8], d1[8], d2[8];
      shape_at<double>(xi, eta, zeta, n, d0, d1, d2);
      double j11 = 0, j12 = 0, j13 = 0, j21 = 0, j22 = 0, j23 = 0, j31 = 0,
             j32 = 0, j33 = 0;
#pragma unroll
      for (int s = 0; s < 8; s++) {
        j11 += xe[s] * d0[s];
        j12 += xe[s] * d1[s];
        j13 += xe[s] * d2[s];
        j21 += ye[s] * d0[s];
        j22 += ye[s] * d1[s];
        j23 += ye[s] * d2[s];
        j31 += ze[s] * d0[s];
        j32 += ze[s] * d1[s];
        j33 += ze[s] * d2[s];
      }
      const double detj = j11 * (j22 * j33 - j23 * j32) -
                          j12 * (j21 * j33 - j23 * j31) +
                          j13 * (j21 * j32 - j22 * j31);
#pragma unroll
      for (int s = 0; s < 8; s++) ws[s] += n[s] * detj;
    }
#pragma unroll
    for (int s = 0; s < 8; s++) w[(size_t)s * E + p] = ws[s];
  }
}

// sum_e sum_s w_s c_s: one thread per element, block partials summed in
// fixed order by the launcher's second kernel (deterministic).
__global__ void __launch_bounds__(256) mass_dot_kernel(
    const int *__restrict__ conn, int E, const double *__restrict__ w,
    const double *__restrict__ c, double *__restrict__ partials) {
  double acc = 0.0;
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < E;
       p += (long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int s = 0; s < 8; s++) {
      const int n = __ldg(conn + (size_t)s * E + p) & NODE_BITS;
      acc += __ldg(w + (size_t)s * E + p) * __ldg(c + n);
    }
  }
  __shared__ double sm[256];
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if (threadIdx.x < off) sm[threadIdx.x] += sm[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sm[0];
}

// integrate_mass_hex8: one thread per element, 2x2x2 Gauss with
// abscissa 1/sqrt(3); block partials summed in fixed order by the host
// launcher's second kernel.
__global__ void __launch_bounds__(256) mass_kernel(
    const int *__restrict__ conn, int E, const double *__restrict__ xx,
    const double *__restrict__ yy, const double *__restrict__ zz,
    const double *__restrict__ c, double *__restrict__ partials) {
  const double g = 1.0 / sqrt(3.0);
  double acc = 0.0;
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < E;
       p += (long)gridDim.x * blockDim.x) {
    double xe[8], ye[8], ze[8], ce[8];
#pragma unroll
    for (int s = 0; s < 8; s++) {
      const int n = __ldg(conn + (size_t)s * E + p) & NODE_BITS;
      xe[s] = __ldg(xx + n);
      ye[s] = __ldg(yy + n);
      ze[s] = __ldg(zz + n);
      ce[s] = __ldg(c + n);
    }
#pragma unroll 1
    for (int q = 0; q < 8; q++) {
      GPData<double> o;
      const double xi = ((q >> 2) & 1) ? g : -g;
      const double eta = ((q >> 1) & 1) ? g : -g;
      const double zeta = (q & 1) ? g : -g;
      // DR weights are not needed: zero velocity keeps W = N.
      gp_eval<double>(VDR_DR_VF, xi, eta, zeta, xe, ye, ze, 1.0, 0.0, 0.0, 0.0, o);
      double cv = 0.0;
#pragma unroll
      for (int s = 0; s < 8; s++) cv += o.n[s] * ce[s];
      acc += cv * o.detj;
    }
  }
  __shared__ double sm[256];
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if (threadIdx.x < off) sm[threadIdx.x] += sm[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sm[0];
}

__global__ void sum_partials_kernel(const double *__restrict__ partials, int n,
                                    double *__restrict__ out) {
  __shared__ double sm[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partials[i];
  sm[threadIdx.x] = acc;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if (threadIdx.x < off) sm[threadIdx.x] += sm[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

}  // namespace

cudaError_t launch_build(const OpArgs &a, const BuildArgs &ba, bool fp32,
                         cudaStream_t s) {
  if (a.E <= 0) return cudaSuccess;
  const long blocks_needed = ((long)a.E + ROWS_EPB - 1) / ROWS_EPB;
  const int grid = (int)std::min<long>(blocks_needed, (long)device_sm_count() * 32);
  if (fp32)
    elem_build_kernel<float><<<grid, 64, 0, s>>>(a, ba);
  else if (ba.exact_fp64)
    elem_build_kernel<double><<<grid, 64, 0, s>>>(a, ba);
  else {
    if (ba.gK ? !ba.gsc : !ba.drs) return cudaErrorInvalidValue;
    static std::once_flag carveout;  // 8 blocks of 27.5 KB need the full carveout,
    std::call_once(carveout, [] {
      cudaFuncSetAttribute(elem_build_df_kernel<true>,
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      cudaFuncSetAttribute(elem_build_df_kernel<false>,
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      // 12 / 16 blocks of 10.5 KB
      cudaFuncSetAttribute(elem_build_geo_kernel<true>,
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      cudaFuncSetAttribute(elem_build_geo_kernel<false>,
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    });
    const int g2 = (int)std::min<long>(((long)a.E + 255) / 256, (long)device_sm_count() * 8);
    if (ba.gK) {  // from the mesh's geometric factors
      elem_geo_scalars_kernel<<<g2, 256, 0, s>>>(a, ba.gsc, ba.bad);
      if (ba.told || ba.Mhi)
        elem_build_geo_kernel<true><<<grid, 64, 0, s>>>(a, ba);
      else
        elem_build_geo_kernel<false><<<grid, 64, 0, s>>>(a, ba);
    } else {
      elem_dr_scalars_kernel<<<g2, 256, 0, s>>>(a, ba.drs);
      if (ba.told || ba.Mhi)  // H and M apart
        elem_build_df_kernel<true><<<grid, 64, 0, s>>>(a, ba);
      else
        elem_build_df_kernel<false><<<grid, 64, 0, s>>>(a, ba);
    }
    count_launches(1);
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t diag_beta_vf(int n, const double *pe, double *beta) {
  if (n <= 0) return cudaSuccess;
  double *d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * 2 * (size_t)n);
  if (e) return e;
  if (!(e = cudaMemcpy(d, pe, sizeof(double) * n, cudaMemcpyHostToDevice))) {
    beta_vf_kernel<<<(n + 127) / 128, 128>>>(n, d, d + n);
    count_launches(1);
    if (!(e = cudaGetLastError()))
      e = cudaMemcpy(beta, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  }
  cudaFree(d);
  return e;
}

cudaError_t launch_geo_factors(const OpArgs &a, const GeoFactors &g, int *bad,
                               cudaStream_t s) {
  if (a.E <= 0) return cudaSuccess;
  const long blocks_needed = ((long)a.E + ROWS_EPB - 1) / ROWS_EPB;
  const int grid = (int)std::min<long>(blocks_needed, (long)device_sm_count() * 32);
  geo_factors_kernel<<<grid, 64, 0, s>>>(a, g, bad);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mf_apply(const OpArgs &a, bool fp32, bool transpose,
                            const double *x, double *y, const int *skip,
                            const int *skip2, cudaStream_t s) {
  if (a.E <= 0) return cudaSuccess;
  const long blocks_needed = ((long)a.E + 31) / 32;
  const int grid = (int)std::min<long>(blocks_needed, (long)device_sm_count() * 8);
  if (fp32) {
    if (transpose)
      mf_apply_kernel<float, true><<<grid, 256, 0, s>>>(a, (float)a.aH, (float)a.aM, x, y, skip, skip2);
    else
      mf_apply_kernel<float, false><<<grid, 256, 0, s>>>(a, (float)a.aH, (float)a.aM, x, y, skip, skip2);
  } else {
    if (transpose)
      mf_apply_kernel<double, true><<<grid, 256, 0, s>>>(a, a.aH, a.aM, x, y, skip, skip2);
    else
      mf_apply_kernel<double, false><<<grid, 256, 0, s>>>(a, a.aH, a.aM, x, y, skip, skip2);
  }
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mass(Handle &h, const double *c, double *partials,
                        double *out, cudaStream_t s) {
  const int grid = std::max(1, std::min((h.E + 255) / 256, device_sm_count() * 4));
  if (!h.massw) {  // per-element weights, once per handle (fixed geometry)
    cudaError_t e = cudaMalloc(&h.massw, sizeof(double) * 8 * (size_t)std::max(h.E, 1));
    if (e) {
      h.massw = nullptr;
      // no room for the weights: integrate directly
      mass_kernel<<<grid, 256, 0, s>>>(h.conn, h.E, h.xx, h.yy, h.zz, c, partials);
      sum_partials_kernel<<<1, 256, 0, s>>>(partials, grid, out);
      count_launches(2);
      cudaGetLastError();  // the allocation failure is not an error here
      return cudaGetLastError();
    }
    mass_weights_kernel<<<grid, 256, 0, s>>>(h.conn, h.E, h.xx, h.yy, h.zz, h.massw);
    count_launches(1);
  }
  mass_dot_kernel<<<grid, 256, 0, s>>>(h.conn, h.E, h.massw, c, partials);
  sum_partials_kernel<<<1, 256, 0, s>>>(partials, grid, out);
  count_launches(2);
  return cudaGetLastError();
}

}  // namespace vdr
