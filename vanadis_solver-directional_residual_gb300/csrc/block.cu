// block.cu -- many right-hand sides with one operator (K <= 64 columns).
//
// Block vectors are node-major, X[n*K + k], so the K values a node carries
// are contiguous.  One warp handles one element at a time:
//
//   block_apply_tf32  Y^T (K x 8) += X_e^T (K x 8) . A_e^T (8 x 8) on the
//                     tensor cores, mma.sync m16n8k8 TF32 (one MMA per 16
//                     columns); FP32 vectors; A_e read from an element-major
//                     FP32 copy (256 contiguous bytes per element and warp),
//                     so the element matrices stream once for all K columns.
//   block_apply_df    the FP64-accurate apply for the refinement residual:
//                     lane = column, double-float contraction of the pair
//                     store (FP32 pipe), FP64 vectors.
//
// The inner solver is K independent Jacobi-BiCGStab iterations sharing every
// launch: per-column scalars (rho, alpha, omega, norms) in FP64, per-column
// deterministic reductions, and a per-column "active" flag that freezes a
// column once it meets its tolerance.  The outer loop refines each column
// in FP64 (residual and update), as the single-RHS mixed solver does.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "dfloat.cuh"
#include "vdr_internal.h"

namespace vdr {
namespace {

constexpr int BT = 256;  // threads per block of the block-vector kernels
constexpr unsigned FULL = 0xffffffffu;

int sm_count_b() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

// --------------------------------------------------------------- applies
__device__ __forceinline__ unsigned to_tf32(float f) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(f));
  return r;
}

// SoA pair store hi part -> element-major FP32 copy Aaos[p*64 + 8i + j].
__global__ void aos_from_hi(const float4 *__restrict__ Ahi, int E,
                            float4 *__restrict__ Aaos) {
  const long total = (long)E * 16;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long p = t >> 4;
    const int chunk = (int)(t & 15);  // = 2i + h
    Aaos[t] = Ahi[(size_t)chunk * E + p];
  }
}

// SoA FP64 pair store -> element-major FP32 copy.
__global__ void aos_from_f64(const double2 *__restrict__ A64, int E,
                             float4 *__restrict__ Aaos) {
  const long total = (long)E * 16;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long p = t >> 4;
    const int chunk = (int)(t & 15);
    const double2 a = A64[(size_t)(2 * chunk) * E + p];
    const double2 b = A64[(size_t)(2 * chunk + 1) * E + p];
    Aaos[t] = make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y);
  }
}

// K = 16 * tiles columns.  Warp per element; lane = (g = lane/4, t = lane%4)
// in the m16n8k8 fragment layout: the MMA's M dimension is the column k
// (16 per tile), N the element's output node i, K its input node j, so
// D[k][i] += sum_j X[node j][k] * A[i][j].  SPLIT: each operand is split
// into a TF32 head and a TF32 tail and three MMAs (hi.hi + hi.lo + lo.hi)
// give FP32-level products; the apply is bound by memory traffic, so the
// extra MMAs cost little.
template <bool SPLIT>
__global__ void __launch_bounds__(256) block_apply_tf32(
    const float *__restrict__ Aaos, const int *__restrict__ conn, int E, int K,
    const float *__restrict__ X, float *__restrict__ Y, const int *skip) {
  if (skip && *(volatile const int *)skip) return;
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  const int tiles = K >> 4;
  for (long p = warp; p < E; p += nwarps) {
    const int cl = lane < 8 ? __ldg(conn + (size_t)lane * E + p) : 0;
    const int na = __shfl_sync(FULL, cl, t);          // A-fragment columns
    const int nb = __shfl_sync(FULL, cl, t + 4);
    const int o0 = __shfl_sync(FULL, cl, 2 * t);      // output rows
    const int o1 = __shfl_sync(FULL, cl, 2 * t + 1);
    const float *ae = Aaos + (size_t)p * 64;
    const float f0 = __ldg(ae + 8 * g + t), f1 = __ldg(ae + 8 * g + t + 4);
    const unsigned b0 = to_tf32(f0), b1 = to_tf32(f1);
    unsigned c0 = 0u, c1 = 0u;
    if (SPLIT) {
      c0 = to_tf32(f0 - __uint_as_float(b0));
      c1 = to_tf32(f1 - __uint_as_float(b1));
    }
    for (int m = 0; m < tiles; m++) {
      const int k0 = 16 * m + g, k1 = k0 + 8;
      float xa[4];
      xa[0] = na < 0 ? 0.f : __ldg(X + (size_t)na * K + k0);
      xa[1] = na < 0 ? 0.f : __ldg(X + (size_t)na * K + k1);
      xa[2] = nb < 0 ? 0.f : __ldg(X + (size_t)nb * K + k0);
      xa[3] = nb < 0 ? 0.f : __ldg(X + (size_t)nb * K + k1);
      unsigned ah[4], al[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        ah[q] = to_tf32(xa[q]);
        al[q] = SPLIT ? to_tf32(xa[q] - __uint_as_float(ah[q])) : 0u;
      }
      float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
      if (SPLIT) {
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
            : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
            : "r"(al[0]), "r"(al[1]), "r"(al[2]), "r"(al[3]), "r"(b0), "r"(b1));
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
            : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
            : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(c0), "r"(c1));
      }
      asm volatile(
          "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
          "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
          : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
          : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(b0), "r"(b1));
      if (o0 >= 0) {
        atomicAdd(Y + (size_t)o0 * K + k0, d0);
        atomicAdd(Y + (size_t)o0 * K + k1, d2);
      }
      if (o1 >= 0) {
        atomicAdd(Y + (size_t)o1 * K + k0, d1);
        atomicAdd(Y + (size_t)o1 * K + k1, d3);
      }
    }
  }
}

// FP64-accurate block apply over the pair store: warp per element, lane =
// columns lane, lane+32.  The element's 64 pairs are staged in shared memory.
__global__ void __launch_bounds__(256) block_apply_df(
    const float4 *__restrict__ Ahi, const float4 *__restrict__ Alo,
    const int *__restrict__ conn, int E, int K, const double *__restrict__ X,
    double *__restrict__ Y) {
  __shared__ float2 sa[8][64];  // per warp: (hi, lo) of entry 8i + j
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long p = warp; p < E; p += nwarps) {
    __syncwarp();
    if (lane < 16) {
      const float4 h = Ahi[(size_t)lane * E + p];
      const float4 l = Alo[(size_t)lane * E + p];
      sa[w][4 * lane + 0] = make_float2(h.x, l.x);
      sa[w][4 * lane + 1] = make_float2(h.y, l.y);
      sa[w][4 * lane + 2] = make_float2(h.z, l.z);
      sa[w][4 * lane + 3] = make_float2(h.w, l.w);
    }
    const int cl = lane < 8 ? __ldg(conn + (size_t)lane * E + p) : 0;
    int c[8];
#pragma unroll
    for (int s = 0; s < 8; s++) c[s] = __shfl_sync(FULL, cl, s);
    __syncwarp();
    for (int k = lane; k < K; k += 32) {
      double xv[8];
      int emax = 0;
#pragma unroll
      for (int s = 0; s < 8; s++) {
        xv[s] = c[s] < 0 ? 0.0 : X[(size_t)c[s] * K + k];
        emax = max(emax, df_exp(xv[s]));
      }
      const int shift = emax - 1023;
      float xh[8], xl[8];
      bool bad = false;
#pragma unroll
      for (int s = 0; s < 8; s++) df_split(xv[s], xh[s], xl[s], bad, shift);
      double out[8];
      if (bad) {  // inf/NaN input: plain FP64 from the merged pairs
#pragma unroll
        for (int i = 0; i < 8; i++) {
          double acc = 0.0;
#pragma unroll
          for (int j = 0; j < 8; j++)
            acc += df_to_double(sa[w][8 * i + j].x, sa[w][8 * i + j].y) * xv[j];
          out[i] = acc;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++) {
          DfAcc acc{0.f, 0.f};
#pragma unroll
          for (int j = 0; j < 8; j++)
            df_fma_acc(acc, sa[w][8 * i + j].x, sa[w][8 * i + j].y, xh[j], xl[j]);
          out[i] = df_to_double(acc.s, acc.c);
          if (!df_scale(out[i], shift)) out[i] = ldexp(out[i], shift);
        }
      }
#pragma unroll
      for (int s = 0; s < 8; s++)
        if (c[s] >= 0) atomicAdd(Y + (size_t)c[s] * K + k, out[s]);
    }
  }
}

// FP64 block apply from the FP64 store (used when the handle holds FP64).
__global__ void __launch_bounds__(256) block_apply_f64(
    const double2 *__restrict__ A64, const int *__restrict__ conn, int E, int K,
    const double *__restrict__ X, double *__restrict__ Y) {
  __shared__ double sa[8][64];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long p = warp; p < E; p += nwarps) {
    __syncwarp();
    {
      const double2 v = A64[(size_t)lane * E + p];
      sa[w][2 * lane] = v.x;
      sa[w][2 * lane + 1] = v.y;
    }
    const int cl = lane < 8 ? __ldg(conn + (size_t)lane * E + p) : 0;
    int c[8];
#pragma unroll
    for (int s = 0; s < 8; s++) c[s] = __shfl_sync(FULL, cl, s);
    __syncwarp();
    for (int k = lane; k < K; k += 32) {
      double xv[8];
#pragma unroll
      for (int s = 0; s < 8; s++) xv[s] = c[s] < 0 ? 0.0 : X[(size_t)c[s] * K + k];
#pragma unroll
      for (int i = 0; i < 8; i++) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < 8; j++) acc += sa[w][8 * i + j] * xv[j];
        if (c[i] >= 0) atomicAdd(Y + (size_t)c[i] * K + k, acc);
      }
    }
  }
}

// ---------------------------------------------------- block right-hand side
// B[n*K + k] += cf * Q[k*E + e] * phi[i*E + e] for the element's nodes.
__global__ void block_rhs(const double *__restrict__ phi,
                          const int *__restrict__ conn, int E, int K,
                          const double *__restrict__ Q,
                          const int *__restrict__ perm, double cf,
                          double *__restrict__ B) {
  const long total = (long)E * K;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t / K;
    const int k = (int)(t % K);
    const long ecaller = perm ? perm[e] : e;  // Q is in the caller's order
    const double qe = Q[(size_t)k * E + ecaller];
    if (qe == 0.0) continue;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int c = conn[(size_t)i * E + e];
      if (c >= 0) atomicAdd(B + (size_t)c * K + k, cf * qe * phi[(size_t)i * E + e]);
    }
  }
}

// ------------------------------------------------------ block Krylov state
struct BState {
  unsigned ticket;
  int done, iter, itmax;
  double tol;
};
// per-column arrays, each of length K (kept in one device buffer)
struct BCols {
  double *bnrm2, *err, *rho, *rho_old, *alpha, *omega, *snrm;
  int *active, *sconv, *status;
};

struct BVec {
  long n;  // N*K
  int K;
  BState *st;
  BCols c;
  double *partials;  // [q][k][block]
  const float *b, *dinv;  // dinv per node
  const unsigned char *m; // per node
  float *x, *r, *rh, *p, *v, *ph, *s, *sh, *t;
  const double *outer_err;  // per column FP64 residual of the refinement
  double outer_tol;         // columns already at outer_tol stay inactive
};

// Per-column block reduction: thread tid owns column tid % K (blockDim is a
// multiple of K, grid stride keeps the column).  Returns in threads
// tid < K the block's per-column sums of NQ quantities; then the last block
// sums the per-block partials of each column in fixed order.
template <int NQ, bool MAX = false>
__device__ __forceinline__ bool col_grid_sum(double (&v)[NQ], const BVec &a,
                                             double *out /* [NQ][K] */) {
  __shared__ double sm[NQ][BT];
  __shared__ bool last;
  const int K = a.K;
  for (int q = 0; q < NQ; q++) sm[q][threadIdx.x] = v[q];
  __syncthreads();
  if (threadIdx.x < K) {
    for (int q = 0; q < NQ; q++) {
      double s = 0.0;
      for (int r = threadIdx.x; r < BT; r += K)
        s = MAX ? fmax(s, sm[q][r]) : s + sm[q][r];
      a.partials[((size_t)q * K + threadIdx.x) * gridDim.x + blockIdx.x] = s;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&a.st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  if (threadIdx.x < K) {
    for (int q = 0; q < NQ; q++) {
      double s = 0.0;
      const double *pp = a.partials + ((size_t)q * K + threadIdx.x) * gridDim.x;
      for (unsigned b = 0; b < gridDim.x; b++)
        s = MAX ? fmax(s, __ldcg(pp + b)) : s + __ldcg(pp + b);
      out[q * K + threadIdx.x] = s;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) a.st->ticket = 0u;
  return threadIdx.x < K;
}

// Per-thread inner-product accumulation in double-float: exact FP32
// products (two-product) summed with TwoSum, i.e. FP64-accurate inner
// products without the FP64 pipe.
__device__ __forceinline__ void dot_acc(DfAcc &acc, float a, float b) {
  df_fma_acc(acc, a, 0.0f, b, 0.0f);
}
__device__ __forceinline__ double dot_val(const DfAcc &acc) {
  return df_to_double(acc.s, acc.c);
}

#define BLOOP(i)                                                      \
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; \
       i += (long)gridDim.x * blockDim.x)

// r = b - r (r holds A x); rh = r; per-column norms; columns with b = 0 are
// inactive from the start.
__global__ void __launch_bounds__(BT) bb_start(BVec a) {
  const int k = threadIdx.x % a.K;
  DfAcc d0{0.f, 0.f}, d1{0.f, 0.f};
  BLOOP(i) {
    const float bi = a.b[i];
    const float ri = bi - a.r[i];
    a.r[i] = ri;
    a.rh[i] = ri;
    dot_acc(d0, bi, bi);
    dot_acc(d1, ri, ri);
  }
  double v[2] = {dot_val(d0), dot_val(d1)};
  __shared__ double out[2 * 64];
  if (col_grid_sum<2>(v, a, out)) {
    const double bb = out[k], rr = out[a.K + k];
    a.c.bnrm2[k] = bb;
    a.c.rho[k] = rr;
    a.c.rho_old[k] = 1.0;
    a.c.alpha[k] = 1.0;
    a.c.omega[k] = 1.0;
    a.c.sconv[k] = 0;
    const double err = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    a.c.err[k] = err;
    a.c.active[k] = (bb > 0.0 && err > a.st->tol &&
                     !(a.outer_err && a.outer_err[k] <= a.outer_tol)) ? 1 : 0;
    a.c.status[k] = a.c.active[k] ? VDR_NOT_CONVERGED : VDR_OK;
  }
}

__global__ void bb_finish_start(BVec a) {  // one block: any column active?
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  if (threadIdx.x < a.K && a.c.active[threadIdx.x]) any = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    a.st->iter = 0;
    a.st->done = any ? 0 : 1;
  }
}

__global__ void __launch_bounds__(BT) bb_p(BVec a) {
  if (a.st->done) return;
  const int k = threadIdx.x % a.K;
  const bool act = a.c.active[k];
  const bool first = a.st->iter == 0;
  const float beta = first ? 0.f
      : (float)((a.c.rho[k] / a.c.rho_old[k]) * (a.c.alpha[k] / a.c.omega[k]));
  const float om = (float)a.c.omega[k];
  BLOOP(i) {
    const long node = i / a.K;
    float pi = 0.f;
    if (act) pi = first ? a.r[i] : a.r[i] + beta * (a.p[i] - om * a.v[i]);
    a.p[i] = pi;
    a.ph[i] = a.m[node] ? 0.f : pi * a.dinv[node];
    a.v[i] = 0.f;
  }
}

__global__ void __launch_bounds__(BT) bb_alpha(BVec a) {
  if (a.st->done) return;
  const int k = threadIdx.x % a.K;
  DfAcc d0{0.f, 0.f};
  BLOOP(i) dot_acc(d0, a.rh[i], a.v[i]);
  double v[1] = {dot_val(d0)};
  __shared__ double out[64];
  if (col_grid_sum<1>(v, a, out)) {
    if (a.c.active[k]) {
      const double rv = out[k];
      if (rv == 0.0 || !isfinite(rv)) {
        a.c.active[k] = 0;
        a.c.status[k] = VDR_BREAKDOWN;
        a.c.alpha[k] = 0.0;
      } else {
        a.c.alpha[k] = a.c.rho[k] / rv;
      }
    }
  }
}

__global__ void __launch_bounds__(BT) bb_s(BVec a) {
  if (a.st->done) return;
  const int k = threadIdx.x % a.K;
  const float al = a.c.active[k] ? (float)a.c.alpha[k] : 0.f;
  DfAcc d0{0.f, 0.f};
  BLOOP(i) {
    const long node = i / a.K;
    const float si = a.r[i] - al * a.v[i];
    a.s[i] = si;
    a.sh[i] = a.m[node] ? 0.f : si * a.dinv[node];
    a.t[i] = 0.f;
    dot_acc(d0, si, si);
  }
  double v[1] = {dot_val(d0)};
  __shared__ double out[64];
  if (col_grid_sum<1>(v, a, out)) {
    const double sn = a.c.bnrm2[k] > 0.0 ? sqrt(out[k] / a.c.bnrm2[k]) : 0.0;
    a.c.snrm[k] = sn;
    a.c.sconv[k] = (a.c.active[k] && sn <= a.st->tol) ? 1 : 0;
  }
}

__global__ void __launch_bounds__(BT) bb_omega(BVec a) {
  if (a.st->done) return;
  const int k = threadIdx.x % a.K;
  DfAcc d0{0.f, 0.f}, d1{0.f, 0.f};
  BLOOP(i) {
    const float ti = a.t[i];
    dot_acc(d0, ti, a.s[i]);
    dot_acc(d1, ti, ti);
  }
  double v[2] = {dot_val(d0), dot_val(d1)};
  __shared__ double out[2 * 64];
  if (col_grid_sum<2>(v, a, out)) {
    if (a.c.active[k] && !a.c.sconv[k]) {
      const double ts = out[k], tt = out[a.K + k];
      if (tt == 0.0 || !isfinite(tt) || !isfinite(ts)) {
        a.c.omega[k] = 0.0;
      } else {
        a.c.omega[k] = ts / tt;
      }
    }
  }
}

__global__ void __launch_bounds__(BT) bb_xr(BVec a) {
  if (a.st->done) return;
  const int k = threadIdx.x % a.K;
  const bool act = a.c.active[k];
  const bool sc = a.c.sconv[k];
  const float al = act ? (float)a.c.alpha[k] : 0.f;
  const float om = (act && !sc) ? (float)a.c.omega[k] : 0.f;
  DfAcc d0{0.f, 0.f}, d1{0.f, 0.f};
  BLOOP(i) {
    if (act) {
      a.x[i] = a.x[i] + al * a.ph[i] + om * a.sh[i];
      const float rn = sc ? a.s[i] : a.s[i] - om * a.t[i];
      a.r[i] = rn;
    }
    const float ri = a.r[i];
    dot_acc(d0, ri, ri);
    dot_acc(d1, a.rh[i], ri);
  }
  double v[2] = {dot_val(d0), dot_val(d1)};
  __shared__ double out[2 * 64];
  if (col_grid_sum<2>(v, a, out)) {
    if (act) {
      a.c.rho_old[k] = a.c.rho[k];
      a.c.rho[k] = out[a.K + k];
      const double err = sqrt(out[k] / a.c.bnrm2[k]);
      a.c.err[k] = err;
      if (!(err == err)) {
        a.c.active[k] = 0;
        a.c.status[k] = VDR_BREAKDOWN;
      } else if (err <= a.st->tol || sc) {
        a.c.active[k] = 0;
        a.c.status[k] = VDR_OK;
      } else if (out[a.K + k] == 0.0 || om == 0.f) {
        a.c.active[k] = 0;
        a.c.status[k] = VDR_BREAKDOWN;
      }
    }
  }
}

// After an iteration: iteration count, and done when no column is active
// or itmax is reached.
__global__ void bb_tail(BVec a) {
  if (a.st->done) return;
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  if (threadIdx.x < a.K && a.c.active[threadIdx.x]) any = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    a.st->iter += 1;
    if (!any || a.st->iter >= a.st->itmax) a.st->done = 1;
  }
}

// ------------------------------------------------ FP64 <-> FP32 block glue
// R = B - R (R holds A X) in FP64; per-column max |R| and max |B|.
__global__ void __launch_bounds__(BT) bo_residual(BVec a, const double *B,
                                                  double *R, double *mx) {
  const int k = threadIdx.x % a.K;
  double v[2] = {0.0, 0.0};
  BLOOP(i) {
    const double bi = B[i];
    const double ri = bi - R[i];
    R[i] = ri;
    v[0] = fmax(v[0], fabs(ri));
    v[1] = fmax(v[1], fabs(bi));
  }
  __shared__ double out[2 * 64];
  if (col_grid_sum<2, true>(v, a, out)) {
    mx[k] = out[k];
    mx[a.K + k] = out[a.K + k];
  }
}

// Per-column scale 2^e >= max |R_k| (a power of two, so scaling is exact);
// Rf = R / scale in FP32 (values in [-1, 1]); err_k = ||R_k|| / ||B_k||
// from the norms of the max-scaled columns (no overflow or underflow).
__global__ void __launch_bounds__(BT) bo_scale(BVec a, const double *B,
                                               const double *R, float *Rf,
                                               const double *mx, double *scale,
                                               double *err_out) {
  const int k = threadIdx.x % a.K;
  const double rm = mx[k], bm = mx[a.K + k];
  int er = 0;
  if (rm > 0.0 && isfinite(rm)) frexp(rm, &er);
  const double inv_r = ldexp(1.0, -er);
  const double inv_b = (bm > 0.0 && isfinite(bm)) ? 1.0 / bm : 1.0;
  double v[2] = {0.0, 0.0};
  BLOOP(i) {
    const double rs = R[i] * inv_r;
    Rf[i] = (float)rs;
    v[0] += rs * rs;
    const double bs = B[i] * inv_b;
    v[1] += bs * bs;
  }
  __shared__ double out[2 * 64];
  if (col_grid_sum<2>(v, a, out)) {
    scale[k] = ldexp(1.0, er);
    double err;
    if (!(rm == rm) || isinf(rm)) err = rm + rm;   // NaN / inf propagate
    else if (rm == 0.0) err = 0.0;
    else if (!(bm > 0.0)) err = INFINITY;          // zero column, nonzero R
    else err = (ldexp(1.0, er) * sqrt(out[k])) / (bm * sqrt(out[a.K + k]));
    err_out[k] = err;
  }
}

__global__ void bo_update(long n, int K, double *X, const float *D,
                          const double *scale) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    X[i] += (double)D[i] * scale[i % K];
}

__global__ void bo_mask(long n, int K, double *X, const unsigned char *m) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    if (m[i / K]) X[i] = 0.0;
}

__global__ void dinv_to_f32(const double *__restrict__ d, float *__restrict__ f,
                            int N) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long)gridDim.x * blockDim.x)
    f[i] = (float)d[i];
}

int grid_n(long n, int threads, int per_sm) {
  const long need = (n + threads - 1) / threads;
  return (int)std::max<long>(1, std::min<long>(need, (long)sm_count_b() * per_sm));
}

}  // namespace

// ------------------------------------------------------------ host side
int block_apply_launches_tf32(const Handle &h, int K, bool split,
                              const float *X, float *Y, const float4 *Aaos,
                              const int *skip, cudaStream_t s) {
  const int grid = grid_n((long)h.E * 32, 256, 8);
  const float *A = reinterpret_cast<const float *>(Aaos);
  if (split)
    block_apply_tf32<true><<<grid, 256, 0, s>>>(A, h.conn, h.E, K, X, Y, skip);
  else
    block_apply_tf32<false><<<grid, 256, 0, s>>>(A, h.conn, h.E, K, X, Y, skip);
  count_launches(1);
  return cudaGetLastError() == cudaSuccess ? VDR_OK : VDR_CUDA_ERROR;
}

cudaError_t launch_block_apply64(const Handle &h, int K, const double *X,
                                 double *Y, cudaStream_t s) {
  const int grid = grid_n((long)h.E * 32, 256, 8);
  if (h.storage == VDR_STORE_DF && h.Ahi)
    block_apply_df<<<grid, 256, 0, s>>>(h.Ahi, h.Alo, h.conn, h.E, K, X, Y);
  else
    block_apply_f64<<<grid, 256, 0, s>>>(h.A64, h.conn, h.E, K, X, Y);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_block_rhs(const Handle &h, const double *phi, int K,
                             const double *Q, double cf, double *B,
                             cudaStream_t s) {
  block_rhs<<<grid_n((long)h.E * K, 256, 8), 256, 0, s>>>(phi, h.conn, h.E, K,
                                                          Q, h.perm_d, cf, B);
  count_launches(1);
  return cudaGetLastError();
}

// Element-major FP32 copy of the operator for the tensor-core apply.
cudaError_t ensure_aos(Handle &h, float4 **out) {
  cudaError_t e;
  if (!h.Aaos) {
    if ((e = cudaMalloc(&h.Aaos, sizeof(float4) * 16 * (size_t)h.E))) return e;
    h.aos_valid = false;
  }
  if (!h.aos_valid) {
    const int grid = grid_n((long)h.E * 16, 256, 16);
    if (h.storage == VDR_STORE_DF && h.Ahi)
      aos_from_hi<<<grid, 256, 0, h.stream>>>(h.Ahi, h.E, h.Aaos);
    else
      aos_from_f64<<<grid, 256, 0, h.stream>>>(h.A64, h.E, h.Aaos);
    count_launches(1);
    if ((e = cudaGetLastError())) return e;
    h.aos_valid = true;
  }
  *out = h.Aaos;
  return cudaSuccess;
}

namespace {
// device workspace of the block solve, carved from h.bk_f / h.bk_d
constexpr int BK_COLS = 16 * 64;            // per-column doubles and ints
constexpr int BK_PARTIALS = 2 * 64 * 2048;  // NQ x K x blocks
constexpr int BK_MAX_GRID = 2048;
}  // namespace

// Block solve: FP64 refinement around K-column FP32 BiCGStab with the TF32
// tensor-core apply.  B, X are N x K FP64 device arrays (node-major).
int solve_block_device(Handle &h, int K, int precision, const double *B,
                       double *X, double tol, double inner_tol, int max_outer,
                       int inner_itmax, int *outer_iters, int *inner_iters,
                       double *errs_host) {
  if (K != 16 && K != 32 && K != 64) {
    set_error("block solve: K must be 16, 32 or 64");
    return VDR_BAD_ARGUMENT;
  }
  if (precision != VDR_BLOCK_TF32 && precision != VDR_BLOCK_TF32X3) {
    set_error("block solve: precision must be VDR_BLOCK_TF32 or VDR_BLOCK_TF32X3");
    return VDR_BAD_ARGUMENT;
  }
  const bool split = precision == VDR_BLOCK_TF32X3;
  cudaError_t e;
  cudaStream_t s = h.stream;
  const long n = (long)h.N * K;
  float4 *Aaos = nullptr;
  if ((e = ensure_aos(h, &Aaos))) return cuda_fail(e, "block operator copy");
  if (h.bk_K != K || !h.bk_f) {
    if (h.bk_f) cudaFree(h.bk_f);
    if (h.bk_d) cudaFree(h.bk_d);
    h.bk_f = nullptr;
    h.bk_d = nullptr;
    h.bk_K = 0;
    if (h.bk_graph) cudaGraphExecDestroy(h.bk_graph);
    h.bk_graph = nullptr;
    if ((e = cudaMalloc(&h.bk_f, sizeof(float) * 10 * (size_t)n)) ||
        (e = cudaMalloc(&h.bk_d, sizeof(double) * ((size_t)n + BK_COLS +
                                                   BK_PARTIALS + 8))))
      return cuda_fail(e, "block workspace");
    h.bk_K = K;
  }
  if (!h.dinv32 && (e = cudaMalloc(&h.dinv32, sizeof(float) * (size_t)h.N)))
    return cuda_fail(e, "block workspace");
  float *fv = h.bk_f;
  double *R = h.bk_d;
  double *colsd = R + n;
  double *partials = colsd + BK_COLS;
  BState *st = reinterpret_cast<BState *>(partials + BK_PARTIALS);
  BVec a{};
  a.n = n;
  a.K = K;
  a.st = st;
  a.partials = partials;
  a.c.bnrm2 = colsd + 0 * 64;
  a.c.err = colsd + 1 * 64;
  a.c.rho = colsd + 2 * 64;
  a.c.rho_old = colsd + 3 * 64;
  a.c.alpha = colsd + 4 * 64;
  a.c.omega = colsd + 5 * 64;
  a.c.snrm = colsd + 6 * 64;
  double *outer_err = colsd + 7 * 64;
  double *mx = colsd + 8 * 64;      // 2 x 64
  double *scale = colsd + 10 * 64;
  int *colsi = reinterpret_cast<int *>(colsd + 11 * 64);  // 3 x 64 ints
  a.c.active = colsi;
  a.c.sconv = colsi + 64;
  a.c.status = colsi + 128;
  a.m = h.mask;
  a.dinv = h.dinv32;
  a.outer_err = outer_err;
  a.outer_tol = tol;
  float *bf = fv;  // inner right-hand side: scaled FP32 residual
  a.b = bf;
  a.x = fv + 1 * n;
  a.r = fv + 2 * n;
  a.rh = fv + 3 * n;
  a.p = fv + 4 * n;
  a.v = fv + 5 * n;
  a.ph = fv + 6 * n;
  a.s = fv + 7 * n;
  a.sh = fv + 8 * n;
  a.t = fv + 9 * n;

  dinv_to_f32<<<grid_n(h.N, 256, 8), 256, 0, s>>>(h.dinv, h.dinv32, h.N);
  count_launches(1);
  const int gv = std::min(BK_MAX_GRID, grid_n(n, BT, 8));
  const int gm = grid_n(n, 256, 8);
  bo_mask<<<gm, 256, 0, s>>>(n, K, X, h.mask);
  count_launches(1);
  if ((e = cudaGetLastError())) return cuda_fail(e, "block setup");

  // KI inner iterations per graph launch (8 kernels each)
  constexpr int KI = 4;
  if (!h.bk_graph || h.bk_graph_split != split) {
    if (h.bk_graph) cudaGraphExecDestroy(h.bk_graph);
    h.bk_graph = nullptr;
    cudaGraph_t graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)))
      return cuda_fail(e, "capture");
    for (int it = 0; it < KI; it++) {
      bb_p<<<gv, BT, 0, s>>>(a);
      block_apply_launches_tf32(h, K, split, a.ph, a.v, Aaos, &st->done, s);
      bb_alpha<<<gv, BT, 0, s>>>(a);
      bb_s<<<gv, BT, 0, s>>>(a);
      block_apply_launches_tf32(h, K, split, a.sh, a.t, Aaos, &st->done, s);
      bb_omega<<<gv, BT, 0, s>>>(a);
      bb_xr<<<gv, BT, 0, s>>>(a);
      bb_tail<<<1, 64, 0, s>>>(a);
    }
    count_launches(-2L * KI);  // the captured applies count at replay
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e2) return cuda_fail(e2, "end capture");
    e = cudaGraphInstantiate(&h.bk_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e) return cuda_fail(e, "instantiate");
    h.bk_graph_split = split;
  }

  BState init{};
  init.tol = inner_tol;
  init.itmax = inner_itmax;
  int total_inner = 0, outer = 0;
  std::vector<double> herr(K, 0.0);
  int status = VDR_NOT_CONVERGED;
  for (outer = 0;; outer++) {
    // FP64 residual of every column, its scale and relative norm
    if ((e = cudaMemsetAsync(R, 0, sizeof(double) * n, s)) ||
        (e = launch_block_apply64(h, K, X, R, s)) ||
        (e = cudaMemsetAsync(st, 0, sizeof(BState), s)))
      return cuda_fail(e, "block residual");
    bo_residual<<<gv, BT, 0, s>>>(a, B, R, mx);
    bo_scale<<<gv, BT, 0, s>>>(a, B, R, bf, mx, scale, outer_err);
    count_launches(2);
    if ((e = cudaMemcpyAsync(herr.data(), outer_err, sizeof(double) * K,
                             cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_fail(e, "block residual");
    double worst = 0.0;
    bool nan = false;
    for (int k = 0; k < K; k++) {
      if (!(herr[k] == herr[k])) nan = true;
      worst = std::max(worst, herr[k]);
    }
    if (nan) {
      status = VDR_BREAKDOWN;
      break;
    }
    if (worst <= tol) {
      status = VDR_OK;
      break;
    }
    if (outer >= max_outer) break;
    // K simultaneous FP32 inner solves of A D = R / scale, D = 0
    if ((e = cudaMemcpyAsync(st, &init, sizeof(BState), cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemsetAsync(a.x, 0, sizeof(float) * n, s)) ||
        (e = cudaMemsetAsync(a.r, 0, sizeof(float) * n, s)))
      return cuda_fail(e, "inner reset");
    bb_start<<<gv, BT, 0, s>>>(a);
    bb_finish_start<<<1, 64, 0, s>>>(a);
    count_launches(2);
    BState hs{};
    for (int c = 0; c * KI < inner_itmax + KI; c++) {
      if ((e = cudaGraphLaunch(h.bk_graph, s))) return cuda_fail(e, "graph");
      count_launches(8L * KI);
      if ((e = cudaMemcpyAsync(&hs, st, sizeof(BState), cudaMemcpyDeviceToHost, s)) ||
          (e = cudaStreamSynchronize(s)))
        return cuda_fail(e, "inner state");
      if (hs.done) break;
    }
    total_inner += hs.iter;
    bo_update<<<gm, 256, 0, s>>>(n, K, X, a.x, scale);
    count_launches(1);
    if ((e = cudaGetLastError())) return cuda_fail(e, "update");
  }
  if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "block solve");
  if (outer_iters) *outer_iters = outer;
  if (inner_iters) *inner_iters = total_inner;
  if (errs_host)
    for (int k = 0; k < K; k++) errs_host[k] = herr[k];
  return status;
}

}  // namespace vdr
