// krylov.cu -- Jacobi-preconditioned BiCG (the reference's dbcg_simple,
// vanadis_full_DR_OpenMP_timing.for:906-984 / kernel_dbcg_simple_,
// src_v2026_2_1/cudatest.cu:301-602) and BiCGStab on the GPU.
//
// GB300 design:
//  * Every Krylov scalar (rho, alpha, omega, beta, norms, the iteration
//    count, convergence and breakdown flags) lives in a device struct
//    (KState).  Dot products are fused into the vector update that produces
//    their operands; each kernel's blocks write partial sums and the last
//    block to finish (ticketed with one atomic) adds the partials in a fixed
//    order and updates the scalars.  Reductions are therefore deterministic
//    for a fixed grid, and no spin-wait exists anywhere.
//  * The Jacobi preconditioner is fused into the vector updates (z = r/d is
//    never stored for BiCG).
//  * One iteration is a fixed chain of launches that read their scalars
//    from KState, so `iters_per_graph` iterations are captured once into a
//    CUDA graph and replayed; once `done` is set every kernel returns at
//    entry.  The host reads KState back asynchronously once per graph
//    launch, one launch behind, so the GPU never waits for the host.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <atomic>
#include <cstring>

#include "dfloat.cuh"
#include "vdr_internal.h"

namespace vdr {
namespace {

constexpr unsigned FULL = 0xffffffffu;

template <int NQ>
__device__ __forceinline__ void block_sum(double (&v)[NQ]) {
  __shared__ double sm[RED_THREADS / 32][MAXQ];
#pragma unroll
  for (int q = 0; q < NQ; q++)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
      v[q] += __shfl_xor_sync(FULL, v[q], off);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++) sm[w][q] = v[q];
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      v[q] = (l < (int)(blockDim.x >> 5)) ? sm[l][q] : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        v[q] += __shfl_xor_sync(FULL, v[q], off);
    }
  }
}

// Grid-wide sum of NQ values.  Returns true in thread 0 of the last block
// to arrive, with the totals in `out`.
template <int NQ>
__device__ __forceinline__ bool grid_sum(double (&v)[NQ], double *partials,
                                         unsigned int *ticket,
                                         double (&out)[NQ]) {
  __shared__ bool last;
  block_sum<NQ>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NQ; q++) partials[q * gridDim.x + blockIdx.x] = v[q];
    __threadfence();
    const unsigned t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double w[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    w[q] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
      w[q] += __ldcg(partials + q * gridDim.x + b);
  }
  block_sum<NQ>(w);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NQ; q++) out[q] = w[q];
    *ticket = 0u;
    return true;
  }
  return false;
}

__device__ __forceinline__ bool finite(double x) { return isfinite(x); }

struct Vec {
  int n;
  KState *st;
  double *partials;
  const double *b;
  const double *dinv;  // 1/diag (diag is 1 on Dirichlet nodes)
  const unsigned char *m;
  double *x, *r, *rh, *p, *v, *ph, *s, *sh, *t;  // BiCGStab
  double *rr, *pp, *z, *zz;                      // BiCG (r, p, x shared)
};

// Grid-stride loops unrolled U times with every load of the U elements
// issued before any use, so each thread keeps U independent memory
// requests in flight (these kernels are bound by HBM bandwidth).
constexpr int U = 4;
#define VLOOP(body_load, body_use)                                          \
  {                                                                         \
    const long stride_ = (long)gridDim.x * blockDim.x;                      \
    for (long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x; i0 < a.n;   \
         i0 += U * stride_) {                                               \
      _Pragma("unroll") for (int u = 0; u < U; u++) {                       \
        const long i = i0 + u * stride_;                                    \
        const bool ok = i < a.n;                                            \
        body_load                                                           \
      }                                                                     \
      _Pragma("unroll") for (int u = 0; u < U; u++) {                       \
        const long i = i0 + u * stride_;                                    \
        if (i < a.n) { body_use }                                           \
      }                                                                     \
    }                                                                       \
  }

// -------- shared start: r = b - r (r holds A x0), residual norms --------
// BiCGStab: rh = r, rho = (rh, r).  BiCG: rr = r, bknum = (r/d, rr).
template <bool BICG>
__global__ void __launch_bounds__(RED_THREADS) k_start(Vec a) {
  double v[3] = {0.0, 0.0, 0.0};
  double bv[U], rv[U], dv[U];
  VLOOP(bv[u] = ok ? a.b[i] : 0.0; rv[u] = ok ? a.r[i] : 0.0;
        dv[u] = (ok && BICG) ? a.dinv[i] : 0.0;,
        const double ri = bv[u] - rv[u];
        a.r[i] = ri;
        if (BICG) {
          a.rr[i] = ri;
          v[2] += (ri * dv[u]) * ri;
        } else {
          a.rh[i] = ri;
        }
        v[0] += bv[u] * bv[u];
        v[1] += ri * ri;)
  double o[3];
  if (grid_sum<3>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    st->bnrm2 = o[0];
    st->iter = 0;
    st->sconv = 0;
    st->status = VDR_NOT_CONVERGED;
    st->done = 0;
    st->rho = o[1];
    st->rho_old = 1.0;
    st->alpha = 1.0;
    st->omega = 1.0;
    st->bknum = o[2];
    st->bkden = 1.0;
    st->reason = 0;
    if (o[0] == 0.0) {  // b = 0: the solution is x = 0
      st->err = 0.0;
      st->status = VDR_OK;
      st->done = 2;  // tells the host to zero x
      return;
    }
    st->err = sqrt(o[1]) / sqrt(o[0]);
    if (!(st->err == st->err)) {
      st->status = VDR_BREAKDOWN;
      st->reason = 5;
      st->done = 1;
    } else if (st->err <= st->tol) {
      st->status = VDR_OK;
      st->done = 1;
    } else if (st->itmax <= 0) {
      st->done = 1;
    }
  }
}

// ---------------------------- BiCGStab ----------------------------------
// p = r + beta (p - omega v); ph = M^-1 p (0 on Dirichlet); v = 0.
__global__ void __launch_bounds__(RED_THREADS) bs_p(Vec a) {
  const KState *st = a.st;
  if (st->done) return;
  const bool first = st->iter == 0;
  const double beta = first ? 0.0 : (st->rho / st->rho_old) * (st->alpha / st->omega);
  const double om = st->omega;
  double rv[U], pv[U], vv[U], dv[U];
  unsigned char mv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.0; pv[u] = (ok && !first) ? a.p[i] : 0.0;
        vv[u] = (ok && !first) ? a.v[i] : 0.0; dv[u] = ok ? a.dinv[i] : 0.0;
        mv[u] = ok ? a.m[i] : 1;,
        const double pi = first ? rv[u] : rv[u] + beta * (pv[u] - om * vv[u]);
        a.p[i] = pi;
        a.ph[i] = mv[u] ? 0.0 : pi * dv[u];
        a.v[i] = 0.0;)
}

// alpha = rho / (rh, v)
__global__ void __launch_bounds__(RED_THREADS) bs_alpha(Vec a) {
  if (a.st->done) return;
  double v[1] = {0.0};
  double hv[U], vv[U];
  VLOOP(hv[u] = ok ? a.rh[i] : 0.0; vv[u] = ok ? a.v[i] : 0.0;,
        v[0] += hv[u] * vv[u];)
  double o[1];
  if (grid_sum<1>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    if (o[0] == 0.0 || !finite(o[0])) {
      st->status = VDR_BREAKDOWN;
      st->reason = 2;
      st->done = 1;
    } else {
      st->alpha = st->rho / o[0];
    }
  }
}

// s = r - alpha v; sh = M^-1 s; t = 0; ||s||.
__global__ void __launch_bounds__(RED_THREADS) bs_s(Vec a) {
  if (a.st->done) return;
  const double al = a.st->alpha;
  double v[1] = {0.0};
  double rv[U], vv[U], dv[U];
  unsigned char mv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.0; vv[u] = ok ? a.v[i] : 0.0;
        dv[u] = ok ? a.dinv[i] : 0.0; mv[u] = ok ? a.m[i] : 1;,
        const double si = rv[u] - al * vv[u];
        a.s[i] = si;
        a.sh[i] = mv[u] ? 0.0 : si * dv[u];
        a.t[i] = 0.0;
        v[0] += si * si;)
  double o[1];
  if (grid_sum<1>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    st->snrm = sqrt(o[0]) / sqrt(st->bnrm2);
    if (st->snrm <= st->tol) st->sconv = 1;
  }
}

// omega = (t, s) / (t, t)
__global__ void __launch_bounds__(RED_THREADS) bs_omega(Vec a) {
  if (a.st->done || a.st->sconv) return;
  double v[2] = {0.0, 0.0};
  double tv[U], sv[U];
  VLOOP(tv[u] = ok ? a.t[i] : 0.0; sv[u] = ok ? a.s[i] : 0.0;,
        v[0] += tv[u] * sv[u];
        v[1] += tv[u] * tv[u];)
  double o[2];
  if (grid_sum<2>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    if (o[1] == 0.0 || !finite(o[1]) || !finite(o[0])) {
      st->status = VDR_BREAKDOWN;
      st->reason = 3;
      st->done = 1;
    } else {
      st->omega = o[0] / o[1];
    }
  }
}

// x += alpha ph + omega sh; r = s - omega t; rho_new = (rh, r); ||r||.
__global__ void __launch_bounds__(RED_THREADS) bs_xr(Vec a) {
  KState *stc = a.st;
  if (stc->done) return;
  const double al = stc->alpha;
  if (stc->sconv) {
    double v[1] = {0.0};
    double xv[U], pv[U], sv[U];
    VLOOP(xv[u] = ok ? a.x[i] : 0.0; pv[u] = ok ? a.ph[i] : 0.0;
          sv[u] = ok ? a.s[i] : 0.0;,
          a.x[i] = xv[u] + al * pv[u];
          a.r[i] = sv[u];)
    double o[1];
    if (grid_sum<1>(v, a.partials, &a.st->ticket, o)) {
      KState *st = a.st;
      st->iter += 1;
      st->err = st->snrm;
      st->status = VDR_OK;
      st->done = 1;
    }
    return;
  }
  const double om = stc->omega;
  double v[2] = {0.0, 0.0};
  double xv[U], pv[U], shv[U], sv[U], tv[U], hv[U];
  VLOOP(xv[u] = ok ? a.x[i] : 0.0; pv[u] = ok ? a.ph[i] : 0.0;
        shv[u] = ok ? a.sh[i] : 0.0; sv[u] = ok ? a.s[i] : 0.0;
        tv[u] = ok ? a.t[i] : 0.0; hv[u] = ok ? a.rh[i] : 0.0;,
        a.x[i] = xv[u] + al * pv[u] + om * shv[u];
        const double ri = sv[u] - om * tv[u];
        a.r[i] = ri;
        v[0] += ri * ri;
        v[1] += hv[u] * ri;)
  double o[2];
  if (grid_sum<2>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    st->iter += 1;
    st->rho_old = st->rho;
    st->rho = o[1];
    st->err = sqrt(o[0]) / sqrt(st->bnrm2);
    if (!(st->err == st->err) || !finite(o[1])) {
      st->status = VDR_BREAKDOWN;
      st->reason = 5;
      st->done = 1;
    } else if (st->err <= st->tol) {
      st->status = VDR_OK;
      st->done = 1;
    } else if (o[1] == 0.0 || om == 0.0) {
      st->status = VDR_BREAKDOWN;
      st->reason = o[1] == 0.0 ? 1 : 4;
      st->done = 1;
    } else if (st->iter >= st->itmax) {
      st->status = VDR_NOT_CONVERGED;
      st->done = 1;
    } else if (st->stall_window > 0) {
      if (st->err < 0.99 * st->best_err) {
        st->best_err = st->err;
        st->since_best = 0;
      } else if (++st->since_best >= st->stall_window) {
        st->status = VDR_NOT_CONVERGED;
        st->reason = 6;  // stalled
        st->done = 1;
      }
    }
  }
}

// ------------------------------ BiCG -------------------------------------
// p = z + bk p, pp = zz + bk pp with z = r/d, zz = rr/d (masked in place as
// matvec_0 masks its input); clears the two apply outputs.
__global__ void __launch_bounds__(RED_THREADS) bc_p(Vec a) {
  const KState *st = a.st;
  if (st->done) return;
  const bool first = st->iter == 0;
  const double bk = first ? 0.0 : st->bknum / st->bkden;
  double rv[U], rrv[U], dv[U], pv[U], ppv[U];
  unsigned char mv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.0; rrv[u] = ok ? a.rr[i] : 0.0;
        dv[u] = ok ? a.dinv[i] : 0.0; mv[u] = ok ? a.m[i] : 1;
        pv[u] = (ok && !first) ? a.p[i] : 0.0;
        ppv[u] = (ok && !first) ? a.pp[i] : 0.0;,
        const double zi = rv[u] * dv[u];
        const double zzi = rrv[u] * dv[u];
        a.p[i] = mv[u] ? 0.0 : (first ? zi : zi + bk * pv[u]);
        a.pp[i] = mv[u] ? 0.0 : (first ? zzi : zzi + bk * ppv[u]);
        a.z[i] = 0.0;
        a.zz[i] = 0.0;)
}

// ak = bknum / (z, pp)
__global__ void __launch_bounds__(RED_THREADS) bc_ak(Vec a) {
  if (a.st->done) return;
  double v[1] = {0.0};
  double zv[U], pv[U];
  VLOOP(zv[u] = ok ? a.z[i] : 0.0; pv[u] = ok ? a.pp[i] : 0.0;,
        v[0] += zv[u] * pv[u];)
  double o[1];
  if (grid_sum<1>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    st->ak = st->bknum / o[0];
    if (!finite(st->ak)) {
      st->status = VDR_BREAKDOWN;
      st->reason = 2;
      st->done = 1;
    }
  }
}

// x += ak p; r -= ak z; rr -= ak zz; err = ||r||/||b||; bknum' = (r/d, rr).
__global__ void __launch_bounds__(RED_THREADS) bc_upd(Vec a) {
  if (a.st->done) return;
  const double ak = a.st->ak;
  double v[2] = {0.0, 0.0};
  double xv[U], pv[U], rv[U], zv[U], rrv[U], zzv[U], dv[U];
  VLOOP(xv[u] = ok ? a.x[i] : 0.0; pv[u] = ok ? a.p[i] : 0.0;
        rv[u] = ok ? a.r[i] : 0.0; zv[u] = ok ? a.z[i] : 0.0;
        rrv[u] = ok ? a.rr[i] : 0.0; zzv[u] = ok ? a.zz[i] : 0.0;
        dv[u] = ok ? a.dinv[i] : 0.0;,
        a.x[i] = xv[u] + ak * pv[u];
        const double ri = rv[u] - ak * zv[u];
        const double rri = rrv[u] - ak * zzv[u];
        a.r[i] = ri;
        a.rr[i] = rri;
        v[0] += ri * ri;
        v[1] += (ri * dv[u]) * rri;)
  double o[2];
  if (grid_sum<2>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    st->iter += 1;
    st->err = sqrt(o[0]) / sqrt(st->bnrm2);
    st->bkden = st->bknum;
    st->bknum = o[1];
    if (!(st->err == st->err)) {
      st->status = VDR_BREAKDOWN;
      st->reason = 5;
      st->done = 1;
    } else if (st->err <= st->tol) {
      st->status = VDR_OK;
      st->done = 1;
    } else if (st->iter >= st->itmax) {
      st->status = VDR_NOT_CONVERGED;
      st->done = 1;
    }
  }
}

__global__ void k_true_residual(Vec a, const double *ax, double *partials,
                                unsigned int *ticket, double *out) {
  double v[2] = {0.0, 0.0};
  double bv[U], av[U];
  VLOOP(bv[u] = ok ? a.b[i] : 0.0; av[u] = ok ? ax[i] : 0.0;,
        const double ri = bv[u] - av[u];
        v[0] += ri * ri;
        v[1] += bv[u] * bv[u];)
  double o[2];
  if (grid_sum<2>(v, partials, ticket, o)) *out = sqrt(o[0]) / sqrt(o[1]);
}

int red_grid(int n) {
  const long need = ((long)n + RED_THREADS - 1) / RED_THREADS;
  return (int)std::max<long>(1, std::min<long>(need, (long)device_sm_count() * 8));
}

Vec make_vec(Handle &h, const double *b, double *x) {
  Vec a{};
  a.n = h.N;
  a.st = h.st;
  a.partials = h.partials;
  a.b = b;
  a.dinv = h.dinv;
  a.m = h.mask;
  a.x = x;
  double *w = h.work;
  const size_t N = h.N;
  a.r = w + 0 * N;
  a.rh = w + 1 * N;
  a.p = w + 2 * N;
  a.v = w + 3 * N;
  a.ph = w + 4 * N;
  a.s = w + 5 * N;
  a.sh = w + 6 * N;
  a.t = w + 7 * N;
  // BiCG reuses the same slots: rr = rh, pp = ph, z = v, zz = t.
  a.rr = a.rh;
  a.pp = a.ph;
  a.z = a.v;
  a.zz = a.t;
  return a;
}

// The fused FP64 BiCGStab iteration (defined below with the fused kernels).
cudaError_t launch_fused64_iteration(Handle &h, const Vec &a, cudaStream_t s);

cudaError_t launch_iteration(Handle &h, int method, const Vec &a,
                             const Precond *prec) {
  const int g = red_grid(h.N);
  cudaStream_t s = h.stream;
  cudaError_t e;
  if (method == VDR_SOLVER_BICGSTAB && !prec && h.fused64)
    return launch_fused64_iteration(h, a, s);
  if (method == VDR_SOLVER_BICGSTAB) {
    bs_p<<<g, RED_THREADS, 0, s>>>(a);
    if (prec && (e = prec->enqueue(prec->ctx, a.p, a.ph, &h.st->done, nullptr, s)))
      return e;
    if ((e = launch_apply(h, false, a.ph, a.v, &h.st->done, nullptr, s))) return e;
    bs_alpha<<<g, RED_THREADS, 0, s>>>(a);
    bs_s<<<g, RED_THREADS, 0, s>>>(a);
    if (prec && (e = prec->enqueue(prec->ctx, a.s, a.sh, &h.st->done,
                                   &h.st->sconv, s)))
      return e;
    if ((e = launch_apply(h, false, a.sh, a.t, &h.st->done, &h.st->sconv, s))) return e;
    bs_omega<<<g, RED_THREADS, 0, s>>>(a);
    bs_xr<<<g, RED_THREADS, 0, s>>>(a);
  } else {
    bc_p<<<g, RED_THREADS, 0, s>>>(a);
    if (can_apply_both(h)) {  // A p and A^T pp in one pass over the store
      if ((e = launch_apply_both(h, a.p, a.z, a.pp, a.zz, &h.st->done, s))) return e;
    } else {
      if ((e = launch_apply(h, false, a.p, a.z, &h.st->done, nullptr, s))) return e;
      if ((e = launch_apply(h, true, a.pp, a.zz, &h.st->done, nullptr, s))) return e;
    }
    bc_ak<<<g, RED_THREADS, 0, s>>>(a);
    bc_upd<<<g, RED_THREADS, 0, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t ensure_solver_workspace(Handle &h, int nvec) {
  cudaError_t e;
  if (h.nwork < nvec) {
    if (h.work) cudaFree(h.work);
    h.work = nullptr;
    h.nwork = 0;
    if ((e = cudaMalloc(&h.work, sizeof(double) * (size_t)h.N * nvec))) return e;
    h.nwork = nvec;
    for (int k = 0; k < Handle::NGRAPH; k++) {
      if (h.graph_exec[k]) cudaGraphExecDestroy(h.graph_exec[k]);
      h.graph_exec[k] = nullptr;
      h.graph_key[k] = nullptr;
    }
  }
  if (!h.st) {
    if ((e = cudaMalloc(&h.st, sizeof(KState)))) return e;
    if ((e = cudaMemset(h.st, 0, sizeof(KState)))) return e;
    if ((e = cudaMallocHost(&h.h_st, 2 * sizeof(KState)))) return e;
    const int g = red_grid(h.N);
    h.red_blocks = g;
    if ((e = cudaMalloc(&h.partials, sizeof(double) * MAXQ * (size_t)std::max(g, 4096))))
      return e;
    for (int k = 0; k < 2; k++)
      if ((e = cudaEventCreateWithFlags(&h.ev[k], cudaEventDisableTiming))) return e;
  }
  return cudaSuccess;
}

// Kernels of one captured iteration.
long launches_graph_nodes(Handle &h, int method, const Precond *prec) {
  if (method == VDR_SOLVER_BICGSTAB && !prec && h.fused64) return 2 + 2 * apply_launches(h);
  long n = (method == VDR_SOLVER_BICGSTAB ? 5 : 3) +
           (method != VDR_SOLVER_BICGSTAB && can_apply_both(h) ? 1 : 2) *
               apply_launches(h);
  if (prec) n += 2 * prec->launches;
  return n;
}

// Solves A x = b on device arrays b (length N) and x (in/out).  With
// `prec`, BiCGStab is right-preconditioned by M (flexible: x is updated with
// the preconditioned vectors actually used, so M may change between
// applications); `stall_window` > 0 stops a solve whose residual has not
// dropped 1% in that many iterations (status NOT_CONVERGED, reason 6);
// `hist` (max_hist x N) receives x after every graph launch.
int solve_device(Handle &h, int method, const double *b, double *x,
                 double tol, int itmax, int *iter, double *err,
                 const Precond *prec, int stall_window, double *hist,
                 int max_hist, int *n_hist) {
  cudaError_t e = ensure_solver_workspace(h, 8);
  if (e) return cuda_fail(e, "solver workspace");
  cudaStream_t s = h.stream;
  Vec a = make_vec(h, b, x);
  const int g = red_grid(h.N);
  const long long launches0 = launches_so_far();
  h.last = vdr_solve_stats{};

  // KState scalars the kernels read: tol, itmax (ticket stays 0 between uses).
  KState init{};
  init.tol = tol;
  init.itmax = itmax;
  init.best_err = INFINITY;
  init.stall_window = stall_window;
  init.x_zero = 1;
  std::memcpy(&h.h_st[0], &init, sizeof(KState));
  if ((e = cudaMemcpyAsync(h.st, &h.h_st[0], sizeof(KState),
                           cudaMemcpyHostToDevice, s)))
    return cuda_fail(e, "state upload");

  // x on Dirichlet nodes is zeroed in place, as matvec_0 does to its input;
  // A x is skipped when x is then zero (a cold start).
  if ((e = launch_mask_vec_flag(x, h.mask, h.N, &h.st->x_zero, s)))
    return cuda_fail(e, "mask x");
  if ((e = cudaMemsetAsync(a.r, 0, sizeof(double) * h.N, s)))
    return cuda_fail(e, "memset");
  if ((e = launch_apply(h, false, x, a.r, &h.st->x_zero, nullptr, s)))
    return cuda_fail(e, "initial apply");
  if (method == VDR_SOLVER_BICGSTAB)
    k_start<false><<<g, RED_THREADS, 0, s>>>(a);
  else
    k_start<true><<<g, RED_THREADS, 0, s>>>(a);
  count_launches(1);
  if ((e = cudaGetLastError())) return cuda_fail(e, "start kernel");

  // One graph per method; its kernels only see handle-owned buffers plus
  // b and x, which are part of the key.
  const int K = h.opt.iters_per_graph > 0 ? h.opt.iters_per_graph : 8;
  if (prec && method != VDR_SOLVER_BICGSTAB) {
    set_error("a preconditioner needs the BiCGStab solver");
    return VDR_BAD_ARGUMENT;
  }
  const int slot = (method & 1) | (h.apply_fp32 ? 2 : 0) | (prec ? 4 : 0);
  const void *key = (const void *)((uintptr_t)b ^ ((uintptr_t)x << 1) ^
                                   ((uintptr_t)h.work << 2) ^ (uintptr_t)K ^
                                   ((uintptr_t)h.apply_mode << 8) ^
                                   ((uintptr_t)h.scatter << 12) ^
                                   ((uintptr_t)h.storage << 16) ^
                                   ((uintptr_t)(prec ? prec->ctx : nullptr) << 3));
  // the kernels' arguments carry N, E and the work-vector offsets, so a
  // graph captured for other sizes (buffers reused by a smaller mesh) is
  // captured again
  const long long size_key = ((long long)h.N << 32) | (unsigned)h.E;
  const bool fusable = method == VDR_SOLVER_BICGSTAB && !prec;
  for (int attempt = 0; attempt < 2; attempt++) {
    const bool fused = fusable && h.fused64;
    const void *fkey = (const void *)((uintptr_t)key ^ ((uintptr_t)fused << 20));
    if (h.graph_exec[slot] && h.graph_key[slot] == fkey && h.graph_size[slot] == size_key)
      break;
    if (h.graph_exec[slot]) cudaGraphExecDestroy(h.graph_exec[slot]);
    h.graph_exec[slot] = nullptr;
    cudaGraph_t graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)))
      return cuda_fail(e, "begin capture");
    const long long before = launches_so_far();
    for (int k = 0; k < K; k++) {
      e = launch_iteration(h, method, a, prec);
      if (e) break;
    }
    count_launches(before - launches_so_far());  // captured, not launched
    cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (!e && !e2) {
      e = cudaGraphInstantiate(&h.graph_exec[slot], graph, 0);
      cudaGraphDestroy(graph);
      if (!e) {
        h.graph_key[slot] = fkey;
        h.graph_size[slot] = size_key;
        break;
      }
      h.graph_exec[slot] = nullptr;
    } else if (!e2) {
      cudaGraphDestroy(graph);
    }
    // a cooperative launch that the capture or the graph refuses: the
    // five-kernel iteration instead
    if (fused) {
      cudaGetLastError();
      h.fused64 = false;
      e = cudaSuccess;
      continue;
    }
    if (e) return cuda_fail(e, "capture");
    return cuda_fail(e2 ? e2 : cudaErrorUnknown, "end capture");
  }
  if (fusable && h.fused64) {  // the first search direction p = r, p^ = D^-1 r, v = 0
    bs_p<<<g, RED_THREADS, 0, s>>>(a);
    count_launches(1);
    if ((e = cudaGetLastError())) return cuda_fail(e, "first direction");
  }
  const long graph_nodes = launches_graph_nodes(h, method, prec);

  const int max_launches = (itmax + K - 1) / K + 1;
  int launched = 0;
  bool finished = false;
  for (int c = 0; c < max_launches && !finished; c++) {
    if ((e = cudaGraphLaunch(h.graph_exec[slot], s))) return cuda_fail(e, "graph launch");
    count_launches((long)K * graph_nodes);
    if (hist && n_hist && *n_hist < max_hist) {
      if ((e = cudaMemcpyAsync(hist + (size_t)(*n_hist) * h.N, x,
                               sizeof(double) * h.N, cudaMemcpyDeviceToDevice, s)))
        return cuda_fail(e, "record iterate");
      (*n_hist)++;
    }
    if ((e = cudaMemcpyAsync(&h.h_st[c & 1], h.st, sizeof(KState),
                             cudaMemcpyDeviceToHost, s)))
      return cuda_fail(e, "state readback");
    if ((e = cudaEventRecord(h.ev[c & 1], s))) return cuda_fail(e, "event");
    launched++;
    if (c > 0) {
      if ((e = cudaEventSynchronize(h.ev[(c - 1) & 1]))) return cuda_fail(e, "sync");
      if (h.h_st[(c - 1) & 1].done) finished = true;
    }
  }
  if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "solve");
  KState fin;
  if ((e = cudaMemcpy(&fin, h.st, sizeof(KState), cudaMemcpyDeviceToHost)))
    return cuda_fail(e, "final state");
  if (fin.done == 2) {  // b == 0
    if ((e = cudaMemsetAsync(x, 0, sizeof(double) * h.N, s))) return cuda_fail(e, "zero x");
    if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "zero x");
  }
  const int status = fin.done ? fin.status : VDR_NOT_CONVERGED;
  h.last.iterations = fin.iter;
  h.last.status = status;
  h.last.graph_launches = launched;
  h.last.kernel_launches = (int)(launches_so_far() - launches0);
  h.last.breakdown = (status == VDR_BREAKDOWN || fin.reason == 6) ? fin.reason : 0;
  if (iter) *iter = fin.iter;
  if (err) *err = fin.err;
  return status;
}

namespace {
// r = b - r (r holds A x); out = ||r|| / ||b||.
__global__ void __launch_bounds__(RED_THREADS) k_residual(Vec a, double *r,
                                                          double *out) {
  double v[2] = {0.0, 0.0};
  double bv[U], av[U];
  VLOOP(bv[u] = ok ? a.b[i] : 0.0; av[u] = ok ? r[i] : 0.0;,
        const double ri = bv[u] - av[u];
        r[i] = ri;
        v[0] += ri * ri;
        v[1] += bv[u] * bv[u];)
  double o[2];
  if (grid_sum<2>(v, a.partials, &a.st->ticket, o)) {
    out[0] = o[1] > 0.0 ? sqrt(o[0]) / sqrt(o[1]) : 0.0;
    out[1] = sqrt(o[0]);
  }
}

// x += d
__global__ void __launch_bounds__(RED_THREADS) k_axpy1(Vec a, const double *d) {
  double xv[U], dv[U];
  VLOOP(xv[u] = ok ? a.x[i] : 0.0; dv[u] = ok ? d[i] : 0.0;,
        a.x[i] = xv[u] + dv[u];)
}

// ------- FP32-vector BiCGStab (the inner solves of the mixed path) -------
// Vectors are FP32; every inner product and norm accumulates exact FP32
// two-products per thread in double-float (TwoSum) and is reduced across
// the grid in FP64; all Krylov scalars stay FP64 in KState.  The operator is
// the FP32 store applied to FP32 vectors (launch_stored_apply32v), so no
// float<->double conversion (an FP64-pipe operation on GB300) runs per node.
struct Vec32 {
  int n;
  KState *st;
  double *partials;
  const float *dinv;
  const unsigned char *m;
  float *b, *x, *r, *rh, *p, *v, *ph, *s, *sh, *t;
};

__device__ __forceinline__ void dot_acc(DfAcc &a, float x, float y) {
  const float p = __fmul_rn(x, y);
  const float e = __fmaf_rn(x, y, -p);
  const float t = __fadd_rn(a.s, p);
  const float bp = __fsub_rn(t, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  a.s = t;
  a.c = __fadd_rn(a.c, __fadd_rn(err, e));
}
__device__ __forceinline__ double dot_val(const DfAcc &a) {
  return df_to_double(a.s, a.c);
}

// x = 0, r = rh = b, rho = ||b||^2.
__global__ void __launch_bounds__(RED_THREADS) k32_start(Vec32 a) {
  DfAcc n2{0.f, 0.f};
  float bv[U];
  VLOOP(bv[u] = ok ? a.b[i] : 0.f;,
        a.x[i] = 0.f;
        a.r[i] = bv[u];
        a.rh[i] = bv[u];
        dot_acc(n2, bv[u], bv[u]);)
  double v[1] = {dot_val(n2)};
  double o[1];
  if (grid_sum<1>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    st->bnrm2 = o[0];
    st->iter = 0;
    st->sconv = 0;
    st->status = VDR_NOT_CONVERGED;
    st->done = 0;
    st->rho = o[0];
    st->rho_old = 1.0;
    st->alpha = 1.0;
    st->omega = 1.0;
    st->reason = 0;
    if (o[0] == 0.0) {
      st->err = 0.0;
      st->status = VDR_OK;
      st->done = 1;
      return;
    }
    st->err = 1.0;
    if (!finite(o[0])) {
      st->status = VDR_BREAKDOWN;
      st->reason = 5;
      st->done = 1;
    } else if (st->err <= st->tol) {
      st->status = VDR_OK;
      st->done = 1;
    } else if (st->itmax <= 0) {
      st->done = 1;
    }
  }
}

// p = r + beta (p - omega v); ph = M^-1 p (0 on Dirichlet); v = 0.
// JAC = false: the operator carries the Jacobi scale and the Dirichlet
// projection (the binary16 store), so p itself is the apply's input and
// neither ph nor the diagonal and mask are touched.
template <bool JAC>
__global__ void __launch_bounds__(RED_THREADS) b32_p(Vec32 a) {
  const KState *st = a.st;
  if (st->done) return;
  const bool first = st->iter == 0;
  const float beta =
      first ? 0.f : (float)((st->rho / st->rho_old) * (st->alpha / st->omega));
  const float om = (float)st->omega;
  float rv[U], pv[U], vv[U], dv[U];
  unsigned char mv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.f; pv[u] = (ok && !first) ? a.p[i] : 0.f;
        vv[u] = (ok && !first) ? a.v[i] : 0.f;
        dv[u] = (JAC && ok) ? a.dinv[i] : 0.f; mv[u] = (JAC && ok) ? a.m[i] : 1;,
        const float pi = first ? rv[u] : rv[u] + beta * (pv[u] - om * vv[u]);
        a.p[i] = pi;
        if (JAC) a.ph[i] = mv[u] ? 0.f : pi * dv[u];
        a.v[i] = 0.f;)
}

// alpha = rho / (rh, v)
__global__ void __launch_bounds__(RED_THREADS) b32_alpha(Vec32 a) {
  if (a.st->done) return;
  DfAcc d{0.f, 0.f};
  float hv[U], vv[U];
  VLOOP(hv[u] = ok ? a.rh[i] : 0.f; vv[u] = ok ? a.v[i] : 0.f;,
        dot_acc(d, hv[u], vv[u]);)
  double v[1] = {dot_val(d)};
  double o[1];
  if (grid_sum<1>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    if (o[0] == 0.0 || !finite(o[0])) {
      st->status = VDR_BREAKDOWN;
      st->reason = 2;
      st->done = 1;
    } else {
      st->alpha = st->rho / o[0];
    }
  }
}

// s = r - alpha v; sh = M^-1 s (JAC only); t = 0; ||s||.
template <bool JAC>
__global__ void __launch_bounds__(RED_THREADS) b32_s(Vec32 a) {
  if (a.st->done) return;
  const float al = (float)a.st->alpha;
  DfAcc n2{0.f, 0.f};
  float rv[U], vv[U], dv[U];
  unsigned char mv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.f; vv[u] = ok ? a.v[i] : 0.f;
        dv[u] = (JAC && ok) ? a.dinv[i] : 0.f; mv[u] = (JAC && ok) ? a.m[i] : 1;,
        const float si = rv[u] - al * vv[u];
        a.s[i] = si;
        if (JAC) a.sh[i] = mv[u] ? 0.f : si * dv[u];
        a.t[i] = 0.f;
        dot_acc(n2, si, si);)
  double v[1] = {dot_val(n2)};
  double o[1];
  if (grid_sum<1>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    st->snrm = sqrt(o[0]) / sqrt(st->bnrm2);
    if (st->snrm <= st->tol) st->sconv = 1;
  }
}

// omega = (t, s) / (t, t)
__global__ void __launch_bounds__(RED_THREADS) b32_omega(Vec32 a) {
  if (a.st->done || a.st->sconv) return;
  DfAcc ts{0.f, 0.f}, tt{0.f, 0.f};
  float tv[U], sv[U];
  VLOOP(tv[u] = ok ? a.t[i] : 0.f; sv[u] = ok ? a.s[i] : 0.f;,
        dot_acc(ts, tv[u], sv[u]);
        dot_acc(tt, tv[u], tv[u]);)
  double v[2] = {dot_val(ts), dot_val(tt)};
  double o[2];
  if (grid_sum<2>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    if (o[1] == 0.0 || !finite(o[1]) || !finite(o[0])) {
      st->status = VDR_BREAKDOWN;
      st->reason = 3;
      st->done = 1;
    } else {
      st->omega = o[0] / o[1];
    }
  }
}

// x += alpha ph + omega sh (JAC = false: alpha p + omega s); r = s - omega t;
// rho_new = (rh, r); ||r||.
template <bool JAC>
__global__ void __launch_bounds__(RED_THREADS) b32_xr(Vec32 a) {
  KState *stc = a.st;
  if (stc->done) return;
  const float al = (float)stc->alpha;
  const float *ph = JAC ? a.ph : a.p;
  const float *sh = JAC ? a.sh : a.s;
  if (stc->sconv) {
    float xv[U], pv[U], sv[U];
    VLOOP(xv[u] = ok ? a.x[i] : 0.f; pv[u] = ok ? ph[i] : 0.f;
          sv[u] = ok ? a.s[i] : 0.f;,
          a.x[i] = xv[u] + al * pv[u];
          a.r[i] = sv[u];)
    double v[1] = {0.0};
    double o[1];
    if (grid_sum<1>(v, a.partials, &a.st->ticket, o)) {
      KState *st = a.st;
      st->iter += 1;
      st->err = st->snrm;
      st->status = VDR_OK;
      st->done = 1;
    }
    return;
  }
  const float om = (float)stc->omega;
  DfAcc rr{0.f, 0.f}, hr{0.f, 0.f};
  float xv[U], pv[U], shv[U], sv[U], tv[U], hv[U];
  VLOOP(xv[u] = ok ? a.x[i] : 0.f; pv[u] = ok ? ph[i] : 0.f;
        shv[u] = ok ? sh[i] : 0.f; sv[u] = ok ? a.s[i] : 0.f;
        tv[u] = ok ? a.t[i] : 0.f; hv[u] = ok ? a.rh[i] : 0.f;,
        a.x[i] = xv[u] + al * pv[u] + om * shv[u];
        const float ri = sv[u] - om * tv[u];
        a.r[i] = ri;
        dot_acc(rr, ri, ri);
        dot_acc(hr, hv[u], ri);)
  double v[2] = {dot_val(rr), dot_val(hr)};
  double o[2];
  if (grid_sum<2>(v, a.partials, &a.st->ticket, o)) {
    KState *st = a.st;
    const double om64 = st->omega;
    st->iter += 1;
    st->rho_old = st->rho;
    st->rho = o[1];
    st->err = sqrt(o[0]) / sqrt(st->bnrm2);
    if (!(st->err == st->err) || !finite(o[1])) {
      st->status = VDR_BREAKDOWN;
      st->reason = 5;
      st->done = 1;
    } else if (st->err <= st->tol) {
      st->status = VDR_OK;
      st->done = 1;
    } else if (o[1] == 0.0 || om64 == 0.0) {
      st->status = VDR_BREAKDOWN;
      st->reason = o[1] == 0.0 ? 1 : 4;
      st->done = 1;
    } else if (st->iter >= st->itmax) {
      st->status = VDR_NOT_CONVERGED;
      st->done = 1;
    }
  }
}

// ---- the FP32 inner iteration as two persistent, fused vector kernels ----
// With the binary16 operator (which carries the Jacobi scale and the
// Dirichlet projection) an inner iteration is apply(p -> v), fused alpha +
// s, apply(s -> t), fused omega + x, r + the next p: two cooperative
// kernels instead of five launches, and the vectors a phase re-reads after
// a grid-wide reduction (v, t, s, r, p; 4 bytes a node) mostly come back
// from L2.  Between the phases of one kernel the grid meets at a barrier;
// every block then adds all blocks' partial sums in the same fixed order,
// so every block holds the same scalars (bit-identical) and block 0 writes
// them to KState.  The launch is cooperative (all blocks resident), and the
// barrier's wait is bounded: a block whose wait runs out marks the solve
// VDR_TIMEOUT (reason 7) and returns.
constexpr long long BAR_LIMIT = 2000000000LL;  // ~1 s of clocks

__device__ bool grid_barrier(KState *st, long long limit = BAR_LIMIT) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = &st->bar_gen;
    const unsigned g0 = *gen;  // cannot advance before this block arrives
    __threadfence();
    bool ok = true;
    if (atomicAdd(&st->bar_count, 1u) == gridDim.x - 1) {
      atomicExch(&st->bar_count, 0u);
      __threadfence();
      atomicAdd(&st->bar_gen, 1u);
    } else {
      const long long t0 = clock64();
      while (*gen == g0) {
        if (clock64() - t0 > limit) {
          ok = false;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

__device__ void barrier_timeout(KState *st) {
  if (threadIdx.x == 0) {
    st->status = VDR_TIMEOUT;
    st->reason = 7;
    st->done = 1;
  }
}

// The barrier's failure path on its own: block 1 of a two-block cooperative
// launch returns at once and never arrives, block 0 waits with a short
// limit, gives up and marks the state VDR_TIMEOUT.
__global__ void barrier_timeout_kernel(KState *st, long long limit) {
  if (blockIdx.x != 0) return;
  if (!grid_barrier(st, limit)) barrier_timeout(st);
}

// This block's sums of NQ quantities into partials[q * gridDim.x + block].
template <int NQ>
__device__ __forceinline__ void put_partials(double (&v)[NQ], double *partials) {
  block_sum<NQ>(v);
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++) partials[q * gridDim.x + blockIdx.x] = v[q];
}
// After a barrier: the grid totals, added in a fixed order, in every thread.
template <int NQ>
__device__ __forceinline__ void all_sum(const double *partials, double (&out)[NQ]) {
  __shared__ double res[NQ];
  double w[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    w[q] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
      w[q] += __ldcg(partials + q * gridDim.x + b);
  }
  block_sum<NQ>(w);
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++) res[q] = w[q];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; q++) out[q] = res[q];
}

// alpha = rho / (rh, v); s = r - alpha v; t = 0; ||s||.
__global__ void __launch_bounds__(RED_THREADS, 4) b32f_alpha_s(Vec32 a) {
  KState *st = a.st;
  if (st->done) return;
  double *pa = a.partials, *pb = a.partials + MAXQ * gridDim.x;
  const double rho = st->rho;
  {
    DfAcc d{0.f, 0.f};
    float hv[U], vv[U];
    VLOOP(hv[u] = ok ? a.rh[i] : 0.f; vv[u] = ok ? a.v[i] : 0.f;,
          dot_acc(d, hv[u], vv[u]);)
    double v[1] = {dot_val(d)};
    put_partials<1>(v, pa);
  }
  if (!grid_barrier(st)) {
    barrier_timeout(st);
    return;
  }
  double o[1];
  all_sum<1>(pa, o);
  if (o[0] == 0.0 || !finite(o[0])) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->status = VDR_BREAKDOWN;
      st->reason = 2;
      st->done = 1;
    }
    return;
  }
  const double alpha = rho / o[0];
  if (blockIdx.x == 0 && threadIdx.x == 0) st->alpha = alpha;
  const float al = (float)alpha;
  DfAcc n2{0.f, 0.f};
  float rv[U], vv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.f; vv[u] = ok ? a.v[i] : 0.f;,
        const float si = rv[u] - al * vv[u];
        a.s[i] = si;
        a.t[i] = 0.f;
        dot_acc(n2, si, si);)
  double v[1] = {dot_val(n2)};
  double o2[1];
  if (grid_sum<1>(v, pb, &st->ticket, o2)) {
    st->snrm = sqrt(o2[0]) / sqrt(st->bnrm2);
    if (st->snrm <= st->tol) st->sconv = 1;
  }
}

// omega = (t, s) / (t, t); x += alpha p + omega s; r = s - omega t; rho =
// (rh, r), ||r||, convergence; then, unless done, the next iteration's
// p = r + beta (p - omega v), v = 0.
__global__ void __launch_bounds__(RED_THREADS, 3) b32f_omega_xr_p(Vec32 a) {
  KState *st = a.st;
  if (st->done) return;
  const float al = (float)st->alpha;
  if (st->sconv) {  // s met the tolerance: x += alpha p, r = s
    float xv[U], pv[U], sv[U];
    VLOOP(xv[u] = ok ? a.x[i] : 0.f; pv[u] = ok ? a.p[i] : 0.f;
          sv[u] = ok ? a.s[i] : 0.f;,
          a.x[i] = xv[u] + al * pv[u];
          a.r[i] = sv[u];)
    double v[1] = {0.0};
    double o[1];
    if (grid_sum<1>(v, a.partials, &st->ticket, o)) {
      st->iter += 1;
      st->err = st->snrm;
      st->status = VDR_OK;
      st->done = 1;
    }
    return;
  }
  double *pa = a.partials, *pb = a.partials + MAXQ * gridDim.x;
  // everything read from KState before block 0 writes it
  const double rho0 = st->rho, alpha = st->alpha, bnrm2 = st->bnrm2, tol = st->tol;
  const int iter0 = st->iter, itmax = st->itmax;
  {
    DfAcc ts{0.f, 0.f}, tt{0.f, 0.f};
    float tv[U], sv[U];
    VLOOP(tv[u] = ok ? a.t[i] : 0.f; sv[u] = ok ? a.s[i] : 0.f;,
          dot_acc(ts, tv[u], sv[u]);
          dot_acc(tt, tv[u], tv[u]);)
    double v[2] = {dot_val(ts), dot_val(tt)};
    put_partials<2>(v, pa);
  }
  if (!grid_barrier(st)) {
    barrier_timeout(st);
    return;
  }
  double o[2];
  all_sum<2>(pa, o);
  if (o[1] == 0.0 || !finite(o[1]) || !finite(o[0])) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->status = VDR_BREAKDOWN;
      st->reason = 3;
      st->done = 1;
    }
    return;
  }
  const double omega = o[0] / o[1];
  const float om = (float)omega;
  {
    DfAcc rr{0.f, 0.f}, hr{0.f, 0.f};
    float xv[U], pv[U], sv[U], tv[U], hv[U];
    VLOOP(xv[u] = ok ? a.x[i] : 0.f; pv[u] = ok ? a.p[i] : 0.f; sv[u] = ok ? a.s[i] : 0.f;
          tv[u] = ok ? a.t[i] : 0.f; hv[u] = ok ? a.rh[i] : 0.f;,
          a.x[i] = xv[u] + al * pv[u] + om * sv[u];
          const float ri = sv[u] - om * tv[u];
          a.r[i] = ri;
          dot_acc(rr, ri, ri);
          dot_acc(hr, hv[u], ri);)
    double v[2] = {dot_val(rr), dot_val(hr)};
    put_partials<2>(v, pb);
  }
  if (!grid_barrier(st)) {
    barrier_timeout(st);
    return;
  }
  double o2[2];
  all_sum<2>(pb, o2);
  // the convergence decision, identical in every block
  const double err = sqrt(o2[0]) / sqrt(bnrm2);
  const int iter = iter0 + 1;
  int status = VDR_NOT_CONVERGED, reason = 0;
  bool done = true;
  if (!(err == err) || !finite(o2[1])) {
    status = VDR_BREAKDOWN;
    reason = 5;
  } else if (err <= tol) {
    status = VDR_OK;
  } else if (o2[1] == 0.0 || omega == 0.0) {
    status = VDR_BREAKDOWN;
    reason = o2[1] == 0.0 ? 1 : 4;
  } else if (iter >= itmax) {
    status = VDR_NOT_CONVERGED;
  } else {
    done = false;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->omega = omega;
    st->iter = iter;
    st->rho_old = rho0;
    st->rho = o2[1];
    st->err = err;
    if (done) {
      st->status = status;
      if (reason) st->reason = reason;
      st->done = 1;
    }
  }
  if (done) return;
  // the next iteration's search direction (r and p just passed through L2)
  const float beta = (float)((o2[1] / rho0) * (alpha / omega));
  float rv[U], pv[U], vv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.f; pv[u] = ok ? a.p[i] : 0.f; vv[u] = ok ? a.v[i] : 0.f;,
        a.p[i] = rv[u] + beta * (pv[u] - om * vv[u]);
        a.v[i] = 0.f;)
}

// The cooperative grid of a fused kernel: at most the blocks that fit on
// the device at once (its own resident blocks per SM, cached in `slot`).
template <typename Kern>
int fused_grid(Kern kern, std::atomic<int> &slot, int n) {
  int per_sm = slot.load(std::memory_order_relaxed);
  if (per_sm <= 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RED_THREADS, 0);
    if (per_sm < 1) per_sm = 1;
    slot.store(per_sm, std::memory_order_relaxed);
  }
  const long need = ((long)n + RED_THREADS - 1) / RED_THREADS;
  return (int)std::max<long>(1, std::min<long>(need, (long)device_sm_count() * std::min(per_sm, 8)));
}
std::atomic<int> g_occ_alpha_s{0}, g_occ_omega_xr_p{0};

template <typename Kern>
cudaError_t launch_cooperative(Kern kern, int grid, const Vec32 &a, cudaStream_t s) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(RED_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, a);
}

// The FP64 Jacobi-BiCGStab iteration in the same two-kernel form (right
// preconditioned: p^ = D^-1 p and s^ = D^-1 s, zero on Dirichlet nodes, are
// the applies' inputs): apply(p^ -> v), fused alpha + s + s^, apply(s^ ->
// t), fused omega + x, r + next p + p^.
__global__ void __launch_bounds__(RED_THREADS, 2) bsf_alpha_s(Vec a) {
  KState *st = a.st;
  if (st->done) return;
  double *pa = a.partials, *pb = a.partials + MAXQ * gridDim.x;
  const double rho = st->rho;
  {
    double v[1] = {0.0};
    double hv[U], vv[U];
    VLOOP(hv[u] = ok ? a.rh[i] : 0.0; vv[u] = ok ? a.v[i] : 0.0;, v[0] += hv[u] * vv[u];)
    put_partials<1>(v, pa);
  }
  if (!grid_barrier(st)) {
    barrier_timeout(st);
    return;
  }
  double o[1];
  all_sum<1>(pa, o);
  if (o[0] == 0.0 || !finite(o[0])) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->status = VDR_BREAKDOWN;
      st->reason = 2;
      st->done = 1;
    }
    return;
  }
  const double al = rho / o[0];
  if (blockIdx.x == 0 && threadIdx.x == 0) st->alpha = al;
  double v[1] = {0.0};
  double rv[U], vv[U], dv[U];
  unsigned char mv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.0; vv[u] = ok ? a.v[i] : 0.0;
        dv[u] = ok ? a.dinv[i] : 0.0; mv[u] = ok ? a.m[i] : 1;,
        const double si = rv[u] - al * vv[u];
        a.s[i] = si;
        a.sh[i] = mv[u] ? 0.0 : si * dv[u];
        a.t[i] = 0.0;
        v[0] += si * si;)
  double o2[1];
  if (grid_sum<1>(v, pb, &st->ticket, o2)) {
    st->snrm = sqrt(o2[0]) / sqrt(st->bnrm2);
    if (st->snrm <= st->tol) st->sconv = 1;
  }
}

__global__ void __launch_bounds__(RED_THREADS, 2) bsf_omega_xr_p(Vec a) {
  KState *st = a.st;
  if (st->done) return;
  const double al = st->alpha;
  if (st->sconv) {  // s met the tolerance: x += alpha p^, r = s
    double xv[U], pv[U], sv[U];
    VLOOP(xv[u] = ok ? a.x[i] : 0.0; pv[u] = ok ? a.ph[i] : 0.0;
          sv[u] = ok ? a.s[i] : 0.0;,
          a.x[i] = xv[u] + al * pv[u];
          a.r[i] = sv[u];)
    double v[1] = {0.0};
    double o[1];
    if (grid_sum<1>(v, a.partials, &st->ticket, o)) {
      st->iter += 1;
      st->err = st->snrm;
      st->status = VDR_OK;
      st->done = 1;
    }
    return;
  }
  double *pa = a.partials, *pb = a.partials + MAXQ * gridDim.x;
  // everything read from KState before block 0 writes it
  const double rho0 = st->rho, bnrm2 = st->bnrm2, tol = st->tol, best0 = st->best_err;
  const int iter0 = st->iter, itmax = st->itmax, window = st->stall_window,
            since0 = st->since_best;
  {
    double v[2] = {0.0, 0.0};
    double tv[U], sv[U];
    VLOOP(tv[u] = ok ? a.t[i] : 0.0; sv[u] = ok ? a.s[i] : 0.0;,
          v[0] += tv[u] * sv[u];
          v[1] += tv[u] * tv[u];)
    put_partials<2>(v, pa);
  }
  if (!grid_barrier(st)) {
    barrier_timeout(st);
    return;
  }
  double o[2];
  all_sum<2>(pa, o);
  if (o[1] == 0.0 || !finite(o[1]) || !finite(o[0])) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->status = VDR_BREAKDOWN;
      st->reason = 3;
      st->done = 1;
    }
    return;
  }
  const double om = o[0] / o[1];
  {
    double v[2] = {0.0, 0.0};
    double xv[U], pv[U], shv[U], sv[U], tv[U], hv[U];
    VLOOP(xv[u] = ok ? a.x[i] : 0.0; pv[u] = ok ? a.ph[i] : 0.0;
          shv[u] = ok ? a.sh[i] : 0.0; sv[u] = ok ? a.s[i] : 0.0;
          tv[u] = ok ? a.t[i] : 0.0; hv[u] = ok ? a.rh[i] : 0.0;,
          a.x[i] = xv[u] + al * pv[u] + om * shv[u];
          const double ri = sv[u] - om * tv[u];
          a.r[i] = ri;
          v[0] += ri * ri;
          v[1] += hv[u] * ri;)
    put_partials<2>(v, pb);
  }
  if (!grid_barrier(st)) {
    barrier_timeout(st);
    return;
  }
  double o2[2];
  all_sum<2>(pb, o2);
  // the convergence decision, identical in every block
  const double err = sqrt(o2[0]) / sqrt(bnrm2);
  const int iter = iter0 + 1;
  int status = VDR_NOT_CONVERGED, reason = 0;
  bool done = true;
  double best = best0;
  int since = since0;
  if (!(err == err) || !finite(o2[1])) {
    status = VDR_BREAKDOWN;
    reason = 5;
  } else if (err <= tol) {
    status = VDR_OK;
  } else if (o2[1] == 0.0 || om == 0.0) {
    status = VDR_BREAKDOWN;
    reason = o2[1] == 0.0 ? 1 : 4;
  } else if (iter >= itmax) {
    status = VDR_NOT_CONVERGED;
  } else {
    done = false;
    if (window > 0) {
      if (err < 0.99 * best) {
        best = err;
        since = 0;
      } else if (++since >= window) {
        status = VDR_NOT_CONVERGED;
        reason = 6;  // stalled
        done = true;
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->omega = om;
    st->iter = iter;
    st->rho_old = rho0;
    st->rho = o2[1];
    st->err = err;
    st->best_err = best;
    st->since_best = since;
    if (done) {
      st->status = status;
      if (reason) st->reason = reason;
      st->done = 1;
    }
  }
  if (done) return;
  // the next iteration's search direction and its Jacobi image
  const double beta = (o2[1] / rho0) * (al / om);
  double rv[U], pv[U], vv[U], dv[U];
  unsigned char mv[U];
  VLOOP(rv[u] = ok ? a.r[i] : 0.0; pv[u] = ok ? a.p[i] : 0.0; vv[u] = ok ? a.v[i] : 0.0;
        dv[u] = ok ? a.dinv[i] : 0.0; mv[u] = ok ? a.m[i] : 1;,
        const double pi = rv[u] + beta * (pv[u] - om * vv[u]);
        a.p[i] = pi;
        a.ph[i] = mv[u] ? 0.0 : pi * dv[u];
        a.v[i] = 0.0;)
}

template <typename Kern>
cudaError_t launch_cooperative64(Kern kern, int grid, const Vec &a, cudaStream_t s) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(RED_THREADS);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, a);
}
std::atomic<int> g_occ_bsf_alpha_s{0}, g_occ_bsf_omega_xr_p{0};

cudaError_t launch_fused64_iteration(Handle &h, const Vec &a, cudaStream_t s) {
  cudaError_t e;
  if ((e = launch_apply(h, false, a.ph, a.v, &h.st->done, nullptr, s))) return e;
  if ((e = launch_cooperative64(bsf_alpha_s, fused_grid(bsf_alpha_s, g_occ_bsf_alpha_s, h.N),
                                a, s)))
    return e;
  if ((e = launch_apply(h, false, a.sh, a.t, &h.st->done, &h.st->sconv, s))) return e;
  return launch_cooperative64(bsf_omega_xr_p,
                              fused_grid(bsf_omega_xr_p, g_occ_bsf_omega_xr_p, h.N), a, s);
}

// b32 = (float)(r * scale); dinv32 = (float)dinv (when dinv32 is given).
__global__ void __launch_bounds__(RED_THREADS) k32_in(Vec32 a, const double *r,
                                                      double scale, const double *dinv,
                                                      float *dinv32) {
  double rv[U], dv[U];
  VLOOP(rv[u] = ok ? r[i] : 0.0; dv[u] = (ok && dinv32) ? dinv[i] : 0.0;,
        a.b[i] = (float)(rv[u] * scale);
        if (dinv32) dinv32[i] = (float)dv[u];)
}

// x += scale * x32, or (dinv given: the inner solve ran on A D^-1) x +=
// scale * dinv * x32 (FP64 update).
__global__ void __launch_bounds__(RED_THREADS) k32_out(Vec32 a, double *x, double scale,
                                                       const double *dinv) {
  double xv[U], sv[U];
  float dv[U];
  VLOOP(xv[u] = ok ? x[i] : 0.0; dv[u] = ok ? a.x[i] : 0.f;
        sv[u] = (ok && dinv) ? dinv[i] : 1.0;,
        x[i] = xv[u] + scale * sv[u] * (double)dv[u];)
}

Vec32 make_vec32(Handle &h) {
  Vec32 a{};
  a.n = h.N;
  a.st = h.st;
  a.partials = h.partials;
  a.dinv = h.dinv32;
  a.m = h.mask;
  float *w = h.work32;
  const size_t N = h.N;
  a.b = w;
  a.x = w + N;
  a.r = w + 2 * N;
  a.rh = w + 3 * N;
  a.p = w + 4 * N;
  a.v = w + 5 * N;
  a.ph = w + 6 * N;
  a.s = w + 7 * N;
  a.sh = w + 8 * N;
  a.t = w + 9 * N;
  return a;
}

cudaError_t launch_iteration32(Handle &h, const Vec32 &a) {
  const int g = red_grid(h.N);
  cudaStream_t s = h.stream;
  cudaError_t e;
  if (h.use_half && h.fused32) {  // p formed by the previous iteration's fused kernel
    if ((e = launch_apply_half(h, a.p, a.v, &h.st->done, nullptr, s))) return e;
    if ((e = launch_cooperative(b32f_alpha_s, fused_grid(b32f_alpha_s, g_occ_alpha_s, h.N), a,
                                s)))
      return e;
    if ((e = launch_apply_half(h, a.s, a.t, &h.st->done, &h.st->sconv, s))) return e;
    return launch_cooperative(b32f_omega_xr_p,
                              fused_grid(b32f_omega_xr_p, g_occ_omega_xr_p, h.N), a, s);
  }
  if (h.use_half) {  // A D^-1 in binary16: no preconditioner vectors
    b32_p<false><<<g, RED_THREADS, 0, s>>>(a);
    if ((e = launch_apply_half(h, a.p, a.v, &h.st->done, nullptr, s))) return e;
    b32_alpha<<<g, RED_THREADS, 0, s>>>(a);
    b32_s<false><<<g, RED_THREADS, 0, s>>>(a);
    if ((e = launch_apply_half(h, a.s, a.t, &h.st->done, &h.st->sconv, s))) return e;
    b32_omega<<<g, RED_THREADS, 0, s>>>(a);
    b32_xr<false><<<g, RED_THREADS, 0, s>>>(a);
    return cudaGetLastError();
  }
  b32_p<true><<<g, RED_THREADS, 0, s>>>(a);
  if ((e = launch_stored_apply32v(h, a.ph, a.v, &h.st->done, nullptr, s))) return e;
  b32_alpha<<<g, RED_THREADS, 0, s>>>(a);
  b32_s<true><<<g, RED_THREADS, 0, s>>>(a);
  if ((e = launch_stored_apply32v(h, a.sh, a.t, &h.st->done, &h.st->sconv, s))) return e;
  b32_omega<<<g, RED_THREADS, 0, s>>>(a);
  b32_xr<true><<<g, RED_THREADS, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

// The fused kernels' barrier timeout, end to end: VDR_TIMEOUT when the wait
// that nothing completes ran out of its (about 1 ms) budget and the state
// said so; the handle stays usable (the next solve resets the state).
int diag_barrier_timeout(Handle &h) {
  cudaError_t e = ensure_solver_workspace(h, 8);
  if (e) return cuda_fail(e, "diag");
  cudaStream_t s = h.stream;
  if ((e = cudaMemsetAsync(h.st, 0, sizeof(KState), s))) return cuda_fail(e, "diag");
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(2);
  cfg.blockDim = dim3(32);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if ((e = cudaLaunchKernelEx(&cfg, barrier_timeout_kernel, h.st, 2000000LL)))
    return cuda_fail(e, "diag launch");
  count_launches(1);
  KState fin;
  if ((e = cudaMemcpyAsync(&fin, h.st, sizeof(KState), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "diag");
  if (fin.done && fin.status == VDR_TIMEOUT && fin.reason == 7) {
    set_error("diag: the grid barrier's wait ran out (as intended)");
    return VDR_TIMEOUT;
  }
  set_error("diag: the grid barrier did not report its timeout");
  return VDR_CUDA_ERROR;
}

namespace {
// Inner solve A32 x32 = b32 (FP32 vectors in work32, x32 from zero) to `tol`
// relative residual; graph-captured like solve_device.
int solve32_inner(Handle &h, double tol, int itmax, int *iter, double *err) {
  cudaError_t e;
  if (!h.work32 && (e = cudaMalloc(&h.work32, sizeof(float) * 10 * (size_t)h.N)))
    return cuda_fail(e, "FP32 workspace");
  cudaStream_t s = h.stream;
  Vec32 a = make_vec32(h);
  const int g = red_grid(h.N);
  KState init{};
  init.tol = tol;
  init.itmax = itmax;
  init.best_err = INFINITY;
  std::memcpy(&h.h_st[0], &init, sizeof(KState));
  if ((e = cudaMemcpyAsync(h.st, &h.h_st[0], sizeof(KState), cudaMemcpyHostToDevice, s)))
    return cuda_fail(e, "state upload");
  k32_start<<<g, RED_THREADS, 0, s>>>(a);
  count_launches(1);
  if ((e = cudaGetLastError())) return cuda_fail(e, "start kernel");
  const int K = h.opt.iters_per_graph > 0 ? h.opt.iters_per_graph : 8;
  for (int attempt = 0; attempt < 2; attempt++) {
    const bool fused = h.use_half && h.fused32;
    const void *key = (const void *)((uintptr_t)h.work32 ^ ((uintptr_t)h.A32v << 1) ^
                                     (uintptr_t)K ^ ((uintptr_t)h.scatter << 12) ^
                                     ((uintptr_t)h.use_half << 20) ^
                                     ((uintptr_t)h.A16 << 2) ^ ((uintptr_t)fused << 21));
    if (h.graph32 && h.graph32_key == key) break;
    if (h.graph32) cudaGraphExecDestroy(h.graph32);
    h.graph32 = nullptr;
    cudaGraph_t graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)))
      return cuda_fail(e, "begin capture");
    const long long before = launches_so_far();
    for (int k = 0; k < K && !e; k++) e = launch_iteration32(h, a);
    count_launches(before - launches_so_far());  // captured, not launched
    cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (!e && !e2) {
      e = cudaGraphInstantiate(&h.graph32, graph, 0);
      cudaGraphDestroy(graph);
      if (!e) {
        h.graph32_key = key;
        break;
      }
      h.graph32 = nullptr;
    } else if (!e2) {
      cudaGraphDestroy(graph);
    }
    // a cooperative launch that the capture or the graph refuses: the
    // unfused kernels instead
    if (fused) {
      cudaGetLastError();
      h.fused32 = false;
      e = cudaSuccess;
      continue;
    }
    if (e) return cuda_fail(e, "capture");
    if (e2) return cuda_fail(e2, "end capture");
  }
  if (h.use_half && h.fused32) {  // the first search direction p = r, v = 0
    b32_p<false><<<g, RED_THREADS, 0, s>>>(a);
    count_launches(1);
    if ((e = cudaGetLastError())) return cuda_fail(e, "first direction");
  }
  const long nodes = (h.use_half && h.fused32) ? 4 : 5 + 2 * (h.use_half ? 1 : apply_launches(h));
  const int max_launches = (itmax + K - 1) / K + 1;
  bool finished = false;
  for (int c = 0; c < max_launches && !finished; c++) {
    if ((e = cudaGraphLaunch(h.graph32, s))) return cuda_fail(e, "graph launch");
    count_launches((long)K * nodes);
    if ((e = cudaMemcpyAsync(&h.h_st[c & 1], h.st, sizeof(KState),
                             cudaMemcpyDeviceToHost, s)))
      return cuda_fail(e, "state readback");
    if ((e = cudaEventRecord(h.ev[c & 1], s))) return cuda_fail(e, "event");
    if (c > 0) {
      if ((e = cudaEventSynchronize(h.ev[(c - 1) & 1]))) return cuda_fail(e, "sync");
      if (h.h_st[(c - 1) & 1].done) finished = true;
    }
  }
  if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "solve");
  KState fin;
  if ((e = cudaMemcpy(&fin, h.st, sizeof(KState), cudaMemcpyDeviceToHost)))
    return cuda_fail(e, "final state");
  if (iter) *iter = fin.iter;
  if (err) *err = fin.err;
  return fin.done ? fin.status : VDR_NOT_CONVERGED;
}
}  // namespace

// Iterative refinement: the residual r = b - A x and the update x += d are
// FP64 (FP64 operator); each correction d solves A32 d = r with the FP32
// operator to max(inner_tol, 0.5 tol / rel) relative to ||r|| (rel =
// ||r||/||b||): a correction is solved no further than the outer residual
// needs to reach tol, so a tight first correction is followed by a short
// second one instead of two full-depth inner solves.  With the stored
// operator and BiCGStab the inner solve runs on FP32 vectors (r scaled by
// 1/||r||, inner products in double-float/FP64); otherwise on FP64 vectors.
int solve_mixed_device(Handle &h, int method, const double *b, double *x,
                       double tol, double inner_tol, int max_outer,
                       int inner_itmax, MixedStats *ms) {
  cudaError_t e = ensure_solver_workspace(h, 11);
  if (e) return cuda_fail(e, "solver workspace");
  cudaStream_t s = h.stream;
  double *r = h.work + 8 * (size_t)h.N;
  double *d = h.work + 9 * (size_t)h.N;
  double *scal = h.work + 10 * (size_t)h.N;  // one double used
  Vec a = make_vec(h, b, x);
  const int g = red_grid(h.N);
  MixedStats st;
  int status = VDR_NOT_CONVERGED;
  // x masked; the first residual's A x is skipped when x is then zero
  if ((e = cudaMemsetAsync(&h.st->x_zero, 1, sizeof(int), s)) ||
      (e = launch_mask_vec_flag(x, h.mask, h.N, &h.st->x_zero, s)))
    return cuda_fail(e, "mask x");
  // The stored FP32 operator runs its inner BiCGStab on FP32 vectors.
  const bool f32v = h.apply_mode == VDR_APPLY_STORED && method == VDR_SOLVER_BICGSTAB;
  if (f32v && !h.dinv32 && (e = cudaMalloc(&h.dinv32, sizeof(float) * (size_t)h.N)))
    return cuda_fail(e, "FP32 diagonal");
  if (f32v && !h.work32 &&
      (e = cudaMalloc(&h.work32, sizeof(float) * 10 * (size_t)h.N)))
    return cuda_fail(e, "FP32 workspace");
  for (int outer = 0; outer <= max_outer; outer++) {
    h.apply_fp32 = false;
    if ((e = cudaMemsetAsync(r, 0, sizeof(double) * h.N, s)) ||
        (e = launch_apply(h, false, x, r, outer == 0 ? &h.st->x_zero : nullptr,
                          nullptr, s)))
      return cuda_fail(e, "outer residual");
    k_residual<<<g, RED_THREADS, 0, s>>>(a, r, scal);
    count_launches(1);
    double rr[2] = {0.0, 0.0};  // ||r||/||b||, ||r||
    if ((e = cudaMemcpyAsync(rr, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_fail(e, "outer residual");
    const double rel = rr[0];
    st.err = rel;
    if (rel <= tol) {
      status = VDR_OK;
      break;
    }
    if (!(rel == rel)) {
      status = VDR_BREAKDOWN;
      break;
    }
    if (outer == max_outer) break;
    st.outer = outer + 1;
    int it = 0;
    double ierr = 0.0;
    const double itol = std::max(inner_tol, 0.5 * tol / rel);
    if (f32v) {
      // d solves A32 d = r / ||r|| on FP32 vectors; x += ||r|| d in FP64
      if (!(1.0 / rr[1] < INFINITY)) break;  // ||r|| at the denormal floor
      Vec32 a32 = make_vec32(h);
      k32_in<<<g, RED_THREADS, 0, s>>>(a32, r, 1.0 / rr[1], h.dinv,
                                       h.use_half ? nullptr : h.dinv32);
      count_launches(1);
      h.apply_fp32 = true;
      const int ist = solve32_inner(h, itol, inner_itmax, &it, &ierr);
      h.apply_fp32 = false;
      if (ist == VDR_CUDA_ERROR || ist == VDR_BAD_ARGUMENT) return ist;
      k32_out<<<g, RED_THREADS, 0, s>>>(a32, x, rr[1],
                                        h.use_half ? h.dinv : nullptr);
      count_launches(1);
    } else {
      if ((e = cudaMemsetAsync(d, 0, sizeof(double) * h.N, s)))
        return cuda_fail(e, "memset");
      h.apply_fp32 = true;
      const int ist = solve_device(h, method, r, d, itol, inner_itmax, &it, &ierr);
      h.apply_fp32 = false;
      if (ist == VDR_CUDA_ERROR || ist == VDR_BAD_ARGUMENT) return ist;
      k_axpy1<<<g, RED_THREADS, 0, s>>>(a, d);
      count_launches(1);
    }
    st.inner += it;
    if ((e = cudaGetLastError())) return cuda_fail(e, "update");
  }
  if (ms) *ms = st;
  h.last.iterations = st.inner;
  h.last.status = status;
  return status;
}

// Relative true residual ||b - A x|| / ||b|| (FP64, device).
int true_residual_device(Handle &h, const double *b, const double *x,
                         double *rel) {
  cudaError_t e = ensure_solver_workspace(h, 8);
  if (e) return cuda_fail(e, "solver workspace");
  cudaStream_t s = h.stream;
  Vec a = make_vec(h, b, const_cast<double *>(x));
  double *ax = a.t;
  double *out = a.sh;  // scalar scratch
  if ((e = cudaMemsetAsync(ax, 0, sizeof(double) * h.N, s))) return cuda_fail(e, "memset");
  if ((e = launch_apply(h, false, x, ax, nullptr, nullptr, s))) return cuda_fail(e, "apply");
  const int g = red_grid(h.N);
  k_true_residual<<<g, RED_THREADS, 0, s>>>(a, ax, h.partials, &h.st->ticket, out);
  count_launches(1);
  if ((e = cudaGetLastError())) return cuda_fail(e, "residual");
  if ((e = cudaMemcpyAsync(rel, out, sizeof(double), cudaMemcpyDeviceToHost, s)))
    return cuda_fail(e, "readback");
  if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "sync");
  return VDR_OK;
}

}  // namespace vdr
