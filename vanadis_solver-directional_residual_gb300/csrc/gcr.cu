// gcr.cu -- restarted GCR(m), the flexible minimal-residual Krylov method
// for a right preconditioner that changes from one application to the next
// (the learned network), with Jacobi as the default preconditioner.
//
// Step k of a cycle (k = 0 .. m-1):
//   z_k = M(r)                 (D^-1 r, plus the network's correction)
//   c_k = A z_k
//   c_k -= sum_{j<k} (c_k, c_j) c_j ;  z_k -= the same combination of z_j
//   c_k, z_k scaled by 1/||c_k||
//   x += (r, c_k) z_k ;  r -= (r, c_k) c_k
// so ||r|| never increases, whatever M does.  M is applied to the current
// residual (the vectors the network was trained on), unlike BiCGStab, which
// applies it to search directions and relies on M being one fixed linear
// operator.  The cycle restarts after m steps (the c_j, z_j are dropped).
//
// All scalars are device-resident (KState plus a small array); every
// reduction is a per-block partial sum combined in a fixed order by the
// last block (deterministic for a fixed grid), so a whole cycle is captured
// as one CUDA graph and replayed until KState.done.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cstring>

#include "vdr_internal.h"

namespace vdr {
namespace {

constexpr int GT = 256;  // threads per block
constexpr unsigned FULLG = 0xffffffffu;

struct GcrArgs {
  long n;
  int m;             // restart length
  KState *st;
  double *sc;        // [GCR_MAX_RESTART] projections, then cc, rc
  double *partials;  // [GCR_MAX_RESTART + 2][gridDim.x]
  const double *b, *dinv;
  const unsigned char *mask;
  double *x, *r, *Z, *C;  // Z, C: [m][n]
};

// Grid sum of Q <= GCR_MAX_RESTART + 2 per-thread values.  The last block
// to finish combines the per-block partials: GT/Q threads per quantity take
// strided slices (four loads in flight), then one thread per quantity adds
// the slices in fixed order.  True in threads q < Q of the last block, with
// out[q] the totals.
constexpr int QMAX = GCR_MAX_RESTART + 2;
__device__ bool multi_sum(double (&v)[QMAX], int Q, const GcrArgs &a,
                          double *out) {
  __shared__ double sw[GT / 32][QMAX];
  __shared__ double sl[GT];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < QMAX; q++) {
    if (q < Q) {
      double x = v[q];
#pragma unroll
      for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(FULLG, x, off);
      if (lane == 0) sw[w][q] = x;
    }
  }
  __syncthreads();
  if (threadIdx.x < Q) {
    double x = 0.0;
    for (int j = 0; j < GT / 32; j++) x += sw[j][threadIdx.x];
    a.partials[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = x;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&a.st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  const int T = GT / Q;  // threads per quantity (>= 7)
  const int q = threadIdx.x % Q, sub = threadIdx.x / Q;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  if (sub < T) {
    const double *pp = a.partials + (size_t)q * gridDim.x;
    const int G = (int)gridDim.x;
    int b = sub;
    for (; b + 3 * T < G; b += 4 * T) {
      s0 += __ldcg(pp + b);
      s1 += __ldcg(pp + b + T);
      s2 += __ldcg(pp + b + 2 * T);
      s3 += __ldcg(pp + b + 3 * T);
    }
    for (; b < G; b += T) s0 += __ldcg(pp + b);
  }
  sl[threadIdx.x] = (s0 + s1) + (s2 + s3);
  __syncthreads();
  if (threadIdx.x < Q) {
    double s = 0.0;
    for (int u = 0; u < T; u++) s += sl[u * Q + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) a.st->ticket = 0u;
  return threadIdx.x < Q;
}

#define GLOOP(i) \
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; \
       i += (long)gridDim.x * blockDim.x)

// r = b - r (r holds A x0); ||b||, ||r||.
__global__ void __launch_bounds__(GT) g_start(GcrArgs a) {
  double v[QMAX];
#pragma unroll
  for (int q = 0; q < QMAX; q++) v[q] = 0.0;
  GLOOP(i) {
    const double bi = a.b[i];
    const double ri = bi - a.r[i];
    a.r[i] = ri;
    v[0] += bi * bi;
    v[1] += ri * ri;
  }
  __shared__ double out[QMAX];
  if (multi_sum(v, 2, a, out) && threadIdx.x == 0) {
    KState *st = a.st;
    st->bnrm2 = out[0];
    st->iter = 0;
    st->status = VDR_NOT_CONVERGED;
    st->reason = 0;
    st->done = 0;
    if (out[0] == 0.0) {
      st->err = 0.0;
      st->status = VDR_OK;
      st->done = 2;  // b = 0: x = 0
      return;
    }
    st->err = sqrt(out[1] / out[0]);
    st->best_err = st->err;
    st->since_best = 0;
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

// z_k = D^-1 r (0 on Dirichlet nodes); c_k = 0.
__global__ void __launch_bounds__(GT) g_jacobi(GcrArgs a, int k) {
  if (a.st->done) return;
  double *z = a.Z + (size_t)k * a.n, *c = a.C + (size_t)k * a.n;
  GLOOP(i) {
    z[i] = a.mask[i] ? 0.0 : a.r[i] * a.dinv[i];
    c[i] = 0.0;
  }
}

// sc[j] = (c_k, c_j), j < k.
__global__ void __launch_bounds__(GT) g_dots(GcrArgs a, int k) {
  if (a.st->done) return;
  const double *c = a.C + (size_t)k * a.n;
  double v[QMAX];
#pragma unroll
  for (int q = 0; q < QMAX; q++) v[q] = 0.0;
  GLOOP(i) {
    const double ci = c[i];
#pragma unroll
    for (int j = 0; j < GCR_MAX_RESTART; j++)
      if (j < k) v[j] += ci * a.C[(size_t)j * a.n + i];
  }
  __shared__ double out[QMAX];
  if (multi_sum(v, k, a, out)) a.sc[threadIdx.x] = out[threadIdx.x];
}

// c_k -= sum_j sc[j] c_j, z_k -= sum_j sc[j] z_j; cc = ||c_k||^2,
// rc = (r, c_k).
__global__ void __launch_bounds__(GT) g_update(GcrArgs a, int k) {
  if (a.st->done) return;
  double *c = a.C + (size_t)k * a.n, *z = a.Z + (size_t)k * a.n;
  double h[GCR_MAX_RESTART];
#pragma unroll
  for (int j = 0; j < GCR_MAX_RESTART; j++) h[j] = j < k ? a.sc[j] : 0.0;
  double v[QMAX];
#pragma unroll
  for (int q = 0; q < QMAX; q++) v[q] = 0.0;
  GLOOP(i) {
    double ci = c[i], zi = z[i];
#pragma unroll
    for (int j = 0; j < GCR_MAX_RESTART; j++)
      if (j < k) {
        ci -= h[j] * a.C[(size_t)j * a.n + i];
        zi -= h[j] * a.Z[(size_t)j * a.n + i];
      }
    c[i] = ci;
    z[i] = zi;
    v[0] += ci * ci;
    v[1] += a.r[i] * ci;
  }
  __shared__ double out[QMAX];
  if (multi_sum(v, 2, a, out) && threadIdx.x == 0) {
    KState *st = a.st;
    const double cc = out[0];
    if (!(cc > 0.0) || !isfinite(cc) || !isfinite(out[1])) {
      st->status = VDR_BREAKDOWN;
      st->reason = 3;
      st->done = 1;
    } else {
      a.sc[GCR_MAX_RESTART] = cc;
      a.sc[GCR_MAX_RESTART + 1] = out[1];
    }
  }
}

// c_k, z_k /= ||c_k||; x += (r, c_k) z_k; r -= (r, c_k) c_k; ||r||.
__global__ void __launch_bounds__(GT) g_xr(GcrArgs a, int k) {
  if (a.st->done) return;
  double *c = a.C + (size_t)k * a.n, *z = a.Z + (size_t)k * a.n;
  const double s = 1.0 / sqrt(a.sc[GCR_MAX_RESTART]);
  const double al = a.sc[GCR_MAX_RESTART + 1] * s;  // (r, c_k) with c_k unit
  double v[QMAX];
#pragma unroll
  for (int q = 0; q < QMAX; q++) v[q] = 0.0;
  GLOOP(i) {
    const double ci = c[i] * s, zi = z[i] * s;
    c[i] = ci;
    z[i] = zi;
    a.x[i] += al * zi;
    const double ri = a.r[i] - al * ci;
    a.r[i] = ri;
    v[0] += ri * ri;
  }
  __shared__ double out[QMAX];
  if (multi_sum(v, 1, a, out) && threadIdx.x == 0) {
    KState *st = a.st;
    st->iter += 1;
    st->err = sqrt(out[0] / st->bnrm2);
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
    } else if (st->stall_window > 0) {
      if (st->err < 0.99 * st->best_err) {
        st->best_err = st->err;
        st->since_best = 0;
      } else if (++st->since_best >= st->stall_window) {
        st->status = VDR_NOT_CONVERGED;
        st->reason = 6;
        st->done = 1;
      }
    }
  }
}

int gcr_grid(long n) {
  const long need = (n + GT - 1) / GT;
  return (int)std::max<long>(1, std::min<long>(need, (long)device_sm_count() * 2));
}

}  // namespace

// One step k of a cycle (jacobi, preconditioner, apply, orthogonalise,
// update).
cudaError_t gcr_step(Handle &h, const GcrArgs &a, int g, int k, const Precond *prec) {
  cudaStream_t s = h.stream;
  cudaError_t e;
  g_jacobi<<<g, GT, 0, s>>>(a, k);
  count_launches(1);
  if (prec &&
      (e = prec->enqueue(prec->ctx, a.r, a.Z + (size_t)k * h.N, &h.st->done, nullptr, s)))
    return e;
  if ((e = launch_apply(h, false, a.Z + (size_t)k * h.N, a.C + (size_t)k * h.N,
                        &h.st->done, nullptr, s)))
    return e;
  if (k > 0) {
    g_dots<<<g, GT, 0, s>>>(a, k);
    count_launches(1);
  }
  g_update<<<g, GT, 0, s>>>(a, k);
  g_xr<<<g, GT, 0, s>>>(a, k);
  count_launches(2);
  return cudaGetLastError();
}

int solve_gcr_device(Handle &h, const double *b, double *x, double tol,
                     int itmax, int m, const Precond *prec, int stall_window,
                     int *iter, double *err, double *hist, int max_hist,
                     int *n_hist) {
  if (m < 1 || m > GCR_MAX_RESTART) {
    set_error("GCR restart length must be 1.." + std::to_string(GCR_MAX_RESTART));
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e = ensure_solver_workspace(h, 8);  // KState, events
  if (e) return cuda_fail(e, "solver workspace");
  cudaStream_t s = h.stream;
  const int g = gcr_grid(h.N);
  const size_t need = (size_t)h.N * (1 + 2 * (size_t)m) + QMAX +
                      (size_t)QMAX * g;
  if (h.gcr_words < need) {
    if (h.gcr_work) cudaFree(h.gcr_work);
    h.gcr_work = nullptr;
    h.gcr_words = 0;
    if (h.gcr_graph) cudaGraphExecDestroy(h.gcr_graph);
    h.gcr_graph = nullptr;
    if ((e = cudaMalloc(&h.gcr_work, sizeof(double) * need))) return cuda_fail(e, "GCR workspace");
    h.gcr_words = need;
  }
  GcrArgs a{};
  a.n = h.N;
  a.m = m;
  a.st = h.st;
  a.r = h.gcr_work;
  a.Z = a.r + h.N;
  a.C = a.Z + (size_t)m * h.N;
  a.sc = a.C + (size_t)m * h.N;
  a.partials = a.sc + QMAX;
  a.b = b;
  a.x = x;
  a.dinv = h.dinv;
  a.mask = h.mask;
  h.last = vdr_solve_stats{};
  const long long launches0 = launches_so_far();

  KState init{};
  init.tol = tol;
  init.itmax = itmax;
  init.best_err = INFINITY;
  init.stall_window = stall_window;
  std::memcpy(&h.h_st[0], &init, sizeof(KState));
  if ((e = cudaMemcpyAsync(h.st, &h.h_st[0], sizeof(KState), cudaMemcpyHostToDevice, s)))
    return cuda_fail(e, "state upload");
  if ((e = launch_mask_vec(x, h.mask, h.N, s)) ||
      (e = cudaMemsetAsync(a.r, 0, sizeof(double) * h.N, s)) ||
      (e = launch_apply(h, false, x, a.r, nullptr, nullptr, s)))
    return cuda_fail(e, "GCR start");
  g_start<<<g, GT, 0, s>>>(a);
  count_launches(1);
  if ((e = cudaGetLastError())) return cuda_fail(e, "GCR start");

  if (hist && n_hist) {
    // Recording: iterations enqueued one by one (no graph), x copied after
    // each; kernels of finished solves return at entry.
    *n_hist = 0;
    int k = 0;
    for (int it = 0; it < itmax && *n_hist < max_hist; it++) {
      if ((e = gcr_step(h, a, g, k, prec))) return cuda_fail(e, "GCR step");
      if ((e = cudaMemcpyAsync(hist + (size_t)(*n_hist) * h.N, x, sizeof(double) * h.N,
                               cudaMemcpyDeviceToDevice, s)))
        return cuda_fail(e, "record iterate");
      (*n_hist)++;
      k = (k + 1) % m;
      if ((it & 7) == 7) {
        if ((e = cudaMemcpyAsync(&h.h_st[0], h.st, sizeof(KState), cudaMemcpyDeviceToHost, s)) ||
            (e = cudaStreamSynchronize(s)))
          return cuda_fail(e, "state");
        if (h.h_st[0].done) break;
      }
    }
  } else {
  const void *key = (const void *)((uintptr_t)b ^ ((uintptr_t)x << 1) ^
                                   ((uintptr_t)h.gcr_work << 2) ^ (uintptr_t)m ^
                                   ((uintptr_t)(prec ? prec->ctx : nullptr) << 3) ^
                                   ((uintptr_t)h.apply_mode << 8) ^
                                   ((uintptr_t)h.scatter << 12));
  long per_cycle = 0;
  if (!h.gcr_graph || h.gcr_key != key) {
    if (h.gcr_graph) cudaGraphExecDestroy(h.gcr_graph);
    h.gcr_graph = nullptr;
    cudaGraph_t graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)))
      return cuda_fail(e, "begin capture");
    const long long before = launches_so_far();
    for (int k = 0; k < m && !e; k++) e = gcr_step(h, a, g, k, prec);
    per_cycle = (long)(launches_so_far() - before);
    h.gcr_cycle_launches = per_cycle;
    count_launches(before - launches_so_far());  // captured, not launched
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e) return cuda_fail(e, "GCR capture");
    if (e2) return cuda_fail(e2, "end capture");
    e = cudaGraphInstantiate(&h.gcr_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e) return cuda_fail(e, "graph instantiate");
    h.gcr_key = key;
  }
  per_cycle = h.gcr_cycle_launches;

  const int max_launches = (itmax + m - 1) / m + 1;
  int launched = 0;
  bool finished = false;
  for (int c = 0; c < max_launches && !finished; c++) {
    if ((e = cudaGraphLaunch(h.gcr_graph, s))) return cuda_fail(e, "graph launch");
    count_launches(per_cycle);
    if ((e = cudaMemcpyAsync(&h.h_st[c & 1], h.st, sizeof(KState),
                             cudaMemcpyDeviceToHost, s)) ||
        (e = cudaEventRecord(h.ev[c & 1], s)))
      return cuda_fail(e, "state readback");
    launched++;
    if (c > 0) {
      if ((e = cudaEventSynchronize(h.ev[(c - 1) & 1]))) return cuda_fail(e, "sync");
      if (h.h_st[(c - 1) & 1].done) finished = true;
    }
  }
  h.last.graph_launches = launched;
  }
  if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "GCR");
  KState fin;
  if ((e = cudaMemcpy(&fin, h.st, sizeof(KState), cudaMemcpyDeviceToHost)))
    return cuda_fail(e, "final state");
  if (fin.done == 2) {
    if ((e = cudaMemsetAsync(x, 0, sizeof(double) * h.N, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_fail(e, "zero x");
  }
  const int status = fin.done ? fin.status : VDR_NOT_CONVERGED;
  h.last.iterations = fin.iter;
  h.last.status = status;
  h.last.kernel_launches = (int)(launches_so_far() - launches0);
  h.last.breakdown = (status == VDR_BREAKDOWN || fin.reason == 6) ? fin.reason : 0;
  if (iter) *iter = fin.iter;
  if (err) *err = fin.err;
  return status;
}

}  // namespace vdr
