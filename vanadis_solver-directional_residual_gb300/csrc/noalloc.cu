// noalloc.cu -- vdr_bicg_noalloc_device: the Jacobi BiCG solve of
// kernel_dbcg_simple_ for callers that may not allocate device memory.
//
// Who needs it: a host program that hands the solver buffers it already
// owns and must not allocate afterwards -- e.g. a time loop running under a
// memory budget fixed at start-up, or next to a framework's caching
// allocator that has reserved the whole device, where a cudaMalloc fails or
// takes memory another part of the program counts on; or a Fortran driver
// whose every step would otherwise pay the allocation and release the
// reference pays per call.
//
// Scratch: the Krylov work vectors (r, rr, p, pp, z, zz), the per-block
// reduction partials and the solver state live in one file-scope device
// array, g_noalloc_scratch, sized for VDR_NOALLOC_MAX_NODES nodes (about
// 3 MB on every GPU that loads the library, held until the process exits).
// Its device address is taken once per device with cudaGetSymbolAddress on
// the first call on that device and kept for the process (a cudaDeviceReset
// of that device would leave it stale).  Every call shares the array: calls
// that overlap on the GPU (two streams, two host threads) race, and each
// call clears the state it relies on before use.  The call is synchronous:
// it reads the solver state back every few iterations and waits for it.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <mutex>

#include "vdr.h"
#include "vdr_internal.h"

namespace vdr {
namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_MAX_BLOCKS = 512;
constexpr long NA_NVEC = 6;

struct NaState {
  double bnrm2, err, bknum, bkden, ak;
  double tol;
  int iter, itmax, done, status;
  unsigned int ticket;
  int bad;  // set when an ISS entry lies outside 1..n
};

constexpr int NA_MAX_Q = 3;  // most sums reduced by one kernel (na_start)
constexpr long NA_STATE_DOUBLES = (sizeof(NaState) + 7) / 8;
constexpr long NA_PARTIAL_DOUBLES = (long)NA_MAX_Q * NA_MAX_BLOCKS;
constexpr long NA_TOTAL_DOUBLES =
    NA_NVEC * VDR_NOALLOC_MAX_NODES + NA_PARTIAL_DOUBLES + NA_STATE_DOUBLES;

// The scratch.  Host code must not take its address directly (that is a
// host-side stand-in); it uses the pointer from cudaGetSymbolAddress.
static __device__ __align__(256) double g_noalloc_scratch[NA_TOTAL_DOUBLES];

struct NaArgs {
  int n, E;
  const double *b, *diag, *bb;
  const int *iss, *bc;
  double *x, *r, *rr, *p, *pp, *z, *zz;
  double *partials;
  NaState *st;
};

__device__ __forceinline__ int na_node(const NaArgs &a, int s, long e) {
  return __ldg(a.iss + (size_t)s * a.E + e) - 1;
}

// y += P A P x (TRANS: P A^T P x) over the reference's BB layout
// BB[64e + 8i + j]; Dirichlet columns read as 0, rows are not written.
template <bool TRANS>
__global__ void na_apply(NaArgs a, const double *__restrict__ xin,
                         double *__restrict__ y) {
  if (a.st->done) return;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < a.E;
       e += (long)gridDim.x * blockDim.x) {
    int nd[8];
    double xv[8];
    bool m[8];
#pragma unroll
    for (int s = 0; s < 8; s++) {
      nd[s] = na_node(a, s, e);
      if ((unsigned)nd[s] >= (unsigned)a.n) {  // never dereferenced
        a.st->bad = 1;
        nd[s] = 0;
        m[s] = true;
      } else {
        m[s] = a.bc && __ldg(a.bc + nd[s]) == 1;
      }
      xv[s] = m[s] ? 0.0 : xin[nd[s]];
    }
    const double *blk = a.bb + 64 * e;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      double acc = 0.0;
#pragma unroll
      for (int j = 0; j < 8; j++)
        acc += (TRANS ? __ldg(blk + 8 * j + i) : __ldg(blk + 8 * i + j)) * xv[j];
      if (!m[i]) atomicAdd(y + nd[i], acc);
    }
  }
}

template <int NQ>
__device__ __forceinline__ bool na_grid_sum(double (&v)[NQ], const NaArgs &a,
                                            double (&out)[NQ]) {
  static_assert(NQ <= NA_MAX_Q, "partials region holds NA_MAX_Q sums per block");
  __shared__ double sm[NA_THREADS / 32][NQ];
  __shared__ bool last;
#pragma unroll
  for (int q = 0; q < NQ; q++)
    for (int off = 16; off > 0; off >>= 1)
      v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int q = 0; q < NQ; q++) sm[w][q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < NQ; q++) {
      double t = 0.0;
      for (int k = 0; k < NA_THREADS / 32; k++) t += sm[k][q];
      a.partials[q * NA_MAX_BLOCKS + blockIdx.x] = t;
    }
    __threadfence();
    last = atomicAdd(&a.st->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return false;
  __threadfence();
  for (int q = 0; q < NQ; q++) {
    double t = 0.0;
    for (unsigned k = 0; k < gridDim.x; k++)
      t += __ldcg(a.partials + q * NA_MAX_BLOCKS + k);
    out[q] = t;
  }
  a.st->ticket = 0u;
  return true;
}

#define NA_LOOP(i) \
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (long)gridDim.x * blockDim.x)

// r = b - r (r holds A x0); rr = r; norms; bknum = (r/d, rr).
__global__ void na_start(NaArgs a) {
  double v[3] = {0.0, 0.0, 0.0};
  NA_LOOP(i) {
    const double bi = a.b[i];
    const double ri = bi - a.r[i];
    a.r[i] = ri;
    a.rr[i] = ri;
    v[0] += bi * bi;
    v[1] += ri * ri;
    v[2] += (ri / a.diag[i]) * ri;
  }
  double o[3];
  if (na_grid_sum<3>(v, a, o)) {
    NaState *st = a.st;
    if (st->bad) {  // a bad ISS entry: no iteration may touch x
      st->status = VDR_BAD_ARGUMENT;
      st->done = 1;
      return;
    }
    st->bnrm2 = o[0];
    st->bknum = o[2];
    st->bkden = 1.0;
    st->iter = 0;
    st->status = VDR_NOT_CONVERGED;
    st->err = sqrt(o[1]) / sqrt(o[0]);
    st->done = (st->err <= st->tol) ? 1 : 0;
    if (st->done) st->status = VDR_OK;
    if (!(st->err == st->err)) {
      st->status = VDR_BREAKDOWN;
      st->done = 1;
    }
  }
}

// p = r/d + bk p, pp = rr/d + bk pp (zero on Dirichlet nodes); z = zz = 0.
__global__ void na_p(NaArgs a) {
  const NaState *st = a.st;
  if (st->done) return;
  const bool first = st->iter == 0;
  const double bk = first ? 0.0 : st->bknum / st->bkden;
  NA_LOOP(i) {
    const bool m = a.bc && a.bc[i] == 1;
    const double zi = a.r[i] / a.diag[i], zzi = a.rr[i] / a.diag[i];
    a.p[i] = m ? 0.0 : (first ? zi : zi + bk * a.p[i]);
    a.pp[i] = m ? 0.0 : (first ? zzi : zzi + bk * a.pp[i]);
    a.z[i] = 0.0;
    a.zz[i] = 0.0;
  }
}

__global__ void na_ak(NaArgs a) {
  if (a.st->done) return;
  double v[1] = {0.0};
  NA_LOOP(i) v[0] += a.z[i] * a.pp[i];
  double o[1];
  if (na_grid_sum<1>(v, a, o)) {
    a.st->ak = a.st->bknum / o[0];
    if (!isfinite(a.st->ak)) {
      a.st->status = VDR_BREAKDOWN;
      a.st->done = 1;
    }
  }
}

__global__ void na_upd(NaArgs a) {
  if (a.st->done) return;
  const double ak = a.st->ak;
  double v[2] = {0.0, 0.0};
  NA_LOOP(i) {
    a.x[i] += ak * a.p[i];
    const double ri = a.r[i] - ak * a.z[i];
    const double rri = a.rr[i] - ak * a.zz[i];
    a.r[i] = ri;
    a.rr[i] = rri;
    v[0] += ri * ri;
    v[1] += (ri / a.diag[i]) * rri;
  }
  double o[2];
  if (na_grid_sum<2>(v, a, o)) {
    NaState *st = a.st;
    st->iter += 1;
    st->err = sqrt(o[0]) / sqrt(st->bnrm2);
    st->bkden = st->bknum;
    st->bknum = o[1];
    if (!(st->err == st->err)) {
      st->status = VDR_BREAKDOWN;
      st->done = 1;
    } else if (st->err <= st->tol) {
      st->status = VDR_OK;
      st->done = 1;
    } else if (st->iter >= st->itmax) {
      st->done = 1;
    }
  }
}

__global__ void na_mask_x(NaArgs a) {
  NA_LOOP(i) if (a.bc && a.bc[i] == 1) a.x[i] = 0.0;
}

// Device address of the scratch, per device, taken once.
std::mutex g_na_mu;
double *g_na_ptr[64] = {};

int na_scratch(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e) return cuda_fail(e, "vdr_bicg_noalloc_device: cudaGetDevice");
  if (dev < 0 || dev >= 64) {
    set_error("vdr_bicg_noalloc_device: device ordinal above 63");
    return VDR_BAD_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_na_mu);
  if (!g_na_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e) return cuda_fail(e, "vdr_bicg_noalloc_device: cudaGetSymbolAddress");
    g_na_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_na_ptr[dev];
  return VDR_OK;
}

}  // namespace
}  // namespace vdr

using namespace vdr;

extern "C" int vdr_bicg_noalloc_device(int n, int nax, int nay, int naz,
                                       const double *b, double *x, double tol,
                                       int itmax, const double *bb,
                                       const int *iss, const double *diag,
                                       const int *bc, void *stream, int *iter,
                                       double *err) {
  if (n < 1 || n > VDR_NOALLOC_MAX_NODES) {
    set_error("vdr_bicg_noalloc_device: n must be 1..VDR_NOALLOC_MAX_NODES "
              "(65536); use kernel_dbcg_simple_ or vdr_solve for larger meshes");
    return VDR_BAD_ARGUMENT;
  }
  const long E = (long)(nax - 1) * (nay - 1) * (naz - 1);
  if (nax < 2 || nay < 2 || naz < 2 || (long)nax * nay * naz != n ||
      !b || !x || !bb || !iss || !diag || !(tol >= 0.0)) {
    set_error("vdr_bicg_noalloc_device: bad arguments (n must equal NAX*NAY*NAZ)");
    return VDR_BAD_ARGUMENT;
  }
  double *scr = nullptr;
  int st = na_scratch(&scr);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  NaArgs a;
  a.n = n;
  a.E = (int)E;
  a.b = b;
  a.x = x;
  a.bb = bb;
  a.iss = iss;
  a.diag = diag;
  a.bc = bc;
  a.r = scr;
  a.rr = scr + 1L * VDR_NOALLOC_MAX_NODES;
  a.p = scr + 2L * VDR_NOALLOC_MAX_NODES;
  a.pp = scr + 3L * VDR_NOALLOC_MAX_NODES;
  a.z = scr + 4L * VDR_NOALLOC_MAX_NODES;
  a.zz = scr + 5L * VDR_NOALLOC_MAX_NODES;
  a.partials = scr + NA_NVEC * VDR_NOALLOC_MAX_NODES;
  a.st = reinterpret_cast<NaState *>(a.partials + NA_PARTIAL_DOUBLES);

  // The array keeps the previous call's contents: reset the state (ticket,
  // flags, scalars) and the vectors the first kernels accumulate into.
  NaState init{};
  init.tol = tol;
  init.itmax = itmax;
  cudaError_t e = cudaMemcpyAsync(a.st, &init, sizeof(NaState),
                                  cudaMemcpyHostToDevice, s);
  if (!e) e = cudaMemsetAsync(a.r, 0, sizeof(double) * n, s);
  if (e) return cuda_fail(e, "vdr_bicg_noalloc_device: reset");
  const int gv = (int)std::min<long>(NA_MAX_BLOCKS, ((long)n + NA_THREADS - 1) / NA_THREADS);
  const int ge = (int)std::min<long>(4096, (E + NA_THREADS - 1) / NA_THREADS);
  na_mask_x<<<gv, NA_THREADS, 0, s>>>(a);
  na_apply<false><<<ge, NA_THREADS, 0, s>>>(a, a.x, a.r);
  na_start<<<gv, NA_THREADS, 0, s>>>(a);
  if ((e = cudaGetLastError())) return cuda_fail(e, "vdr_bicg_noalloc_device: start");
  NaState h{};
  const int chunk = 8;
  for (int k = 0; k < itmax; k += chunk) {
    for (int c = 0; c < chunk; c++) {
      na_p<<<gv, NA_THREADS, 0, s>>>(a);
      na_apply<false><<<ge, NA_THREADS, 0, s>>>(a, a.p, a.z);
      na_apply<true><<<ge, NA_THREADS, 0, s>>>(a, a.pp, a.zz);
      na_ak<<<gv, NA_THREADS, 0, s>>>(a);
      na_upd<<<gv, NA_THREADS, 0, s>>>(a);
    }
    if ((e = cudaGetLastError())) return cuda_fail(e, "vdr_bicg_noalloc_device: launch");
    e = cudaMemcpyAsync(&h, a.st, sizeof(NaState), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) return cuda_fail(e, "vdr_bicg_noalloc_device: state");
    if (h.bad) break;
    if (h.done) break;
  }
  e = cudaMemcpyAsync(&h, a.st, sizeof(NaState), cudaMemcpyDeviceToHost, s);
  if (!e) e = cudaStreamSynchronize(s);
  if (e) return cuda_fail(e, "vdr_bicg_noalloc_device: state");
  if (h.bad) {
    set_error("vdr_bicg_noalloc_device: ISS entry outside 1..n");
    return VDR_BAD_ARGUMENT;
  }
  if (iter) *iter = h.iter;
  if (err) *err = h.err;
  return h.done ? h.status : VDR_NOT_CONVERGED;
}
