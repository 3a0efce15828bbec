// abi.cu -- the extern "C" surface of libvdr.so (include/vdr.h): handle
// lifetime, host-side mesh preparation (structured-numbering detection,
// element colouring, storage permutation), uploads, and the drop-in
// kernel_dbcg_simple_ entry point of the reference
// (src_v2026_2_1/cudatest.cu:301-602).
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "vdr.h"
#include "vdr_internal.h"

struct vdr_handle {
  vdr::Handle h;
  // host-API staging buffers on the device
  double *io = nullptr;  // [3][N]: x, y / b, scratch
  double *mass_partials = nullptr;
  double *mass_out = nullptr;
};

namespace vdr {

int true_residual_device(Handle &h, const double *b, const double *x, double *rel);

namespace {
thread_local std::string g_err;

template <typename T>
cudaError_t dalloc(T **p, size_t n) {
  if (*p) return cudaSuccess;
  return cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(n, 1));
}
void dfree(void *p) {
  if (p) cudaFree(p);
}

// The reference driver's numbering (w_el): returns true and the node
// counts when iss is exactly the canonical structured connectivity.
bool detect_structured(int N, int E, const int *iss, int *nax, int *nay,
                       int *naz) {
  if (E < 1) return false;
  const long a = (long)iss[3L * E] - iss[0];
  if (a < 2) return false;
  const long ab = (long)iss[4L * E] - iss[0];
  if (ab % a) return false;
  const long b = ab / a;
  if (b < 2 || (long)N % (a * b)) return false;
  const long c = (long)N / (a * b);
  if (c < 2 || (a - 1) * (b - 1) * (c - 1) != (long)E) return false;
  const long ex = a - 1, ey = b - 1;
  const long pl = a * b;
  const long offs[8] = {0, 1, 1 + a, a, pl, 1 + pl, 1 + pl + a, pl + a};
  for (long e = 0; e < E; e++) {
    const long i = e % ex, j = (e / ex) % ey, k = e / (ex * ey);
    const long base = i + a * j + pl * k + 1;
    for (int s = 0; s < 8; s++)
      if ((long)iss[(long)s * E + e] != base + offs[s]) return false;
  }
  *nax = (int)a;
  *nay = (int)b;
  *naz = (int)c;
  return true;
}

// Colours: the reference's parity colouring on its structured numbering
// (cudatest_coloring_gtx1060_optimized.cu:50-74), first-fit greedy in
// element order otherwise (which reproduces the parity colouring on the
// structured numbering).  Host only.
int element_colors(int N, int E, int nax, int nay, const int *iss,
                   std::vector<int> &color) {
  color.assign(E, 0);
  if (nax > 0) {
    const long ex = nax - 1, ey = nay - 1;
    for (long e = 0; e < E; e++) {
      const long i = e % ex, j = (e / ex) % ey, k = e / (ex * ey);
      color[e] = (int)((i & 1) + 2 * (j & 1) + 4 * (k & 1));
    }
    return 8;
  }
  std::vector<uint32_t> used(N, 0u);
  int nc = 0;
  for (long e = 0; e < E; e++) {
    uint32_t m = 0;
    for (int s = 0; s < 8; s++) m |= used[iss[(long)s * E + e] - 1];
    if (m == 0xffffffffu) return -1;
    int c = 0;
    while (m & (1u << c)) c++;
    color[e] = c;
    nc = std::max(nc, c + 1);
    for (int s = 0; s < 8; s++) used[iss[(long)s * E + e] - 1] |= (1u << c);
  }
  return nc;
}

template <typename T>
void permute_cols(const T *src, T *dst, long E, int ncols,
                  const std::vector<int> &perm) {
  for (int c = 0; c < ncols; c++)
    for (long p = 0; p < E; p++) dst[(long)c * E + p] = src[(long)c * E + perm[p]];
}

int check_handle(vdr_handle *H) {
  if (!H) {
    set_error("null handle");
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e = cudaSetDevice(H->h.device);
  if (e) return cuda_fail(e, "cudaSetDevice");
  return VDR_OK;
}

void free_geometry(Handle &h) {
  dfree(h.geo.Ji);
  dfree(h.geo.Dj);
  dfree(h.geo.K);
  h.geo = GeoFactors{};
}

// The mesh's geometric factors for the double-float build, formed at the
// first build that can use them (h.flag allocated).  *use = false where the
// build evaluates the Jacobians itself: VDR_BUILD_RECOMPUTE, no device memory
// for the factors, a factor outside the pair window.
int ensure_geometry(Handle &h, bool *use) {
  *use = false;
  if (h.build_mode == VDR_BUILD_RECOMPUTE || h.geo_state < 0) return VDR_OK;
  if (h.geo_state > 0) {
    *use = true;
    return VDR_OK;
  }
  const size_t E = (size_t)std::max(h.E, 1);
  // only where they leave at least half of the free device memory to the
  // rest of the work
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess ||
      sizeof(float2) * GEO_PAIRS * E > free_b / 2) {
    cudaGetLastError();
    h.geo_state = -1;
    return VDR_OK;
  }
  if (cudaMalloc(&h.geo.Ji, sizeof(float2) * 72 * E) ||
      cudaMalloc(&h.geo.Dj, sizeof(float2) * 8 * E) ||
      cudaMalloc(&h.geo.K, sizeof(float2) * 36 * E)) {
    cudaGetLastError();  // no room for them: not an error
    free_geometry(h);
    h.geo_state = -1;
    return VDR_OK;
  }
  cudaError_t e;
  int bad = 0;
  if ((e = cudaMemsetAsync(h.flag, 0, sizeof(int), h.stream)) ||
      (e = launch_geo_factors(op_args(h), h.geo, h.flag, h.stream)) ||
      (e = cudaMemcpyAsync(&bad, h.flag, sizeof(int), cudaMemcpyDeviceToHost,
                           h.stream)) ||
      (e = cudaStreamSynchronize(h.stream)))
    return cuda_fail(e, "geometric factors");
  if (bad) {
    free_geometry(h);
    h.geo_state = -1;
    return VDR_OK;
  }
  h.geo_state = 1;
  *use = true;
  return VDR_OK;
}

// Builds the stored element matrices and the Jacobi diagonal if they are
// stale; when `rhs` is given, the right-hand side is assembled in the same
// element pass (or alone, if the operator is already valid).
int build_operator(Handle &h, const BuildArgs *rhs) {
  if (!h.fields_set) {
    set_error("fields not set (vdr_set_fields)");
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e;
  const bool need_op = !(h.op64_valid && h.diag_valid);
  if (!need_op && !rhs) return VDR_OK;
  const bool stored = h.apply_mode == VDR_APPLY_STORED;
  if ((e = dalloc(&h.flag, 1))) return cuda_fail(e, "alloc flag");
  if (need_op && ((e = dalloc(&h.diag, h.N)) || (e = dalloc(&h.dinv, h.N))))
    return cuda_fail(e, "alloc diag");
  // The H/M rows are accumulated in double-float unless a value left the
  // pairs' safe window (flag bit 2: redo with FP64 rows), and the store is
  // double-float unless an entry left the store window (bit 1: FP64 store).
  for (int attempt = 0; attempt < 3; attempt++) {
    const bool df = stored && h.storage == VDR_STORE_DF;
    BuildArgs ba;
    ba.exact_fp64 = h.exact_build;
    ba.bad = h.flag;
    if (rhs) {
      ba.cf = rhs->cf;
      ba.rM = rhs->rM;
      ba.told = rhs->told;
      ba.b = rhs->b;
      if ((e = cudaMemsetAsync(ba.b, 0, sizeof(double) * h.N, h.stream)))
        return cuda_fail(e, "memset rhs");
      // time loop: keep M and F of this operator (double-float build only)
      if (rhs->Mhi && !h.exact_build) {
        ba.Mhi = rhs->Mhi;
        ba.Mlo = rhs->Mlo;
        ba.f = rhs->f;
        if ((e = cudaMemsetAsync(ba.f, 0, sizeof(double) * h.N, h.stream)))
          return cuda_fail(e, "memset f");
      }
    }
    if (need_op) {
      if (stored && !df && (e = dalloc(&h.A64, (size_t)h.E * 32)))
        return cuda_fail(e, "alloc element matrices");
      if (df && ((e = dalloc(&h.Ahi, (size_t)h.E * 16)) ||
                 (e = dalloc(&h.Alo, (size_t)h.E * 16))))
        return cuda_fail(e, "alloc element matrices");
      if ((e = cudaMemsetAsync(h.diag, 0, sizeof(double) * h.N, h.stream)))
        return cuda_fail(e, "memset diag");
      ba.aH = h.aH;
      ba.aM = h.aM;
      ba.A64 = (stored && !df) ? h.A64 : nullptr;
      ba.Ahi = df ? h.Ahi : nullptr;
      ba.Alo = df ? h.Alo : nullptr;
      ba.diag = h.diag;
      if (h.want_phi) {
        if ((e = dalloc(&h.phi, (size_t)h.E * 8))) return cuda_fail(e, "alloc phi");
        ba.phi = h.phi;
      }
    }
    // from the mesh's geometric factors unless the rows are FP64 or a
    // Robin term is on; each double-float build has its per-element scalars
    if (!h.exact_build) {
      bool geo = false;
      if (!(h.robin && h.robin_alpha != 0.0)) {
        const int gst = ensure_geometry(h, &geo);
        if (gst) return gst;
      }
      if (geo) {
        if ((e = dalloc(&h.gsc, (size_t)h.E * 10)))
          return cuda_fail(e, "alloc element scalars");
        ba.gJi = h.geo.Ji;
        ba.gDj = h.geo.Dj;
        ba.gK = h.geo.K;
        ba.gsc = h.gsc;
      } else {
        if ((e = dalloc(&h.drs, (size_t)h.E * 5))) return cuda_fail(e, "alloc DR scalars");
        ba.drs = h.drs;
      }
    }
    if ((e = cudaMemsetAsync(h.flag, 0, sizeof(int), h.stream)))
      return cuda_fail(e, "memset flag");
    if ((e = launch_build(op_args(h), ba, false, h.stream)))
      return cuda_fail(e, "element matrices");
    int bad = 0;
    if ((e = cudaMemcpyAsync(&bad, h.flag, sizeof(int), cudaMemcpyDeviceToHost,
                             h.stream)) ||
        (e = cudaStreamSynchronize(h.stream)))
      return cuda_fail(e, "flag");
    // bit 3: the M store left its window (M is then not kept)
    h.mass_valid = ba.Mhi && !(bad & 4) && !(bad & 3);
    if (!(bad & 3)) break;
    if (bad & 2) h.exact_build = true;
    if ((bad & 1) && df) h.storage = VDR_STORE_FP64;
  }
  if (need_op) {
    if ((e = launch_diag_fix(h.diag, h.dinv, h.mask, h.N, h.stream)) ||
        (e = launch_emask(h)))
      return cuda_fail(e, "diag");
    h.op64_valid = true;
    h.diag_valid = true;
    h.phi_valid = h.want_phi;
    if (stored) {  // the apply's launch shape, once per handle
      const int st = tune_stored_apply(h);
      if (st) return st;
    }
  }
  return VDR_OK;
}

int ensure_operator(Handle &h) { return build_operator(h, nullptr); }

// FP32 element matrices from the FP32 DR recompute (Jacobians and DR terms
// evaluated in FP32), for the inner solves of the mixed-precision path.
int ensure_operator32(Handle &h) {
  if (h.op32_valid) return VDR_OK;
  if (h.apply_mode != VDR_APPLY_STORED) {
    h.op32_valid = true;  // matrix-free: recomputed in FP32 at each apply
    return VDR_OK;
  }
  h.use_half = false;
  if (h.mixed_op == VDR_MIXED_HALF) {
    // the binary16 Jacobi-scaled store for the FP32-vector inner solves;
    // the rounded FP32 operator stays the one of FP64-vector inner solves
    int st = ensure_operator(h);
    if (st) return st;
    cudaError_t e;
    if (!h.flag && (e = cudaMalloc(&h.flag, sizeof(int))))
      return cuda_fail(e, "flag");
    int bad = 0;
    if ((e = cudaMemsetAsync(h.flag, 0, sizeof(int), h.stream)) ||
        (e = launch_half_store(h, h.flag, h.stream)) ||
        (e = cudaMemcpyAsync(&bad, h.flag, sizeof(int), cudaMemcpyDeviceToHost,
                             h.stream)) ||
        (e = cudaStreamSynchronize(h.stream)))
      return cuda_fail(e, "16-bit element matrices");
    h.use_half = bad == 0;  // out of range: the rounded FP32 operator
    if (h.use_half) {
      const int st = tune_half_apply(h);
      if (st) return st;
    }
  }
  if (h.mixed_op == VDR_MIXED_ROUNDED || h.mixed_op == VDR_MIXED_HALF) {
    // the hi parts of the double-float store are the FP64 element matrices
    // rounded to FP32, in the FP32 store's layout: no second build
    int st = ensure_operator(h);
    if (st) return st;
    if (h.storage == VDR_STORE_DF && h.Ahi) {
      h.A32v = h.Ahi;
      h.op32_valid = true;
      return VDR_OK;
    }
  }
  cudaError_t e;
  if ((e = dalloc(&h.A32, (size_t)h.E * 16))) return cuda_fail(e, "alloc FP32 matrices");
  BuildArgs ba;
  ba.aH = h.aH;
  ba.aM = h.aM;
  ba.A32 = h.A32;
  if ((e = launch_build(op_args(h), ba, true, h.stream)))
    return cuda_fail(e, "FP32 element matrices");
  h.A32v = h.A32;
  h.op32_valid = true;
  return VDR_OK;
}

// The solve of vdr_solve, vdr_solve_device and vdr_time_steps: FP64
// Krylov, or (VDR_PRECISION_MIXED) FP64 refinement around FP32-operator
// inner solves to the same FP64 tolerance; *iter counts inner iterations.
int solve_by_option(Handle &h, int method, const double *b, double *x,
                    double tol, int itmax, int *iter, double *err) {
  if (h.opt.precision != VDR_PRECISION_MIXED)
    return solve_device(h, method, b, x, tol, itmax, iter, err);
  int st = ensure_operator32(h);
  if (st) return st;
  // each correction to 1e-5, or to 1e-3 with the binary16 operator, whose
  // rounding (2^-11 per element) a tighter inner solve cannot get past
  MixedStats ms;
  st = solve_mixed_device(h, method, b, x, tol, h.use_half ? 1e-3 : 1e-5, 20,
                          itmax, &ms);
  if (iter) *iter = ms.inner;
  if (err) *err = ms.err;
  return st;
}

void invalidate(Handle &h) {
  h.op64_valid = h.op32_valid = h.diag_valid = false;
  h.mass_valid = false;
  h.aos_valid = h.phi_valid = false;
}

// d64[c][p] = src[c][perm[p]] (perm null: identity), d32 the FP32 copy.
__global__ void fields_convert_kernel(const double *__restrict__ src, int ncols, long E,
                                      const int *__restrict__ perm, double *d64,
                                      float *d32) {
  const long total = (long)ncols * E;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long c = t / E, p = t - c * E;
    const double v = src[c * E + (perm ? perm[p] : p)];
    d64[t] = v;
    if (d32) d32[t] = (float)v;
  }
}

cudaError_t launch_fields_convert(const double *src, int ncols, long E, const int *perm,
                                  double *d64, float *d32, cudaStream_t s) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long need = ((long)ncols * E + 255) / 256;
  const int grid = (int)std::max<long>(1, std::min<long>(need, (long)sms * 8));
  fields_convert_kernel<<<grid, 256, 0, s>>>(src, ncols, E, perm, d64, d32);
  count_launches(1);
  return cudaGetLastError();
}

int upload(void *dst, const void *src, size_t bytes, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  if (e) return cuda_fail(e, "upload");
  return VDR_OK;
}

void free_handle(Handle &h) {
  dfree(h.xx); dfree(h.yy); dfree(h.zz);
  dfree(h.xx32); dfree(h.yy32); dfree(h.zz32);
  dfree(h.conn); dfree(h.mask); dfree(h.emask);
  dfree(h.vel); dfree(h.lam); dfree(h.pdec); dfree(h.q);
  dfree(h.vel32); dfree(h.lam32); dfree(h.pdec32); dfree(h.robin);
  dfree(h.A64); dfree(h.A32); dfree(h.diag); dfree(h.dinv);
  dfree(h.Ahi); dfree(h.Alo); dfree(h.flag); dfree(h.A16); dfree(h.e16);
  dfree(h.Aaos); dfree(h.phi); dfree(h.perm_d); dfree(h.dinv32); dfree(h.block_err);
  dfree(h.bk_f); dfree(h.bk_d);
  if (h.bk_graph) cudaGraphExecDestroy(h.bk_graph);
  dfree(h.gcr_work); dfree(h.stage_d); dfree(h.drs); dfree(h.work32);
  dfree(h.Mhi); dfree(h.Mlo); dfree(h.Fvec); dfree(h.rhs_tmp); dfree(h.massw);
  free_geometry(h);
  dfree(h.gsc);
  if (h.graph32) cudaGraphExecDestroy(h.graph32);
  if (h.gcr_graph) cudaGraphExecDestroy(h.gcr_graph);
  dfree(h.seg_d); dfree(h.seg_i); dfree(h.seg_ticket); dfree(h.seg_of_elem);
  if (h.seg_graph) cudaGraphExecDestroy(h.seg_graph);
  dfree(h.work); dfree(h.st); dfree(h.partials);
  if (h.h_st) cudaFreeHost(h.h_st);
  for (int k = 0; k < Handle::NGRAPH; k++)
    if (h.graph_exec[k]) cudaGraphExecDestroy(h.graph_exec[k]);
  for (int k = 0; k < 2; k++)
    if (h.ev[k]) cudaEventDestroy(h.ev[k]);
  if (h.stream) cudaStreamDestroy(h.stream);
  h = Handle();
}

}  // namespace

int prepare_operator(Handle &h) { return ensure_operator(h); }
Handle &handle_of(vdr_handle *H) { return H->h; }

void set_error(const std::string &msg) { g_err = msg; }

namespace {
std::atomic<long long> g_launches{0};
}
void count_launches(long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

int device_sm_count() {
  static std::atomic<int> cached{0};
  int n = cached.load(std::memory_order_relaxed);
  if (n > 0) return n;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  if (n <= 0) n = 1;
  cached.store(n, std::memory_order_relaxed);
  return n;
}

int cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return VDR_CUDA_ERROR;
}

OpArgs op_args(const Handle &h) {
  OpArgs a;
  a.E = h.E;
  a.N = h.N;
  a.variant = h.opt.dr_variant;
  a.conn = h.conn;
  a.xx = h.xx;
  a.yy = h.yy;
  a.zz = h.zz;
  a.xx32 = h.xx32;
  a.yy32 = h.yy32;
  a.zz32 = h.zz32;
  a.f.vel = h.vel;
  a.f.lam = h.lam;
  a.f.pdec = h.pdec;
  a.f.q = h.q;
  a.f.robin = h.robin;
  a.f.robin_alpha = h.robin_alpha;
  a.vel32 = h.vel32;
  a.lam32 = h.lam32;
  a.pdec32 = h.pdec32;
  a.aH = h.aH;
  a.aM = h.aM;
  return a;
}

}  // namespace vdr

using namespace vdr;

extern "C" {

const char *vdr_last_error(void) { return g_err.c_str(); }

int vdr_default_options(vdr_options *o) {
  if (!o) return VDR_BAD_ARGUMENT;
  std::memset(o, 0, sizeof(*o));
  o->dr_variant = VDR_DR_VF;
  o->scatter = VDR_SCATTER_AUTO;
  o->apply_mode = VDR_APPLY_AUTO;
  o->solver = VDR_SOLVER_BICGSTAB;
  o->iters_per_graph = 8;
  o->device = 0;
  return VDR_OK;
}

int vdr_create(vdr_handle **out, int nnode, int nelem, const double *xx,
               const double *yy, const double *zz, const int *iss,
               const int *kod, const vdr_options *opt) {
  if (!out || !xx || !yy || !zz || !iss || nnode < 8 || nelem < 1) {
    set_error("vdr_create: null pointer or empty mesh");
    return VDR_BAD_ARGUMENT;
  }
  *out = nullptr;
  const long E = nelem;
  for (long t = 0; t < 8 * E; t++) {
    if (iss[t] < 1 || iss[t] > nnode) {
      char buf[128];
      std::snprintf(buf, sizeof buf,
                    "vdr_create: iss entry %ld = %d outside 1..%d", t, iss[t], nnode);
      set_error(buf);
      return VDR_BAD_ARGUMENT;
    }
  }
  vdr_options o;
  if (opt) o = *opt; else vdr_default_options(&o);
  if (o.dr_variant < VDR_DR_OT || o.dr_variant > VDR_DR_VF) {
    set_error("vdr_create: unknown dr_variant");
    return VDR_BAD_ARGUMENT;
  }
  if (o.precision != VDR_PRECISION_FP64 && o.precision != VDR_PRECISION_MIXED) {
    set_error("vdr_create: unknown precision");
    return VDR_BAD_ARGUMENT;
  }
  vdr_handle *H = new vdr_handle();
  Handle &h = H->h;
  h.N = nnode;
  h.E = nelem;
  h.opt = o;
  h.device = o.device;
  h.scatter = (o.scatter == VDR_SCATTER_COLOR) ? VDR_SCATTER_COLOR : VDR_SCATTER_ATOMIC;
  h.warp_agg = o.scatter == VDR_SCATTER_WARP;
  h.apply_mode = (o.apply_mode == VDR_APPLY_MATRIX_FREE) ? VDR_APPLY_MATRIX_FREE
                                                         : VDR_APPLY_STORED;
  h.storage = (o.matrix_storage == VDR_STORE_FP64) ? VDR_STORE_FP64 : VDR_STORE_DF;
  cudaError_t e;
  int st = VDR_OK;
  if ((e = cudaSetDevice(h.device)) ||
      (e = cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking))) {
    st = cuda_fail(e, "vdr_create: device/stream");
    delete H;
    return st;
  }
  detect_structured(nnode, nelem, iss, &h.nax, &h.nay, &h.naz);

  // storage order
  h.perm.resize(E);
  std::iota(h.perm.begin(), h.perm.end(), 0);
  h.color_off.assign(2, 0);
  h.color_off[1] = nelem;
  h.ncolors = 1;
  if (h.scatter == VDR_SCATTER_COLOR) {
    std::vector<int> color;
    const int nc = element_colors(h.N, h.E, h.nax, h.nay, iss, color);
    if (nc < 1) {
      set_error("vdr_create: colouring needs more than 32 colours");
      free_handle(h);
      delete H;
      return VDR_BAD_ARGUMENT;
    }
    h.ncolors = nc;
    h.color_off.assign(nc + 1, 0);
    for (long e2 = 0; e2 < E; e2++) h.color_off[color[e2] + 1]++;
    for (int c = 0; c < nc; c++) h.color_off[c + 1] += h.color_off[c];
    std::vector<int> cursor(h.color_off.begin(), h.color_off.end() - 1);
    for (long e2 = 0; e2 < E; e2++) h.perm[cursor[color[e2]]++] = (int)e2;
  }

  std::vector<int> conn(8 * E);
  for (int s = 0; s < 8; s++)
    for (long p = 0; p < E; p++) conn[s * E + p] = iss[s * E + h.perm[p]] - 1;
  std::vector<float> c32(nnode);
  std::vector<unsigned char> robin(E, 0);
  bool any_robin = false;
  if (kod)
    for (long p = 0; p < E; p++) {
      robin[p] = kod[2 * E + h.perm[p]] == 3;
      any_robin |= robin[p] != 0;
    }
  do {
    if ((e = dalloc(&h.xx, nnode)) || (e = dalloc(&h.yy, nnode)) ||
        (e = dalloc(&h.zz, nnode)) || (e = dalloc(&h.xx32, nnode)) ||
        (e = dalloc(&h.yy32, nnode)) || (e = dalloc(&h.zz32, nnode)) ||
        (e = dalloc(&h.conn, 8 * E)) || (e = dalloc(&h.mask, nnode))) {
      st = cuda_fail(e, "vdr_create: alloc");
      break;
    }
    if ((st = upload(h.xx, xx, sizeof(double) * nnode, h.stream)) ||
        (st = upload(h.yy, yy, sizeof(double) * nnode, h.stream)) ||
        (st = upload(h.zz, zz, sizeof(double) * nnode, h.stream)) ||
        (st = upload(h.conn, conn.data(), sizeof(int) * 8 * E, h.stream)))
      break;
    const double *src[3] = {xx, yy, zz};
    float *dst[3] = {h.xx32, h.yy32, h.zz32};
    for (int k = 0; k < 3 && !st; k++) {
      for (long i = 0; i < nnode; i++) c32[i] = (float)src[k][i];
      st = upload(dst[k], c32.data(), sizeof(float) * nnode, h.stream);
      if (!st && (e = cudaStreamSynchronize(h.stream))) st = cuda_fail(e, "sync");
    }
    if (st) break;
    if ((e = cudaMemsetAsync(h.mask, 0, nnode, h.stream))) {
      st = cuda_fail(e, "memset");
      break;
    }
    if (h.scatter == VDR_SCATTER_COLOR) {
      if ((e = dalloc(&h.perm_d, E))) {
        st = cuda_fail(e, "alloc");
        break;
      }
      if ((st = upload(h.perm_d, h.perm.data(), sizeof(int) * E, h.stream))) break;
    }
    if (any_robin) {
      if ((e = dalloc(&h.robin, E))) {
        st = cuda_fail(e, "alloc");
        break;
      }
      if ((st = upload(h.robin, robin.data(), E, h.stream))) break;
    }
    if ((e = cudaStreamSynchronize(h.stream))) st = cuda_fail(e, "vdr_create");
  } while (0);
  if (st) {
    free_handle(h);
    delete H;
    return st;
  }
  *out = H;
  return VDR_OK;
}

int vdr_set_fields(vdr_handle *H, const double *vel, const double *lam,
                   const double *pdec, const double *q, double robin_alpha) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!vel || !lam) {
    set_error("vdr_set_fields: vel and lam are required");
    return VDR_BAD_ARGUMENT;
  }
  const long E = h.E;
  cudaError_t e;
  if ((e = dalloc(&h.vel, 3 * E)) || (e = dalloc(&h.lam, E)) ||
      (e = dalloc(&h.pdec, E)) || (e = dalloc(&h.q, E)) ||
      (e = dalloc(&h.vel32, 3 * E)) || (e = dalloc(&h.lam32, E)) ||
      (e = dalloc(&h.pdec32, E)))
    return cuda_fail(e, "vdr_set_fields: alloc");
  // Each field goes straight from the caller's array into a device staging
  // buffer (a DMA when the caller's memory is pinned); a kernel puts it into
  // storage order and writes the FP32 copy.  One synchronisation at the end
  // (the caller may reuse its arrays after the call).
  if ((e = dalloc(&h.stage_d, 3 * E))) return cuda_fail(e, "vdr_set_fields: alloc");
  auto put = [&](const double *src, int ncols, double *d64, float *d32) -> int {
    cudaError_t e2;
    if (src)
      e2 = cudaMemcpyAsync(h.stage_d, src, sizeof(double) * ncols * E,
                           cudaMemcpyHostToDevice, h.stream);
    else
      e2 = cudaMemsetAsync(h.stage_d, 0, sizeof(double) * ncols * E, h.stream);
    if (!e2) e2 = launch_fields_convert(h.stage_d, ncols, E, h.perm_d, d64, d32, h.stream);
    return e2 ? cuda_fail(e2, "vdr_set_fields") : VDR_OK;
  };
  if ((st = put(vel, 3, h.vel, h.vel32)) || (st = put(lam, 1, h.lam, h.lam32)) ||
      (st = put(pdec, 1, h.pdec, h.pdec32)) || (st = put(q, 1, h.q, nullptr)))
    return st;
  if ((e = cudaStreamSynchronize(h.stream))) return cuda_fail(e, "vdr_set_fields");
  h.robin_alpha = robin_alpha;
  h.fields_set = true;
  invalidate(h);
  return VDR_OK;
}

int vdr_set_dirichlet(vdr_handle *H, const int *bc) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  cudaError_t e;
  std::vector<unsigned char> m(h.N, 0);
  if (bc)
    for (long i = 0; i < h.N; i++) m[i] = bc[i] == 1;
  if ((st = upload(h.mask, m.data(), h.N, h.stream))) return st;
  if ((e = launch_mask_conn(h.conn, h.E, h.mask, h.stream)))
    return cuda_fail(e, "mask");
  if ((e = cudaStreamSynchronize(h.stream))) return cuda_fail(e, "mask");
  h.mask_set = true;
  invalidate(h);
  return VDR_OK;
}

int vdr_set_operator(vdr_handle *H, double aH, double aM) {
  int st = check_handle(H);
  if (st) return st;
  H->h.aH = aH;
  H->h.aM = aM;
  invalidate(H->h);
  return VDR_OK;
}

static int ensure_io(vdr_handle *H) {
  cudaError_t e = dalloc(&H->io, 3 * (size_t)H->h.N);
  return e ? cuda_fail(e, "alloc io") : VDR_OK;
}

int vdr_apply_device(vdr_handle *H, const double *x, double *y, int transpose) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!x || !y) {
    set_error("vdr_apply_device: null vector");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h))) return st;
  cudaError_t e;
  if ((e = cudaMemsetAsync(y, 0, sizeof(double) * h.N, h.stream)))
    return cuda_fail(e, "memset");
  if ((e = launch_apply(h, transpose != 0, x, y, nullptr, nullptr, h.stream)))
    return cuda_fail(e, "apply");
  return VDR_OK;
}

int vdr_apply_accumulate_device(vdr_handle *H, const double *x, double *y,
                                int transpose) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!x || !y) {
    set_error("vdr_apply_accumulate_device: null vector");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h))) return st;
  cudaError_t e = launch_apply(h, transpose != 0, x, y, nullptr, nullptr, h.stream);
  return e ? cuda_fail(e, "apply") : VDR_OK;
}

int vdr_apply32_device(vdr_handle *H, const double *x, double *y,
                       int transpose) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!x || !y) {
    set_error("vdr_apply32_device: null vector");
    return VDR_BAD_ARGUMENT;
  }
  if (!h.fields_set) {
    set_error("fields not set (vdr_set_fields)");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator32(h))) return st;
  cudaError_t e = cudaMemsetAsync(y, 0, sizeof(double) * h.N, h.stream);
  if (e) return cuda_fail(e, "memset");
  h.apply_fp32 = true;
  e = launch_apply(h, transpose != 0, x, y, nullptr, nullptr, h.stream);
  h.apply_fp32 = false;
  return e ? cuda_fail(e, "apply32") : VDR_OK;
}

int vdr_apply(vdr_handle *H, const double *x, double *y, int transpose) {
  int st = check_handle(H);
  if (st) return st;
  if ((st = ensure_io(H))) return st;
  Handle &h = H->h;
  double *dx = H->io, *dy = H->io + h.N;
  if ((st = upload(dx, x, sizeof(double) * h.N, h.stream))) return st;
  if ((st = vdr_apply_device(H, dx, dy, transpose))) return st;
  cudaError_t e = cudaMemcpyAsync(y, dy, sizeof(double) * h.N,
                                  cudaMemcpyDeviceToHost, h.stream);
  if (!e) e = cudaStreamSynchronize(h.stream);
  return e ? cuda_fail(e, "vdr_apply") : VDR_OK;
}

int vdr_assemble_rhs_device(vdr_handle *H, double cf, double rM,
                            const double *t_old, double *b) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!b) {
    set_error("vdr_assemble_rhs_device: null b");
    return VDR_BAD_ARGUMENT;
  }
  BuildArgs rhs;
  rhs.cf = cf;
  rhs.rM = rM;
  rhs.told = t_old;
  rhs.b = b;
  return build_operator(h, &rhs);
}

int vdr_assemble_rhs(vdr_handle *H, double cf, double rM, const double *t_old,
                     double *b) {
  int st = check_handle(H);
  if (st) return st;
  if ((st = ensure_io(H))) return st;
  Handle &h = H->h;
  double *dt = nullptr, *db = H->io + h.N;
  if (t_old) {
    dt = H->io;
    if ((st = upload(dt, t_old, sizeof(double) * h.N, h.stream))) return st;
  }
  if ((st = vdr_assemble_rhs_device(H, cf, rM, dt, db))) return st;
  cudaError_t e = cudaMemcpyAsync(b, db, sizeof(double) * h.N,
                                  cudaMemcpyDeviceToHost, h.stream);
  if (!e) e = cudaStreamSynchronize(h.stream);
  return e ? cuda_fail(e, "vdr_assemble_rhs") : VDR_OK;
}

int vdr_get_diag(vdr_handle *H, double *diag) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if ((st = ensure_operator(h))) return st;
  cudaError_t e = cudaMemcpyAsync(diag, h.diag, sizeof(double) * h.N,
                                  cudaMemcpyDeviceToHost, h.stream);
  if (!e) e = cudaStreamSynchronize(h.stream);
  return e ? cuda_fail(e, "vdr_get_diag") : VDR_OK;
}

int vdr_get_element_matrices_device(vdr_handle *H, double *bb) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!bb) {
    set_error("vdr_get_element_matrices_device: null bb");
    return VDR_BAD_ARGUMENT;
  }
  if (h.apply_mode != VDR_APPLY_STORED) {
    set_error("vdr_get_element_matrices: the matrix-free operator stores no matrices");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h))) return st;
  cudaError_t e = launch_export_bb(h, bb, h.stream);
  if (!e) e = cudaStreamSynchronize(h.stream);
  return e ? cuda_fail(e, "vdr_get_element_matrices_device") : VDR_OK;
}

int vdr_get_element_matrices(vdr_handle *H, double *bb) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!bb) {
    set_error("vdr_get_element_matrices: null bb");
    return VDR_BAD_ARGUMENT;
  }
  double *d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * 64 * (size_t)std::max(h.E, 1));
  if (e) return cuda_fail(e, "vdr_get_element_matrices: alloc");
  st = vdr_get_element_matrices_device(H, d);
  if (!st) {
    e = cudaMemcpy(bb, d, sizeof(double) * 64 * (size_t)h.E, cudaMemcpyDeviceToHost);
    if (e) st = cuda_fail(e, "vdr_get_element_matrices: download");
  }
  cudaFree(d);
  return st;
}

int vdr_solve_device(vdr_handle *H, const double *b, double *x, double tol,
                     int itmax, int *iter, double *err) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!b || !x || !(tol >= 0.0)) {
    set_error("vdr_solve_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h))) return st;
  if ((st = ensure_io(H))) return st;
  // Homogeneous Dirichlet rows of b are imposed (b = 0 there), as przest3d
  // does before the solve (vanadis_full_DR_OpenMP_timing.for:766-772).
  double *bm = H->io + 2 * (size_t)h.N;
  cudaError_t e = cudaMemcpyAsync(bm, b, sizeof(double) * h.N,
                                  cudaMemcpyDeviceToDevice, h.stream);
  if (!e) e = launch_mask_vec(bm, h.mask, h.N, h.stream);
  if (e) return cuda_fail(e, "rhs copy");
  const int method = h.opt.solver == VDR_SOLVER_BICG ? VDR_SOLVER_BICG
                                                     : VDR_SOLVER_BICGSTAB;
  return solve_by_option(h, method, bm, x, tol, itmax, iter, err);
}

int vdr_solve_mixed_device(vdr_handle *H, const double *b, double *x,
                           double tol, double inner_tol, int max_outer,
                           int inner_itmax, int *outer_iters, int *inner_iters,
                           double *err) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!b || !x || !(tol >= 0.0) || !(inner_tol > 0.0) || max_outer < 0) {
    set_error("vdr_solve_mixed_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h)) || (st = ensure_operator32(h))) return st;
  if ((st = ensure_io(H))) return st;
  double *bm = H->io + 2 * (size_t)h.N;
  cudaError_t e = cudaMemcpyAsync(bm, b, sizeof(double) * h.N,
                                  cudaMemcpyDeviceToDevice, h.stream);
  if (!e) e = launch_mask_vec(bm, h.mask, h.N, h.stream);
  if (e) return cuda_fail(e, "rhs copy");
  const int method = h.opt.solver == VDR_SOLVER_BICG ? VDR_SOLVER_BICG
                                                     : VDR_SOLVER_BICGSTAB;
  MixedStats ms;
  st = solve_mixed_device(h, method, bm, x, tol, inner_tol, max_outer,
                          inner_itmax, &ms);
  if (outer_iters) *outer_iters = ms.outer;
  if (inner_iters) *inner_iters = ms.inner;
  if (err) *err = ms.err;
  return st;
}

int vdr_apply_half_device(vdr_handle *H, const float *x, float *y) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!x || !y) {
    set_error("vdr_apply_half_device: null vector");
    return VDR_BAD_ARGUMENT;
  }
  if (h.apply_mode != VDR_APPLY_STORED || h.mixed_op != VDR_MIXED_HALF) {
    set_error("vdr_apply_half_device: needs the stored operator and "
              "vdr_set_mixed_operator(h, VDR_MIXED_HALF)");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h)) || (st = ensure_operator32(h))) return st;
  if (!h.use_half) {
    set_error("vdr_apply_half_device: an element scale is outside the "
              "binary16 store's range");
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e = cudaMemsetAsync(y, 0, sizeof(float) * h.N, h.stream);
  if (!e) e = launch_apply_half(h, x, y, nullptr, nullptr, h.stream);
  return e ? cuda_fail(e, "apply half") : VDR_OK;
}

int vdr_assemble_rhs_block_device(vdr_handle *H, int K, const double *Q,
                                  double cf, double *B) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (K < 1 || K > VDR_MAX_BLOCK_RHS || !Q || !B) {
    set_error("vdr_assemble_rhs_block_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  if (!h.phi_valid) {
    h.want_phi = true;
    h.op64_valid = false;
  }
  if ((st = ensure_operator(h))) return st;
  cudaError_t e = cudaMemsetAsync(B, 0, sizeof(double) * h.N * (size_t)K, h.stream);
  if (!e) e = launch_block_rhs(h, h.phi, K, Q, cf, B, h.stream);
  return e ? cuda_fail(e, "block rhs") : VDR_OK;
}

static int apply_block(vdr_handle *H, int K, const void *X, void *Y,
                       int precision, bool zero, const char *who) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (K < 1 || K > VDR_MAX_BLOCK_RHS || !X || !Y ||
      (precision != VDR_BLOCK_FP64 && precision != VDR_BLOCK_TF32 &&
       precision != VDR_BLOCK_TF32X3) ||
      (precision != VDR_BLOCK_FP64 && K != 16 && K != 32 && K != 64) ||
      h.apply_mode != VDR_APPLY_STORED) {
    set_error(std::string(who) + ": bad arguments (TF32 needs K = 16, 32 "
              "or 64; block applies need the stored operator)");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h))) return st;
  cudaError_t e;
  if (precision != VDR_BLOCK_FP64) {
    float4 *Aaos = nullptr;
    if ((e = ensure_aos(h, false, &Aaos))) return cuda_fail(e, "block operator copy");
    if (zero && (e = cudaMemsetAsync(Y, 0, sizeof(float) * h.N * (size_t)K, h.stream)))
      return cuda_fail(e, "memset");
    if (block_apply_launches_tf32(h, K, precision == VDR_BLOCK_TF32X3,
                                  static_cast<const float *>(X), nullptr,
                                  static_cast<float *>(Y), Aaos, nullptr,
                                  h.stream))
      return cuda_fail(cudaGetLastError(), "block apply");
    if (!h.block_tma) return VDR_OK;
    // the bulk-copy variant reports a device wait that ran out
    int tma_err = 0;
    if ((e = cudaMemcpyAsync(&tma_err, h.block_err, sizeof(int), cudaMemcpyDeviceToHost,
                             h.stream)) ||
        (e = cudaStreamSynchronize(h.stream)))
      return cuda_fail(e, "block apply");
    if (tma_err) {
      cudaMemset(h.block_err, 0, sizeof(int));
      set_error("block apply: a bulk-copy wait ran out of time");
      return VDR_TIMEOUT;
    }
    return VDR_OK;
  }
  if ((zero && (e = cudaMemsetAsync(Y, 0, sizeof(double) * h.N * (size_t)K, h.stream))) ||
      (e = launch_block_apply64(h, K, static_cast<const double *>(X),
                                static_cast<double *>(Y), h.stream)))
    return cuda_fail(e, "block apply");
  return VDR_OK;
}

int vdr_apply_block_device(vdr_handle *H, int K, const void *X, void *Y,
                           int precision) {
  return apply_block(H, K, X, Y, precision, true, "vdr_apply_block_device");
}

int vdr_apply_block_accumulate_device(vdr_handle *H, int K, const void *X,
                                      void *Y, int precision) {
  return apply_block(H, K, X, Y, precision, false,
                     "vdr_apply_block_accumulate_device");
}

int vdr_set_build_mode(vdr_handle *H, int mode) {
  int st = check_handle(H);
  if (st) return st;
  if (mode != VDR_BUILD_AUTO && mode != VDR_BUILD_RECOMPUTE) {
    set_error("vdr_set_build_mode: unknown mode");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = H->h;
  if (h.build_mode != mode) {
    h.build_mode = mode;
    if (mode == VDR_BUILD_RECOMPUTE) {
      free_geometry(h);
      if (h.geo_state > 0) h.geo_state = 0;
    }
    invalidate(h);
  }
  return VDR_OK;
}

int vdr_geometry_status(vdr_handle *H, int *cached, long long *bytes) {
  int st = check_handle(H);
  if (st) return st;
  const Handle &h = H->h;
  if (cached) *cached = h.geo_state;
  if (bytes)
    *bytes = h.geo_state > 0 ? (long long)sizeof(float2) * GEO_PAIRS * h.E : 0;
  return VDR_OK;
}

int vdr_diag_beta_vf(int n, const double *pe, double *beta) {
  if (n < 0 || (n > 0 && (!pe || !beta))) {
    set_error("vdr_diag_beta_vf: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  for (int i = 0; i < n; i++)
    if (!(pe[i] > 0.0)) {
      set_error("vdr_diag_beta_vf: pe must be positive");
      return VDR_BAD_ARGUMENT;
    }
  cudaError_t e = diag_beta_vf(n, pe, beta);
  return e ? cuda_fail(e, "vdr_diag_beta_vf") : VDR_OK;
}

int vdr_set_mixed_operator(vdr_handle *H, int mode) {
  int st = check_handle(H);
  if (st) return st;
  if (mode != VDR_MIXED_ROUNDED && mode != VDR_MIXED_RECOMPUTE &&
      mode != VDR_MIXED_HALF) {
    set_error("vdr_set_mixed_operator: unknown mode");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = H->h;
  if (h.mixed_op != mode) {
    h.mixed_op = mode;
    h.op32_valid = false;
  }
  return VDR_OK;
}

int vdr_diag_wait_timeout(vdr_handle *H) {
  int st = check_handle(H);
  if (st) return st;
  return diag_wait_timeout(H->h);
}

int vdr_diag_barrier_timeout(vdr_handle *H) {
  int st = check_handle(H);
  if (st) return st;
  return diag_barrier_timeout(H->h);
}

int vdr_set_block_apply(vdr_handle *H, int variant) {
  int st = check_handle(H);
  if (st) return st;
  if (variant != VDR_BLOCK_APPLY_BULK && variant != VDR_BLOCK_APPLY_LSU &&
      variant != VDR_BLOCK_APPLY_TILE && variant != VDR_BLOCK_APPLY_TCGEN05 &&
      variant != VDR_BLOCK_APPLY_AUTO) {
    set_error("vdr_set_block_apply: unknown variant");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = H->h;
  h.block_tma = variant == VDR_BLOCK_APPLY_BULK;
  h.block_tile = variant == VDR_BLOCK_APPLY_TILE || variant == VDR_BLOCK_APPLY_TCGEN05 ||
                 variant == VDR_BLOCK_APPLY_AUTO;
  h.blk_tc_mode = variant == VDR_BLOCK_APPLY_TCGEN05 ? 1 : (variant == VDR_BLOCK_APPLY_AUTO ? -1 : 0);
  if (h.bk_graph) cudaGraphExecDestroy(h.bk_graph);
  h.bk_graph = nullptr;
  return VDR_OK;
}

int vdr_solve_block_device(vdr_handle *H, int K, int precision,
                           const double *B, double *X, double tol,
                           double inner_tol, int max_outer, int inner_itmax,
                           int *outer_iters, int *inner_iters, double *errs) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!B || !X || !(tol >= 0.0) || !(inner_tol > 0.0) || max_outer < 0 ||
      h.apply_mode != VDR_APPLY_STORED) {
    set_error("vdr_solve_block_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h))) return st;
  return solve_block_device(h, K, precision, B, X, tol, inner_tol, max_outer,
                            inner_itmax, outer_iters, inner_iters, errs);
}

int vdr_set_segments(vdr_handle *H, int nseg, const int *node_off) {
  int st = check_handle(H);
  if (st) return st;
  return set_segments(H->h, nseg, node_off);
}

int vdr_segment_tuning(vdr_handle *H, int *tile_nodes, int *threads) {
  int st = check_handle(H);
  if (st) return st;
  if (tile_nodes) *tile_nodes = H->h.seg_tile;
  if (threads) *threads = H->h.seg_threads;
  return VDR_OK;
}

int vdr_solve_segmented_device(vdr_handle *H, const double *b, double *x,
                               double tol, int itmax, int *iters, double *errs,
                               int *statuses) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (!b || !x || !(tol >= 0.0) || itmax < 0) {
    set_error("vdr_solve_segmented_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_operator(h))) return st;
  return solve_segmented_device(h, b, x, tol, itmax, iters, errs, statuses);
}

int vdr_solve(vdr_handle *H, const double *b, double *x, double tol,
              int itmax, int *iter, double *err) {
  int st = check_handle(H);
  if (st) return st;
  if ((st = ensure_io(H))) return st;
  Handle &h = H->h;
  double *db = H->io, *dx = H->io + h.N;
  if ((st = upload(db, b, sizeof(double) * h.N, h.stream)) ||
      (st = upload(dx, x, sizeof(double) * h.N, h.stream)))
    return st;
  st = vdr_solve_device(H, db, dx, tol, itmax, iter, err);
  if (st == VDR_CUDA_ERROR || st == VDR_BAD_ARGUMENT) return st;
  cudaError_t e = cudaMemcpyAsync(x, dx, sizeof(double) * h.N,
                                  cudaMemcpyDeviceToHost, h.stream);
  if (!e) e = cudaStreamSynchronize(h.stream);
  return e ? cuda_fail(e, "vdr_solve") : st;
}

int vdr_true_residual_device(vdr_handle *H, const double *b, const double *x,
                             double *rel) {
  int st = check_handle(H);
  if (st) return st;
  if ((st = ensure_operator(H->h))) return st;
  return true_residual_device(H->h, b, x, rel);
}

int vdr_time_steps(vdr_handle *H, int nsteps, double cf, double rM,
                   double *t, double tol, int itmax, double *masses,
                   int *iters, double *errs, int *steps_done) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  if (steps_done) *steps_done = 0;
  if (nsteps < 0 || !t || !(tol >= 0.0)) {
    set_error("vdr_time_steps: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = ensure_io(H))) return st;
  cudaError_t e;
  double *b = H->io + (size_t)h.N;
  double *dmass = nullptr;
  if (masses && nsteps > 0) {
    if ((e = cudaMalloc(&dmass, sizeof(double) * nsteps)))
      return cuda_fail(e, "vdr_time_steps: alloc");
  }
  if ((e = dalloc(&H->mass_partials, 8192))) {
    if (dmass) cudaFree(dmass);
    return cuda_fail(e, "alloc");
  }
  const int method = h.opt.solver == VDR_SOLVER_BICG ? VDR_SOLVER_BICG
                                                     : VDR_SOLVER_BICGSTAB;
  // With the stored operator the first step keeps M and F; every later step
  // (whose T_old is a solve's output, zero on Dirichlet nodes) forms
  // b = cf F - (H - rM M) T_old from two applies instead of a Gauss pass.
  const bool keep_mass = h.apply_mode == VDR_APPLY_STORED && h.aH != 0.0;
  if (keep_mass &&
      ((e = dalloc(&h.Mhi, (size_t)h.E * 16)) || (e = dalloc(&h.Mlo, (size_t)h.E * 16)) ||
       (e = dalloc(&h.Fvec, h.N)) || (e = dalloc(&h.rhs_tmp, 2 * (size_t)h.N)))) {
    if (dmass) cudaFree(dmass);
    return cuda_fail(e, "vdr_time_steps: alloc");
  }
  int status = VDR_OK, done = 0;
  for (int k = 0; k < nsteps; k++) {
    if (k > 0 && keep_mass && h.mass_valid && h.op64_valid) {
      if ((e = launch_rhs_from_mass(h, cf, rM, t, b, h.stream))) {
        status = cuda_fail(e, "rhs");
        break;
      }
    } else {
      BuildArgs rhs;
      rhs.cf = cf;
      rhs.rM = rM;
      rhs.told = t;
      rhs.b = b;
      if (keep_mass) {
        rhs.Mhi = h.Mhi;
        rhs.Mlo = h.Mlo;
        rhs.f = h.Fvec;
      }
      if ((st = build_operator(h, &rhs))) {
        status = st;
        break;
      }
    }
    int it = 0;
    double err = 0.0;
    st = solve_by_option(h, method, b, t, tol, itmax, &it, &err);
    if (iters) iters[k] = it;
    if (errs) errs[k] = err;
    if (dmass && (e = launch_mass(h, t, H->mass_partials, dmass + k, h.stream))) {
      status = cuda_fail(e, "mass");
      break;
    }
    if (st != VDR_OK) {
      status = st;
      break;
    }
    done = k + 1;
  }
  if (dmass) {
    e = cudaMemcpyAsync(masses, dmass, sizeof(double) * nsteps,
                        cudaMemcpyDeviceToHost, h.stream);
    if (!e) e = cudaStreamSynchronize(h.stream);
    cudaFree(dmass);
    if (e && status == VDR_OK) status = cuda_fail(e, "masses");
  }
  if (steps_done) *steps_done = done;
  return status;
}

int vdr_mass_device(vdr_handle *H, const double *c, double *mass) {
  int st = check_handle(H);
  if (st) return st;
  Handle &h = H->h;
  cudaError_t e;
  if ((e = dalloc(&H->mass_partials, 8192)) || (e = dalloc(&H->mass_out, 1)))
    return cuda_fail(e, "alloc");
  if ((e = launch_mass(h, c, H->mass_partials, H->mass_out, h.stream)))
    return cuda_fail(e, "mass");
  e = cudaMemcpyAsync(mass, H->mass_out, sizeof(double), cudaMemcpyDeviceToHost,
                      h.stream);
  if (!e) e = cudaStreamSynchronize(h.stream);
  return e ? cuda_fail(e, "mass") : VDR_OK;
}

int vdr_mass(vdr_handle *H, const double *c, double *mass) {
  int st = check_handle(H);
  if (st) return st;
  if ((st = ensure_io(H))) return st;
  if ((st = upload(H->io, c, sizeof(double) * H->h.N, H->h.stream))) return st;
  return vdr_mass_device(H, H->io, mass);
}

int vdr_color_elements(int nnode, int nelem, const int *iss, int *colors) {
  if (!iss || !colors || nnode < 1 || nelem < 1) {
    set_error("vdr_color_elements: bad arguments");
    return -VDR_BAD_ARGUMENT;
  }
  for (long t = 0; t < 8L * nelem; t++)
    if (iss[t] < 1 || iss[t] > nnode) {
      set_error("vdr_color_elements: iss entry outside 1..nnode");
      return -VDR_BAD_ARGUMENT;
    }
  int nax = 0, nay = 0, naz = 0;
  detect_structured(nnode, nelem, iss, &nax, &nay, &naz);
  std::vector<int> color;
  const int nc = element_colors(nnode, nelem, nax, nay, iss, color);
  if (nc < 1) {
    set_error("vdr_color_elements: more than 32 colours needed");
    return -VDR_BAD_ARGUMENT;
  }
  std::memcpy(colors, color.data(), sizeof(int) * (size_t)nelem);
  return nc;
}

int vdr_last_solve_stats(vdr_handle *H, vdr_solve_stats *stats) {
  if (!H || !stats) {
    set_error("vdr_last_solve_stats: null argument");
    return VDR_BAD_ARGUMENT;
  }
  *stats = H->h.last;
  return VDR_OK;
}

long long vdr_kernel_launch_count(void) { return launches_so_far(); }

void *vdr_stream(vdr_handle *H) { return H ? (void *)H->h.stream : nullptr; }

int vdr_destroy(vdr_handle *H) {
  if (!H) return VDR_OK;
  cudaSetDevice(H->h.device);
  if (H->h.stream) cudaStreamSynchronize(H->h.stream);
  dfree(H->io);
  dfree(H->mass_partials);
  dfree(H->mass_out);
  free_handle(H->h);
  delete H;
  return VDR_OK;
}

// ---------------------------------------------------------------------------
// Drop-in: kernel_dbcg_simple_ (src_v2026_2_1/cudatest.cu:301-602).
// Device buffers persist in a process-wide context and grow as needed, so a
// time loop pays for cudaMalloc once, not per step as the reference does
// (cudatest.cu:408-432, 576-601).
// ---------------------------------------------------------------------------
namespace {
struct Legacy {
  std::mutex mu;
  Handle h;
  int capN = 0, capE = 0;
  double *bb = nullptr, *b = nullptr, *x = nullptr;
  int *iss = nullptr, *bc = nullptr, *bad = nullptr;
};
Legacy &legacy() {
  static Legacy L;
  return L;
}

int legacy_prepare(Legacy &L, int N, int E) {
  Handle &h = L.h;
  cudaError_t e;
  if (!h.stream) {
    vdr_default_options(&h.opt);
    h.opt.solver = VDR_SOLVER_BICG;
    if ((e = cudaGetDevice(&h.device))) return cuda_fail(e, "device");
    if ((e = cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking)))
      return cuda_fail(e, "stream");
    h.scatter = VDR_SCATTER_ATOMIC;
    h.apply_mode = VDR_APPLY_STORED;
    h.storage = VDR_STORE_DF;
  }
  if (N > L.capN || E > L.capE) {
    dfree(h.A64); h.A64 = nullptr;
    dfree(h.Ahi); h.Ahi = nullptr;
    dfree(h.Alo); h.Alo = nullptr;
    dfree(h.conn); h.conn = nullptr;
    dfree(h.diag); h.diag = nullptr;
    dfree(h.dinv); h.dinv = nullptr;
    dfree(h.mask); h.mask = nullptr;
    dfree(L.bb); L.bb = nullptr;
    dfree(L.b); L.b = nullptr;
    dfree(L.x); L.x = nullptr;
    dfree(L.iss); L.iss = nullptr;
    dfree(L.bc); L.bc = nullptr;
    dfree(h.work); h.work = nullptr; h.nwork = 0;
    dfree(h.partials); h.partials = nullptr;
    dfree(h.st); h.st = nullptr;
    if (h.h_st) cudaFreeHost(h.h_st);
    h.h_st = nullptr;
    for (int k = 0; k < Handle::NGRAPH; k++) {
      if (h.graph_exec[k]) cudaGraphExecDestroy(h.graph_exec[k]);
      h.graph_exec[k] = nullptr;
      h.graph_key[k] = nullptr;
    }
    for (int k = 0; k < 2; k++) {
      if (h.ev[k]) cudaEventDestroy(h.ev[k]);
      h.ev[k] = nullptr;
    }
    const size_t cN = std::max(N, L.capN), cE = std::max(E, L.capE);
    if ((e = dalloc(&h.Ahi, cE * 16)) ||
        (e = dalloc(&h.Alo, cE * 16)) || (e = dalloc(&h.conn, cE * 8)) ||
        (e = dalloc(&h.diag, cN)) || (e = dalloc(&h.dinv, cN)) ||
        (e = dalloc(&h.mask, cN)) ||
        (e = dalloc(&L.bb, cE * 64)) || (e = dalloc(&L.b, cN)) ||
        (e = dalloc(&L.x, cN)) || (e = dalloc(&L.iss, cE * 8)) ||
        (e = dalloc(&L.bc, cN)) || (e = dalloc(&L.bad, 1))) {
      L.capN = L.capE = 0;
      return cuda_fail(e, "kernel_dbcg_simple_: alloc");
    }
    L.capN = (int)cN;
    L.capE = (int)cE;
  }
  return VDR_OK;
}
}  // namespace

void kernel_dbcg_simple_(int *Np, double *B, double *X, double *TOLp,
                         int *ITMAXp, int *ITERp, double *ERRp, double *BB,
                         int *ISS, double *DIAG, int *NAXp, int *NAYp,
                         int *NAZp, int *bc_dirichlet) {
  const double inf = std::numeric_limits<double>::infinity();
  if (!Np || !B || !X || !TOLp || !ITMAXp || !ITERp || !ERRp || !BB || !ISS ||
      !DIAG || !NAXp || !NAYp || !NAZp) {
    set_error("kernel_dbcg_simple_: null argument");
    if (ERRp) *ERRp = inf;
    return;
  }
  const int N = *Np;
  const long nax = *NAXp, nay = *NAYp, naz = *NAZp;
  const long E = (nax - 1) * (nay - 1) * (naz - 1);
  if (N < 1 || nax < 2 || nay < 2 || naz < 2 || nax * nay * naz != N ||
      E > 0x7fffffffL / 64) {
    set_error("kernel_dbcg_simple_: N must equal NAX*NAY*NAZ");
    *ERRp = inf;
    return;
  }
  Legacy &L = legacy();
  std::lock_guard<std::mutex> lock(L.mu);
  Handle &h = L.h;
  int st = legacy_prepare(L, N, (int)E);
  if (st) {
    *ERRp = inf;
    return;
  }
  h.N = N;
  h.E = (int)E;
  cudaStream_t s = h.stream;
  cudaError_t e;
  int bad = 0;
  do {
    if ((e = cudaMemcpyAsync(L.b, B, sizeof(double) * N, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(L.x, X, sizeof(double) * N, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(L.bb, BB, sizeof(double) * 64 * E, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(L.iss, ISS, sizeof(int) * 8 * E, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(h.diag, DIAG, sizeof(double) * N, cudaMemcpyHostToDevice, s)))
      break;
    if (bc_dirichlet) {
      if ((e = cudaMemcpyAsync(L.bc, bc_dirichlet, sizeof(int) * N, cudaMemcpyHostToDevice, s)) ||
          (e = launch_bc_to_mask(L.bc, h.mask, N, s)))
        break;
    } else if ((e = cudaMemsetAsync(h.mask, 0, N, s))) {
      break;
    }
    if ((e = cudaMemsetAsync(L.bad, 0, sizeof(int), s)) ||
        (e = launch_legacy_conn(L.iss, (int)E, N, bc_dirichlet ? L.bc : nullptr,
                                h.conn, L.bad, s)) ||
        (e = launch_legacy_bb_df(L.bb, (int)E, h.Ahi, h.Alo, L.bad, s)) ||
        (e = launch_diag_fix(h.diag, h.dinv, nullptr, N, s)) ||
        (e = cudaMemcpyAsync(&bad, L.bad, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      break;
    // BB entries outside the double-float window: the FP64 store (allocated
    // on first need, at the buffers' capacity)
    h.storage = (bad & 2) ? VDR_STORE_FP64 : VDR_STORE_DF;
    if ((bad & 2) && ((e = dalloc(&h.A64, (size_t)L.capE * 32)) ||
                      (e = launch_legacy_bb(L.bb, (int)E, h.A64, s))))
      break;
  } while (0);
  if (e) {
    cuda_fail(e, "kernel_dbcg_simple_: upload");
    *ERRp = inf;
    return;
  }
  if (bad & 1) {
    set_error("kernel_dbcg_simple_: ISS entry outside 1..N");
    *ERRp = inf;
    return;
  }
  h.op64_valid = h.diag_valid = true;
  h.fields_set = true;
  int iter = 0;
  double err = inf;
  st = solve_device(h, VDR_SOLVER_BICG, L.b, L.x, *TOLp, *ITMAXp, &iter, &err);
  if (st == VDR_CUDA_ERROR || st == VDR_BAD_ARGUMENT) {
    *ERRp = inf;
    return;
  }
  e = cudaMemcpyAsync(X, L.x, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
  if (!e) e = cudaStreamSynchronize(s);
  if (e) {
    cuda_fail(e, "kernel_dbcg_simple_: download");
    *ERRp = inf;
    return;
  }
  *ITERp = iter;
  *ERRp = err;
}

}  // extern "C"
