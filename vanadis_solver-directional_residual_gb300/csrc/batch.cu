// batch.cu -- many independent meshes solved together.
//
// The meshes are concatenated into one block-diagonal system (node and
// element ranges per mesh; no element couples two meshes), so the element
// build and the operator apply of the handle process every mesh in single
// launches.  The Krylov method is Jacobi-BiCGStab with one set of scalars
// per mesh ("segment"):
//
//  * the node range is cut into tiles that never straddle a segment; a
//    block processes one tile, so its partial sums belong to one segment;
//  * each tile writes its partials and takes a ticket on its segment; the
//    last tile of a segment adds the segment's partials in tile order
//    (deterministic) and updates the segment's scalars -- no grid-wide
//    wait and no spin anywhere;
//  * a segment that converges (or breaks down) freezes: its vectors stop
//    changing, and when the last active segment finishes the global `done`
//    flag is raised, which every kernel checks at entry, so K iterations of
//    all meshes are captured once as a CUDA graph and replayed;
//  * the tile size and block size are chosen by measurement at the first
//    solve (autotuner over a representative segmented reduction pass on the
//    actual segment layout).
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "vdr_internal.h"

namespace vdr {
namespace {

constexpr unsigned FULLB = 0xffffffffu;

struct SegTile {
  int seg, start, end;
};

// Per-segment state, structure of arrays in one device buffer.
struct SegState {
  double *bnrm2, *err, *rho, *rho_old, *alpha, *omega, *snrm, *partials;
  int *active, *sconv, *status, *iter, *tile_begin, *tile_count;
  unsigned *ticket;
  int *nactive;  // active segments left
  int *done;     // 1 when no segment is active (gates every kernel)
  int itmax;
  double tol;
};

struct SegVec {
  const SegTile *tiles;
  SegState s;
  const double *b, *dinv;
  const unsigned char *m;
  double *x, *r, *rh, *p, *v, *ph, *sv, *sh, *t;
};

// Block sum of NQ values; valid in thread 0.
template <int NQ>
__device__ __forceinline__ void bsum(double (&v)[NQ]) {
  __shared__ double sm[32][NQ];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; q++) {
#pragma unroll
    for (int off = 16; off; off >>= 1) v[q] += __shfl_xor_sync(FULLB, v[q], off);
  }
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; q++) sm[w][q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (int)(blockDim.x >> 5);
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      double a = 0.0;
      for (int j = 0; j < nw; j++) a += sm[j][q];
      v[q] = a;
    }
  }
}

// Writes this tile's partials; true in thread 0 of the segment's last tile
// with the segment totals in out.
template <int NQ>
__device__ __forceinline__ bool seg_sum(double (&v)[NQ], const SegVec &a, int tile,
                                        int seg, double (&out)[NQ]) {
  bsum<NQ>(v);
  if (threadIdx.x != 0) return false;
  const int tb = a.s.tile_begin[seg], tc = a.s.tile_count[seg];
  const int local = tile - tb;
#pragma unroll
  for (int q = 0; q < NQ; q++) a.s.partials[(size_t)q * gridDim.x + tile] = v[q];
  __threadfence();
  if (atomicAdd(a.s.ticket + seg, 1u) != (unsigned)(tc - 1)) return false;
  __threadfence();
  (void)local;
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    double s = 0.0;
    for (int k = 0; k < tc; k++) s += __ldcg(a.s.partials + (size_t)q * gridDim.x + tb + k);
    out[q] = s;
  }
  a.s.ticket[seg] = 0u;
  return true;
}

__device__ __forceinline__ void seg_finish(const SegVec &a, int seg, int status) {
  a.s.active[seg] = 0;
  a.s.status[seg] = status;
  if (atomicSub(a.s.nactive, 1) == 1) *a.s.done = 1;
}

#define TLOOP(i) for (int i = tl.start + threadIdx.x; i < tl.end; i += blockDim.x)

// r = b - r (r holds A x); rh = r; per-segment ||b||, ||r||.
__global__ void sg_start(SegVec a) {
  const int tile = blockIdx.x;
  const SegTile tl = a.tiles[tile];
  double v[2] = {0.0, 0.0};
  TLOOP(i) {
    const double bi = a.b[i];
    const double ri = bi - a.r[i];
    a.r[i] = ri;
    a.rh[i] = ri;
    v[0] += bi * bi;
    v[1] += ri * ri;
  }
  double o[2];
  if (seg_sum<2>(v, a, tile, tl.seg, o)) {
    const int s = tl.seg;
    a.s.bnrm2[s] = o[0];
    a.s.rho[s] = o[1];
    a.s.rho_old[s] = 1.0;
    a.s.alpha[s] = 1.0;
    a.s.omega[s] = 1.0;
    a.s.sconv[s] = 0;
    a.s.iter[s] = 0;
    const double err = o[0] > 0.0 ? sqrt(o[1] / o[0]) : 0.0;
    a.s.err[s] = err;
    if (o[0] == 0.0 || err <= a.s.tol) {
      seg_finish(a, s, VDR_OK);
    } else if (!(err == err)) {
      seg_finish(a, s, VDR_BREAKDOWN);
    } else {
      a.s.status[s] = VDR_NOT_CONVERGED;
    }
  }
}

// x = 0 on segments whose b is zero (their solution).
__global__ void sg_zero(SegVec a) {
  const SegTile tl = a.tiles[blockIdx.x];
  if (a.s.bnrm2[tl.seg] != 0.0) return;
  TLOOP(i) a.x[i] = 0.0;
}

__global__ void sg_p(SegVec a) {
  if (*a.s.done) return;
  const SegTile tl = a.tiles[blockIdx.x];
  const int s = tl.seg;
  const bool act = a.s.active[s];
  if (!act) return;  // frozen: its elements are skipped by the apply too
  const bool first = a.s.iter[s] == 0;
  const double beta = first ? 0.0
      : (a.s.rho[s] / a.s.rho_old[s]) * (a.s.alpha[s] / a.s.omega[s]);
  const double om = a.s.omega[s];
  TLOOP(i) {
    double pi = 0.0;
    if (act) pi = first ? a.r[i] : a.r[i] + beta * (a.p[i] - om * a.v[i]);
    a.p[i] = pi;
    a.ph[i] = a.m[i] ? 0.0 : pi * a.dinv[i];
    a.v[i] = 0.0;
  }
}

__global__ void sg_alpha(SegVec a) {
  if (*a.s.done) return;
  const int tile = blockIdx.x;
  const SegTile tl = a.tiles[tile];
  if (!a.s.active[tl.seg]) return;
  double v[1] = {0.0};
  TLOOP(i) v[0] += a.rh[i] * a.v[i];
  double o[1];
  if (seg_sum<1>(v, a, tile, tl.seg, o)) {
    const int s = tl.seg;
    if (a.s.active[s]) {
      if (o[0] == 0.0 || !isfinite(o[0])) {
        a.s.alpha[s] = 0.0;
        seg_finish(a, s, VDR_BREAKDOWN);
      } else {
        a.s.alpha[s] = a.s.rho[s] / o[0];
      }
    }
  }
}

__global__ void sg_s(SegVec a) {
  if (*a.s.done) return;
  const int tile = blockIdx.x;
  const SegTile tl = a.tiles[tile];
  const int s = tl.seg;
  if (!a.s.active[s]) return;
  const double al = a.s.active[s] ? a.s.alpha[s] : 0.0;
  double v[1] = {0.0};
  TLOOP(i) {
    const double si = a.r[i] - al * a.v[i];
    a.sv[i] = si;
    a.sh[i] = a.m[i] ? 0.0 : si * a.dinv[i];
    a.t[i] = 0.0;
    v[0] += si * si;
  }
  double o[1];
  if (seg_sum<1>(v, a, tile, s, o)) {
    const double sn = a.s.bnrm2[s] > 0.0 ? sqrt(o[0] / a.s.bnrm2[s]) : 0.0;
    a.s.snrm[s] = sn;
    a.s.sconv[s] = (a.s.active[s] && sn <= a.s.tol) ? 1 : 0;
  }
}

__global__ void sg_omega(SegVec a) {
  if (*a.s.done) return;
  const int tile = blockIdx.x;
  const SegTile tl = a.tiles[tile];
  if (!a.s.active[tl.seg]) return;
  double v[2] = {0.0, 0.0};
  TLOOP(i) {
    v[0] += a.t[i] * a.sv[i];
    v[1] += a.t[i] * a.t[i];
  }
  double o[2];
  if (seg_sum<2>(v, a, tile, tl.seg, o)) {
    const int s = tl.seg;
    if (a.s.active[s] && !a.s.sconv[s]) {
      if (o[1] == 0.0 || !isfinite(o[1]) || !isfinite(o[0])) {
        a.s.omega[s] = 0.0;
        seg_finish(a, s, VDR_BREAKDOWN);
      } else {
        a.s.omega[s] = o[0] / o[1];
      }
    }
  }
}

__global__ void sg_xr(SegVec a) {
  if (*a.s.done) return;
  const int tile = blockIdx.x;
  const SegTile tl = a.tiles[tile];
  const int s = tl.seg;
  const bool act = a.s.active[s];
  if (!act) return;
  const bool sc = a.s.sconv[s];
  const double al = a.s.alpha[s];
  const double om = sc ? 0.0 : a.s.omega[s];
  double v[2] = {0.0, 0.0};
  TLOOP(i) {
    double ri = a.r[i];
    if (act) {
      a.x[i] += al * a.ph[i] + om * a.sh[i];
      ri = sc ? a.sv[i] : a.sv[i] - om * a.t[i];
      a.r[i] = ri;
    }
    v[0] += ri * ri;
    v[1] += a.rh[i] * ri;
  }
  double o[2];
  if (seg_sum<2>(v, a, tile, s, o)) {
    if (act) {
      a.s.iter[s] += 1;
      a.s.rho_old[s] = a.s.rho[s];
      a.s.rho[s] = o[1];
      const double err = sqrt(o[0] / a.s.bnrm2[s]);
      a.s.err[s] = err;
      if (!(err == err)) {
        seg_finish(a, s, VDR_BREAKDOWN);
      } else if (err <= a.s.tol || sc) {
        if (sc) a.s.err[s] = a.s.snrm[s];
        seg_finish(a, s, VDR_OK);
      } else if (o[1] == 0.0 || om == 0.0) {
        seg_finish(a, s, VDR_BREAKDOWN);
      } else if (a.s.iter[s] >= a.s.itmax) {
        seg_finish(a, s, VDR_NOT_CONVERGED);
      }
    }
  }
}

// Autotuning probe: a two-vector segmented dot product (the shape of the
// reduction passes); results go to scratch.
__global__ void sg_probe(SegVec a) {
  const int tile = blockIdx.x;
  const SegTile tl = a.tiles[tile];
  double v[2] = {0.0, 0.0};
  TLOOP(i) {
    v[0] += a.b[i] * a.r[i];
    v[1] += a.r[i] * a.r[i];
  }
  double o[2];
  if (seg_sum<2>(v, a, tile, tl.seg, o)) a.s.snrm[tl.seg] = o[0] + o[1];
}

}  // namespace

// Builds the tile list for a tile size (nodes) from the segment offsets.
static void make_tiles(const std::vector<int> &off, int tile, std::vector<SegTile> &tiles,
                       std::vector<int> &begin, std::vector<int> &count) {
  tiles.clear();
  begin.assign(off.size() - 1, 0);
  count.assign(off.size() - 1, 0);
  for (size_t s = 0; s + 1 < off.size(); s++) {
    begin[s] = (int)tiles.size();
    for (int i = off[s]; i < off[s + 1]; i += tile)
      tiles.push_back(SegTile{(int)s, i, std::min(off[s + 1], i + tile)});
    count[s] = (int)tiles.size() - begin[s];
  }
}

int set_segments(Handle &h, int nseg, const int *node_off) {
  if (nseg < 1 || !node_off || node_off[0] != 0 || node_off[nseg] != h.N) {
    set_error("segments: need node_off[0] = 0, node_off[nseg] = N");
    return VDR_BAD_ARGUMENT;
  }
  for (int s = 0; s < nseg; s++)
    if (node_off[s + 1] <= node_off[s]) {
      set_error("segments: node offsets must increase");
      return VDR_BAD_ARGUMENT;
    }
  // every element's nodes must lie in one segment
  std::vector<int> conn((size_t)h.E * 8);
  cudaError_t e = cudaMemcpy(conn.data(), h.conn, sizeof(int) * conn.size(),
                             cudaMemcpyDeviceToHost);
  if (e) return cuda_fail(e, "segments: connectivity");
  std::vector<int> off(node_off, node_off + nseg + 1);
  std::vector<int> eseg(h.E);
  for (long p = 0; p < h.E; p++) {
    const int n0 = conn[p] & NODE_BITS;
    const int s0 = (int)(std::upper_bound(off.begin(), off.end(), n0) - off.begin()) - 1;
    eseg[p] = s0;
    for (int k = 1; k < 8; k++) {
      const int n = conn[(size_t)k * h.E + p] & NODE_BITS;
      if (n < off[s0] || n >= off[s0 + 1]) {
        set_error("segments: an element couples two segments");
        return VDR_BAD_ARGUMENT;
      }
    }
  }
  if (!h.seg_of_elem && (e = cudaMalloc(&h.seg_of_elem, sizeof(int) * (size_t)h.E)))
    return cuda_fail(e, "segments: alloc");
  if ((e = cudaMemcpy(h.seg_of_elem, eseg.data(), sizeof(int) * (size_t)h.E,
                      cudaMemcpyHostToDevice)))
    return cuda_fail(e, "segments: upload");
  h.seg_off = off;
  h.seg_tile = 0;  // re-tune at the next solve
  if (h.seg_graph) cudaGraphExecDestroy(h.seg_graph);
  h.seg_graph = nullptr;
  return VDR_OK;
}

namespace {
struct SegLayout {
  SegVec a;
  int ntiles, threads;
};

// Device layout for a tile size: tiles, per-segment arrays, vectors.
cudaError_t seg_layout(Handle &h, int tile, int threads, const double *b, double *x,
                       SegLayout &L) {
  const int nseg = (int)h.seg_off.size() - 1;
  std::vector<SegTile> tiles;
  std::vector<int> begin, count;
  make_tiles(h.seg_off, tile, tiles, begin, count);
  const int nt = (int)tiles.size();
  // doubles: 7 per segment + partials 2 per tile; ints: 6 per segment + 2
  const size_t dwords = (size_t)7 * nseg + 2 * (size_t)nt;
  const size_t iwords = (size_t)6 * nseg + 2 + 3 * (size_t)nt;
  cudaError_t e;
  if (h.seg_dwords < dwords) {
    if (h.seg_d) cudaFree(h.seg_d);
    h.seg_d = nullptr;
    h.seg_dwords = 0;
    if ((e = cudaMalloc(&h.seg_d, sizeof(double) * dwords))) return e;
    h.seg_dwords = dwords;
  }
  if (h.seg_iwords < iwords) {
    if (h.seg_i) cudaFree(h.seg_i);
    h.seg_i = nullptr;
    h.seg_iwords = 0;
    if ((e = cudaMalloc(&h.seg_i, sizeof(int) * iwords))) return e;
    h.seg_iwords = iwords;
  }
  int *ip = h.seg_i;
  SegTile *dt = reinterpret_cast<SegTile *>(ip + 6 * (size_t)nseg + 2);
  if ((e = cudaMemcpyAsync(dt, tiles.data(), sizeof(SegTile) * nt, cudaMemcpyHostToDevice,
                           h.stream)) ||
      (e = cudaMemcpyAsync(ip + 4 * (size_t)nseg, begin.data(), sizeof(int) * nseg,
                           cudaMemcpyHostToDevice, h.stream)) ||
      (e = cudaMemcpyAsync(ip + 5 * (size_t)nseg, count.data(), sizeof(int) * nseg,
                           cudaMemcpyHostToDevice, h.stream)))
    return e;
  SegVec &a = L.a;
  a = SegVec{};
  a.tiles = dt;
  double *dp = h.seg_d;
  a.s.bnrm2 = dp;
  a.s.err = dp + nseg;
  a.s.rho = dp + 2 * (size_t)nseg;
  a.s.rho_old = dp + 3 * (size_t)nseg;
  a.s.alpha = dp + 4 * (size_t)nseg;
  a.s.omega = dp + 5 * (size_t)nseg;
  a.s.snrm = dp + 6 * (size_t)nseg;
  a.s.partials = dp + 7 * (size_t)nseg;
  a.s.active = ip;
  a.s.sconv = ip + nseg;
  a.s.status = ip + 2 * (size_t)nseg;
  a.s.iter = ip + 3 * (size_t)nseg;
  a.s.tile_begin = ip + 4 * (size_t)nseg;
  a.s.tile_count = ip + 5 * (size_t)nseg;
  a.s.ticket = reinterpret_cast<unsigned *>(h.seg_ticket);
  a.s.nactive = ip + 6 * (size_t)nseg;
  a.s.done = ip + 6 * (size_t)nseg + 1;
  a.b = b;
  a.x = x;
  a.dinv = h.dinv;
  a.m = h.mask;
  double *w = h.work;
  const size_t N = h.N;
  a.r = w;
  a.rh = w + N;
  a.p = w + 2 * N;
  a.v = w + 3 * N;
  a.ph = w + 4 * N;
  a.sv = w + 5 * N;
  a.sh = w + 6 * N;
  a.t = w + 7 * N;
  L.ntiles = nt;
  L.threads = threads;
  return cudaSuccess;
}
}  // namespace

int solve_segmented_device(Handle &h, const double *b, double *x, double tol, int itmax,
                           int *iters, double *errs, int *statuses) {
  const int nseg = (int)h.seg_off.size() - 1;
  if (nseg < 1) {
    set_error("segmented solve: no segments (vdr_set_segments)");
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e = ensure_solver_workspace(h, 8);
  if (e) return cuda_fail(e, "solver workspace");
  cudaStream_t s = h.stream;
  if (!h.seg_ticket || h.seg_ticket_n < nseg) {
    if (h.seg_ticket) cudaFree(h.seg_ticket);
    h.seg_ticket = nullptr;
    if ((e = cudaMalloc(&h.seg_ticket, sizeof(unsigned) * nseg))) return cuda_fail(e, "alloc");
    if ((e = cudaMemset(h.seg_ticket, 0, sizeof(unsigned) * nseg))) return cuda_fail(e, "memset");
    h.seg_ticket_n = nseg;
  }
  SegLayout L;
  // ---- autotune the tile shape once per segment layout ----
  if (h.seg_tile == 0) {
    const int tiles_c[] = {512, 1024, 2048, 4096};
    const int threads_c[] = {128, 256, 512};
    float best = 1e30f;
    int bt = 1024, bth = 256;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int tile : tiles_c)
      for (int th : threads_c) {
        if (th > tile) continue;
        if ((e = seg_layout(h, tile, th, b, h.work, L))) return cuda_fail(e, "layout");
        for (int rep = 0; rep < 2; rep++) sg_probe<<<L.ntiles, th, 0, s>>>(L.a);
        cudaEventRecord(e0, s);
        for (int rep = 0; rep < 5; rep++) sg_probe<<<L.ntiles, th, 0, s>>>(L.a);
        cudaEventRecord(e1, s);
        count_launches(7);
        if ((e = cudaEventSynchronize(e1))) return cuda_fail(e, "autotune");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          bt = tile;
          bth = th;
        }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h.seg_tile = bt;
    h.seg_threads = bth;
    if (h.seg_graph) cudaGraphExecDestroy(h.seg_graph);
    h.seg_graph = nullptr;
  }
  if ((e = seg_layout(h, h.seg_tile, h.seg_threads, b, x, L))) return cuda_fail(e, "layout");
  const int nt = L.ntiles, th = L.threads;
  SegVec &a = L.a;
  a.s.tol = tol;
  a.s.itmax = itmax;
  const long long launches0 = launches_so_far();
  // initial state: all segments active, done = 0
  std::vector<int> ones(nseg, 1);
  int ctl[2] = {nseg, 0};
  if ((e = cudaMemcpyAsync(a.s.active, ones.data(), sizeof(int) * nseg,
                           cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(a.s.nactive, ctl, sizeof(int) * 2, cudaMemcpyHostToDevice, s)) ||
      (e = launch_mask_vec(x, h.mask, h.N, s)) ||
      (e = cudaMemsetAsync(a.r, 0, sizeof(double) * h.N, s)) ||
      (e = launch_apply(h, false, x, a.r, nullptr, nullptr, s)))
    return cuda_fail(e, "segmented start");
  sg_start<<<nt, th, 0, s>>>(a);
  sg_zero<<<nt, th, 0, s>>>(a);
  count_launches(2);
  if ((e = cudaGetLastError())) return cuda_fail(e, "segmented start");

  // the applies skip the elements of frozen meshes
  struct GateScope {
    Handle &h;
    GateScope(Handle &hh, const int *active) : h(hh) {
      h.gate_eseg = h.seg_of_elem;
      h.gate_active = active;
    }
    ~GateScope() {
      h.gate_eseg = nullptr;
      h.gate_active = nullptr;
    }
  } gate(h, a.s.active);
  const int K = h.opt.iters_per_graph > 0 ? h.opt.iters_per_graph : 8;
  const void *key = (const void *)((uintptr_t)b ^ ((uintptr_t)x << 1) ^
                                   ((uintptr_t)h.work << 2) ^ (uintptr_t)K ^
                                   ((uintptr_t)h.seg_tile << 16) ^ (uintptr_t)th);
  if (!h.seg_graph || h.seg_key != key) {
    if (h.seg_graph) cudaGraphExecDestroy(h.seg_graph);
    h.seg_graph = nullptr;
    cudaGraph_t graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)))
      return cuda_fail(e, "begin capture");
    const long long before = launches_so_far();
    for (int k = 0; k < K && !e; k++) {
      sg_p<<<nt, th, 0, s>>>(a);
      e = launch_apply(h, false, a.ph, a.v, a.s.done, nullptr, s);
      if (e) break;
      sg_alpha<<<nt, th, 0, s>>>(a);
      sg_s<<<nt, th, 0, s>>>(a);
      e = launch_apply(h, false, a.sh, a.t, a.s.done, nullptr, s);
      if (e) break;
      sg_omega<<<nt, th, 0, s>>>(a);
      sg_xr<<<nt, th, 0, s>>>(a);
      count_launches(5);
      e = cudaGetLastError();
    }
    h.seg_graph_launches = (long)(launches_so_far() - before);
    count_launches(before - launches_so_far());
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e) return cuda_fail(e, "segmented capture");
    if (e2) return cuda_fail(e2, "end capture");
    e = cudaGraphInstantiate(&h.seg_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e) return cuda_fail(e, "graph instantiate");
    h.seg_key = key;
  }
  const int max_launches = (itmax + K - 1) / K + 1;
  int *h_done = reinterpret_cast<int *>(h.h_st);  // pinned scratch
  int launched = 0;
  for (int c = 0; c < max_launches; c++) {
    if ((e = cudaGraphLaunch(h.seg_graph, s))) return cuda_fail(e, "graph launch");
    count_launches(h.seg_graph_launches);
    launched++;
    if ((e = cudaMemcpyAsync(h_done, a.s.done, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_fail(e, "state readback");
    if (*h_done) break;
  }
  if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "segmented solve");
  std::vector<int> st(nseg), it(nseg);
  std::vector<double> er(nseg);
  if ((e = cudaMemcpy(st.data(), a.s.status, sizeof(int) * nseg, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(it.data(), a.s.iter, sizeof(int) * nseg, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(er.data(), a.s.err, sizeof(double) * nseg, cudaMemcpyDeviceToHost)))
    return cuda_fail(e, "segment results");
  int status = VDR_OK, maxit = 0;
  for (int k = 0; k < nseg; k++) {
    if (st[k] == VDR_BREAKDOWN) status = VDR_BREAKDOWN;
    else if (st[k] != VDR_OK && status == VDR_OK) status = VDR_NOT_CONVERGED;
    maxit = std::max(maxit, it[k]);
  }
  if (iters) std::copy(it.begin(), it.end(), iters);
  if (errs) std::copy(er.begin(), er.end(), errs);
  if (statuses) std::copy(st.begin(), st.end(), statuses);
  h.last = vdr_solve_stats{};
  h.last.iterations = maxit;
  h.last.status = status;
  h.last.graph_launches = launched;
  h.last.kernel_launches = (int)(launches_so_far() - launches0);
  return status;
}

}  // namespace vdr
