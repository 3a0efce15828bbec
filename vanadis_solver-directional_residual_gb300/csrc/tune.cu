// tune.cu -- launch shapes of the operator applies chosen by measurement.
//
// The stored applies stream their element matrices once per launch with
// grid-stride loops; how many blocks per SM the grid carries (and so how
// many elements each thread walks) changes the bytes in flight and the tail
// of the last wave.  Rather than fix it by hand, each handle times the
// candidates (TUNE_GRID_PER_SM resident blocks per SM) on its own operator
// the first time the operator is built -- before any solve captures an
// iteration into a CUDA graph -- and keeps the fastest; the binary16 inner
// operator's apply is tuned the same way when its store is first built.
// The results are cached per (scatter form, storage, element-count octave)
// for the process, so handles of similar size reuse them.  Meshes below 65,536
// elements, where the launch is too short to time, keep the default of 8.
// vdr_apply_tuning reports the choices and the measured times.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

#include "vdr_internal.h"

namespace vdr {
namespace {

constexpr int TUNE_MIN_ELEMENTS = 65536;

std::mutex g_tune_mu;
// (device, kind, scatter form, storage, floor(log2 E)) -> (blocks per SM, times)
struct TuneEntry {
  int per_sm;
  float ms[TUNE_GRIDS];
};
std::map<std::pair<long, long>, TuneEntry> g_tune_cache;

int ilog2(long v) {
  int r = 0;
  while (v > 1) {
    v >>= 1;
    r++;
  }
  return r;
}

bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}

// Times `launch` (3 launches after one warm-up) for every grid candidate,
// setting *per_sm before each; keeps the fastest in *per_sm.
template <typename F>
int time_grids(Handle &h, int *per_sm, float *ms_out, long key_kind, F launch) {
  int dev = 0;
  cudaGetDevice(&dev);
  // the scatter form changes the kernel (and its resident blocks per SM)
  const long form = (long)h.scatter * 2 + (h.warp_agg ? 1 : 0);
  const std::pair<long, long> key{((long)dev << 8) | key_kind,
                                  (form << 16) | ((long)h.storage << 8) | ilog2(h.E)};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *per_sm = it->second.per_sm;
      for (int c = 0; c < TUNE_GRIDS; c++) ms_out[c] = it->second.ms[c];
      return VDR_OK;
    }
  }
  cudaEvent_t e0, e1;
  cudaError_t e;
  if ((e = cudaEventCreate(&e0))) return cuda_fail(e, "tune events");
  if ((e = cudaEventCreate(&e1))) {
    cudaEventDestroy(e0);
    return cuda_fail(e, "tune events");
  }
  float best = 1e30f;
  int bc = 8;
  for (int c = 0; c < TUNE_GRIDS && !e; c++) {
    *per_sm = TUNE_GRID_PER_SM[c];
    if ((e = launch())) break;
    cudaEventRecord(e0, h.stream);
    for (int rep = 0; rep < 3 && !e; rep++) e = launch();
    cudaEventRecord(e1, h.stream);
    if (e || (e = cudaEventSynchronize(e1))) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms_out[c] = ms / 3.f;
    if (ms < best) {
      best = ms;
      bc = TUNE_GRID_PER_SM[c];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *per_sm = bc;
  if (e) return cuda_fail(e, "apply tuning");
  TuneEntry t;
  t.per_sm = bc;
  for (int c = 0; c < TUNE_GRIDS; c++) t.ms[c] = ms_out[c];
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache[key] = t;
  return VDR_OK;
}

}  // namespace

int tune_stored_apply(Handle &h) {
  if (h.apply_tuned) return VDR_OK;
  if (h.apply_mode != VDR_APPLY_STORED || h.E < TUNE_MIN_ELEMENTS || capturing(h.stream))
    return VDR_OK;
  h.apply_tuned = true;
  cudaError_t e = ensure_solver_workspace(h, 8);
  if (e) return cuda_fail(e, "tuning workspace");
  // x = the inverse diagonal (realistic magnitudes), y = scratch
  const double *x = h.dinv;
  double *y = h.work;
  const int st = time_grids(h, &h.apply_per_sm, h.apply_tune_ms, 1, [&]() {
    return launch_stored_apply(h, false, false, x, y, nullptr, nullptr, h.stream);
  });  // (the launchers count their own launches)
  // the solve graphs captured so far used the old grid
  for (int k = 0; k < Handle::NGRAPH; k++) {
    if (h.graph_exec[k]) cudaGraphExecDestroy(h.graph_exec[k]);
    h.graph_exec[k] = nullptr;
    h.graph_key[k] = nullptr;
  }
  return st;
}

int tune_half_apply(Handle &h) {
  if (h.half_tuned) return VDR_OK;
  if (!h.use_half || h.E < TUNE_MIN_ELEMENTS || capturing(h.stream)) return VDR_OK;
  h.half_tuned = true;
  cudaError_t e;
  if (!h.work32 && (e = cudaMalloc(&h.work32, sizeof(float) * 10 * (size_t)h.N)))
    return cuda_fail(e, "tuning workspace");
  const float *x = h.work32;
  float *y = h.work32 + h.N;
  if ((e = cudaMemsetAsync(h.work32, 0, sizeof(float) * 2 * (size_t)h.N, h.stream)))
    return cuda_fail(e, "tuning workspace");
  const int st = time_grids(h, &h.half_per_sm, h.half_tune_ms, 2, [&]() {
    return launch_apply_half(h, x, y, nullptr, nullptr, h.stream);
  });
  if (h.graph32) cudaGraphExecDestroy(h.graph32);
  h.graph32 = nullptr;
  return st;
}

}  // namespace vdr

using namespace vdr;

extern "C" int vdr_apply_tuning(vdr_handle *H, vdr_apply_tuning_info *info) {
  if (!H || !info) {
    set_error("vdr_apply_tuning: null argument");
    return VDR_BAD_ARGUMENT;
  }
  const Handle &h = handle_of(H);
  info->apply_blocks_per_sm = h.apply_per_sm;
  info->half_blocks_per_sm = h.half_per_sm;
  info->block_tile_y = h.blk_ty;
  info->block_halves = h.blk_halves;
  for (int c = 0; c < TUNE_GRIDS; c++) {
    info->grid_candidates[c] = TUNE_GRID_PER_SM[c];
    info->apply_ms[c] = h.apply_tune_ms[c];
    info->half_ms[c] = h.half_tune_ms[c];
  }
  for (int c = 0; c < TUNE_TILES; c++) info->block_ms[c] = h.blk_tune_ms[c];
  info->block_tcgen05 = h.blk_use_tc ? 1 : 0;
  return VDR_OK;
}
