// half.cu -- the 16-bit inner operator of the mixed-precision solve.
//
// The refinement loop of vdr_solve_mixed_device solves each correction
// A d = r approximately; its operator only has to be good to a few digits
// (the FP64 residual of the outer loop decides).  This store keeps the
// Jacobi-scaled, Dirichlet-projected operator
//
//     A^ = P A P D^-1     (D = the assembled diagonal, 1 on Dirichlet nodes)
//
// per element in IEEE binary16 with one power-of-two scale per element:
// entry (i,j) of element p is h16[i][p].j * 2^e16[p], every element's
// largest entry lying in [2^14, 2^15).  That is 128 bytes per element plus
// one exponent byte (the FP64 store holds 512, the FP32 one 256), and the
// element rows and columns of Dirichlet nodes are zero, so the apply reads
// no mask and the inner BiCGStab needs no preconditioner vectors (the
// correction is d = D^-1 y for A^ y = r).  Entries are rounded once, from
// the FP32 (hi) parts of the double-float store or from the FP64 store;
// relative rounding error <= 2^-11 of each element's largest entry.
//
// Layout: uint4 A16[i*E + p] = the 8 halves of row i of element p (a warp
// reads 512 contiguous bytes per row); signed char e16[p].
//
// Apply (y += A^ x, FP32 vectors, FP32 accumulation): one thread per
// element.  On the canonical structured numbering the node numbers come
// from the element number and the scatter is aggregated within the warp:
// element p and element p + 1 of the same x row share four nodes (local
// nodes 1,2,5,6 of p are 0,3,4,7 of p + 1), so each lane hands its +x
// face's four sums to the next lane by a shuffle and issues four FP32
// atomics instead of eight (the last element of a run in the warp issues
// all eight).  Off the structured numbering it reads the connectivity table
// and scatters all eight.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "dfloat.cuh"
#include "vdr_internal.h"

namespace vdr {
namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float exp2i(int e) {
  return __int_as_float((127 + e) << 23);  // 2^e, e in [-126, 127]
}

// A^ from the FP32 (hi) rows of the double-float store or the FP64 rows,
// with D^-1 and the Dirichlet projection folded in; one thread per element.
template <bool STRUCT>
__global__ void __launch_bounds__(256) half_store_kernel(
    const float4 *__restrict__ Ahi, const double2 *__restrict__ A64,
    const ConnView cv, int E, const double *__restrict__ dinv,
    uint4 *__restrict__ A16, signed char *__restrict__ e16, int *bad) {
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < E;
       p += (long)gridDim.x * blockDim.x) {
    ElemNodes<STRUCT> c;
    c.load(cv, E, p);
    float cs[8];  // column scale: 1/diag, 0 on Dirichlet columns
#pragma unroll
    for (int s = 0; s < 8; s++)
      cs[s] = c[s] < 0 ? 0.f : (float)__ldg(dinv + c[s]);
    float v[8][8];
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      float r[8];
      if (Ahi) {
        const float4 a0 = __ldg(Ahi + (size_t)(2 * i) * E + p);
        const float4 a1 = __ldg(Ahi + (size_t)(2 * i + 1) * E + p);
        r[0] = a0.x; r[1] = a0.y; r[2] = a0.z; r[3] = a0.w;
        r[4] = a1.x; r[5] = a1.y; r[6] = a1.z; r[7] = a1.w;
      } else {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const double2 a = __ldg(A64 + (size_t)(4 * i + q) * E + p);
          r[2 * q] = (float)a.x;
          r[2 * q + 1] = (float)a.y;
        }
      }
      const float rs = c[i] < 0 ? 0.f : 1.f;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        v[i][j] = r[j] * cs[j] * rs;
        mx = fmaxf(mx, fabsf(v[i][j]));
      }
    }
    int e = 0;
    if (mx > 0.f) {
      if (!(mx < INFINITY)) {
        atomicOr(bad, 1);
      } else {
        e = ilogbf(mx) - 14;  // largest entry * 2^-e in [2^14, 2^15)
        if (e < -126 || e > 113) atomicOr(bad, 1);
        e = max(-126, min(113, e));
      }
    }
    const float sc = exp2i(-e);
#pragma unroll
    for (int i = 0; i < 8; i++) {
      __half2 h[4];
#pragma unroll
      for (int q = 0; q < 4; q++)
        h[q] = __floats2half2_rn(v[i][2 * q] * sc, v[i][2 * q + 1] * sc);
      uint4 w;
      w.x = *reinterpret_cast<unsigned *>(&h[0]);
      w.y = *reinterpret_cast<unsigned *>(&h[1]);
      w.z = *reinterpret_cast<unsigned *>(&h[2]);
      w.w = *reinterpret_cast<unsigned *>(&h[3]);
      A16[(size_t)i * E + p] = w;
    }
    e16[p] = (signed char)e;
  }
}

__device__ __forceinline__ float row_dot(const uint4 w, const float (&xv)[8]) {
  const __half2 *h = reinterpret_cast<const __half2 *>(&w);
  float2 f0 = __half22float2(h[0]), f1 = __half22float2(h[1]);
  float2 f2 = __half22float2(h[2]), f3 = __half22float2(h[3]);
  float o = f0.x * xv[0];
  o = fmaf(f0.y, xv[1], o);
  o = fmaf(f1.x, xv[2], o);
  o = fmaf(f1.y, xv[3], o);
  o = fmaf(f2.x, xv[4], o);
  o = fmaf(f2.y, xv[5], o);
  o = fmaf(f3.x, xv[6], o);
  o = fmaf(f3.y, xv[7], o);
  return o;
}

// y += A^ x on the canonical structured numbering, natural element order,
// warp-aggregated FP32 atomics.  The loop is warp-uniform (every lane of a
// warp runs the same trips) so that the shuffles see all 32 lanes.
__global__ void __launch_bounds__(256) apply_half_struct(
    const uint4 *__restrict__ A16, const signed char *__restrict__ e16, int E,
    int nex, int ney, int nax, int pl, const float *__restrict__ x,
    float *__restrict__ y, const int *skip, const int *skip2) {
  if (skip && *(volatile const int *)skip) return;
  if (skip2 && *(volatile const int *)skip2) return;
  const int lane = threadIdx.x & 31;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long w0 = (long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); w0 < E;
       w0 += stride) {
    const long p = w0 + lane;
    const bool valid = p < E;
    int i = 0, base = 0;
    float o[8];
    if (valid) {
      const unsigned u = (unsigned)p;
      const unsigned r = u / (unsigned)nex;
      i = (int)(u - r * (unsigned)nex);
      const unsigned k = r / (unsigned)ney, j = r - k * (unsigned)ney;
      base = i + nax * (int)j + pl * (int)k;
      float xv[8];
      xv[0] = __ldg(x + base);
      xv[1] = __ldg(x + base + 1);
      xv[2] = __ldg(x + base + 1 + nax);
      xv[3] = __ldg(x + base + nax);
      xv[4] = __ldg(x + base + pl);
      xv[5] = __ldg(x + base + 1 + pl);
      xv[6] = __ldg(x + base + 1 + nax + pl);
      xv[7] = __ldg(x + base + nax + pl);
      uint4 w[8];
#pragma unroll
      for (int q = 0; q < 8; q++) w[q] = __ldcs(A16 + (size_t)q * E + p);
      const float sc = exp2i(__ldg(e16 + p));
#pragma unroll
      for (int q = 0; q < 8; q++) o[q] = row_dot(w[q], xv) * sc;
    } else {
#pragma unroll
      for (int q = 0; q < 8; q++) o[q] = 0.f;
    }
    // local nodes 1,2,5,6 (+x face) of lane l are 0,3,4,7 of lane l + 1
    // when both elements lie in the same x row
    const float h1 = __shfl_up_sync(FULL, o[1], 1);
    const float h2 = __shfl_up_sync(FULL, o[2], 1);
    const float h5 = __shfl_up_sync(FULL, o[5], 1);
    const float h6 = __shfl_up_sync(FULL, o[6], 1);
    if (!valid) continue;
    if (lane > 0 && i > 0) {
      o[0] += h1;
      o[3] += h2;
      o[4] += h5;
      o[7] += h6;
    }
    atomicAdd(y + base, o[0]);
    atomicAdd(y + base + nax, o[3]);
    atomicAdd(y + base + pl, o[4]);
    atomicAdd(y + base + nax + pl, o[7]);
    const bool handed = lane < 31 && p + 1 < E && i + 1 < nex;
    if (!handed) {
      atomicAdd(y + base + 1, o[1]);
      atomicAdd(y + base + 1 + nax, o[2]);
      atomicAdd(y + base + 1 + pl, o[5]);
      atomicAdd(y + base + 1 + nax + pl, o[6]);
    }
  }
}

// y += A^ x off the structured numbering: the connectivity table (bit 31,
// the Dirichlet flag, is cleared: those rows and columns are zero in A^);
// atomics, or plain adds within one colour.
template <bool ATOMIC>
__global__ void __launch_bounds__(256) apply_half_table(
    const uint4 *__restrict__ A16, const signed char *__restrict__ e16,
    const int *__restrict__ conn, int E, int p0, int p1,
    const float *__restrict__ x, float *__restrict__ y, const int *skip,
    const int *skip2) {
  if (skip && *(volatile const int *)skip) return;
  if (skip2 && *(volatile const int *)skip2) return;
  for (long p = p0 + (long)blockIdx.x * blockDim.x + threadIdx.x; p < p1;
       p += (long)gridDim.x * blockDim.x) {
    int nd[8];
    float xv[8];
#pragma unroll
    for (int s = 0; s < 8; s++) {
      nd[s] = __ldg(conn + (size_t)s * E + p) & NODE_BITS;
      xv[s] = __ldg(x + nd[s]);
    }
    const float sc = exp2i(__ldg(e16 + p));
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const float o = row_dot(__ldcs(A16 + (size_t)q * E + p), xv) * sc;
      if (ATOMIC)
        atomicAdd(y + nd[q], o);
      else
        y[nd[q]] += o;
    }
  }
}

int grid_for(long n, int threads, int per_sm) {
  const long need = (n + threads - 1) / threads;
  return (int)std::max<long>(1, std::min<long>(need, (long)device_sm_count() * per_sm));
}

}  // namespace

bool half_store_available(const Handle &h) {
  return h.apply_mode == VDR_APPLY_STORED && (h.Ahi || h.A64) && h.dinv &&
         h.conn;
}

cudaError_t launch_half_store(Handle &h, int *bad, cudaStream_t s) {
  cudaError_t e;
  if (!h.A16 && (e = cudaMalloc(&h.A16, sizeof(uint4) * 8 * (size_t)h.E)))
    return e;
  if (!h.e16 && (e = cudaMalloc(&h.e16, (size_t)h.E))) return e;
  const ConnView cv = conn_view(h);
  const float4 *hi = (h.storage == VDR_STORE_DF) ? h.Ahi : nullptr;
  const double2 *a64 = hi ? nullptr : h.A64;
  const int grid = grid_for(h.E, 256, 8);
  if (cv.emask)
    half_store_kernel<true><<<grid, 256, 0, s>>>(hi, a64, cv, h.E, h.dinv, h.A16,
                                                 h.e16, bad);
  else
    half_store_kernel<false><<<grid, 256, 0, s>>>(hi, a64, cv, h.E, h.dinv, h.A16,
                                                  h.e16, bad);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_apply_half(const Handle &h, const float *x, float *y,
                              const int *skip, const int *skip2, cudaStream_t s) {
  const ConnView cv = conn_view(h);
  if (cv.emask) {
    // whole warps of elements: the grid covers E rounded up to 32
    const int grid = grid_for(h.E, 256, h.half_per_sm);
    apply_half_struct<<<grid, 256, 0, s>>>(h.A16, h.e16, h.E, cv.nex, cv.ney,
                                           cv.nax, cv.pl, x, y, skip, skip2);
    count_launches(1);
    return cudaGetLastError();
  }
  const bool color = h.scatter == VDR_SCATTER_COLOR;
  const int nranges = color ? h.ncolors : 1;
  for (int r = 0; r < nranges; r++) {
    const int p0 = color ? h.color_off[r] : 0;
    const int p1 = color ? h.color_off[r + 1] : h.E;
    if (p1 <= p0) continue;
    const int grid = grid_for(p1 - p0, 256, h.half_per_sm);
    if (color)
      apply_half_table<false><<<grid, 256, 0, s>>>(h.A16, h.e16, h.conn, h.E, p0,
                                                   p1, x, y, skip, skip2);
    else
      apply_half_table<true><<<grid, 256, 0, s>>>(h.A16, h.e16, h.conn, h.E, p0,
                                                  p1, x, y, skip, skip2);
    count_launches(1);
  }
  return cudaGetLastError();
}

}  // namespace vdr
