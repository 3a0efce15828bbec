// apply.cu -- element-by-element operator apply over the HBM-resident
// element matrices, plus the small conversion kernels around it.
//
// y = P A P x with A = sum_e A_e (never assembled): one thread per element
// gathers x at its 8 nodes (Dirichlet columns read as 0 through the sign
// bit of the connectivity), multiplies by the element's 8x8 block and adds
// the 8 results into y.  The FP32-vector apply forms the node numbers from
// the element number on the canonical structured numbering (ConnView: 1
// byte of Dirichlet bits per element instead of 32 bytes of connectivity).  Same operation as matvec_0 / mttvec_0
// (vanadis_full_DR_OpenMP_timing.for:1837-1933) and MATVEC_C_cu /
// MTTVEC_C_cu (src_v2026_2_1/cudatest.cu:184-227).
//
// Layout of the element-matrix stores (GB300-first, not the reference's BB),
// all slot-major with stride E so that every warp load is 32 consecutive
// elements' same entries (512 contiguous bytes), streamed once per apply
// with the evict-first (.cs) cache hint so that x and y stay in the 129 MB
// L2: the default double-float store float4 Ahi/Alo[(2i + j/4)*E + p] (hi
// and lo FP32 parts of entry (i,j); the hi parts are also the rounded FP32
// operator), the FP64 store double2 A64[(4i + j/2)*E + p] (entries outside
// the pair window), the recomputed FP32 store float4 A32[(2i + j/4)*E + p].
//
// Scatter: VDR_SCATTER_ATOMIC uses fp64 atomics (red.global.add.f64) in
// natural element order; VDR_SCATTER_COLOR runs one pass per colour over a
// colour-major element order, with plain read-modify-writes (no two elements
// of a colour share a node, cudatest_coloring_gtx1060_optimized.cu:50-74).
#include <cuda_runtime.h>

#include <algorithm>

#include "dfloat.cuh"
#include "vdr_internal.h"

namespace vdr {
namespace {

template <bool TRANS, bool ATOMIC>
__global__ void __launch_bounds__(256) stored_apply_f64(
    const double2 *__restrict__ A, const int *__restrict__ conn, int E, int p0,
    int p1, const double *__restrict__ x, double *__restrict__ y,
    const int *skip, const int *skip2) {
  if (skip && *(volatile const int *)skip) return;
  if (skip2 && *(volatile const int *)skip2) return;
  for (long p = p0 + (long)blockIdx.x * blockDim.x + threadIdx.x; p < p1;
       p += (long)gridDim.x * blockDim.x) {
    int c[8];
    double xv[8];
#pragma unroll
    for (int s = 0; s < 8; s++) {
      c[s] = __ldg(conn + (size_t)s * E + p);
      xv[s] = c[s] < 0 ? 0.0 : __ldg(x + c[s]);
    }
    double acc[8];
    if (!TRANS) {
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const double2 a0 = __ldcs(A + (size_t)(4 * i + 0) * E + p);
        const double2 a1 = __ldcs(A + (size_t)(4 * i + 1) * E + p);
        const double2 a2 = __ldcs(A + (size_t)(4 * i + 2) * E + p);
        const double2 a3 = __ldcs(A + (size_t)(4 * i + 3) * E + p);
        acc[i] = a0.x * xv[0] + a0.y * xv[1] + a1.x * xv[2] + a1.y * xv[3] +
                 a2.x * xv[4] + a2.y * xv[5] + a3.x * xv[6] + a3.y * xv[7];
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) acc[j] = 0.0;
#pragma unroll
      for (int i = 0; i < 8; i++) {
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
          const double2 a = __ldcs(A + (size_t)(4 * i + jj) * E + p);
          acc[2 * jj] += a.x * xv[i];
          acc[2 * jj + 1] += a.y * xv[i];
        }
      }
    }
#pragma unroll
    for (int s = 0; s < 8; s++) {
      if (c[s] >= 0) {
        if (ATOMIC)
          atomicAdd(y + c[s], acc[s]);
        else
          y[c[s]] += acc[s];
      }
    }
  }
}

template <bool TRANS, bool ATOMIC>
__global__ void __launch_bounds__(256) stored_apply_f32(
    const float4 *__restrict__ A, const int *__restrict__ conn, int E, int p0,
    int p1, const double *__restrict__ x, double *__restrict__ y,
    const int *skip, const int *skip2) {
  if (skip && *(volatile const int *)skip) return;
  if (skip2 && *(volatile const int *)skip2) return;
  for (long p = p0 + (long)blockIdx.x * blockDim.x + threadIdx.x; p < p1;
       p += (long)gridDim.x * blockDim.x) {
    int c[8];
    float xv[8];
#pragma unroll
    for (int s = 0; s < 8; s++) {
      c[s] = __ldg(conn + (size_t)s * E + p);
      xv[s] = c[s] < 0 ? 0.f : (float)__ldg(x + c[s]);
    }
    float acc[8];
    if (!TRANS) {
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const float4 a0 = __ldcs(A + (size_t)(2 * i) * E + p);
        const float4 a1 = __ldcs(A + (size_t)(2 * i + 1) * E + p);
        acc[i] = a0.x * xv[0] + a0.y * xv[1] + a0.z * xv[2] + a0.w * xv[3] +
                 a1.x * xv[4] + a1.y * xv[5] + a1.z * xv[6] + a1.w * xv[7];
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) acc[j] = 0.f;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const float4 a0 = __ldcs(A + (size_t)(2 * i) * E + p);
        const float4 a1 = __ldcs(A + (size_t)(2 * i + 1) * E + p);
        acc[0] += a0.x * xv[i];
        acc[1] += a0.y * xv[i];
        acc[2] += a0.z * xv[i];
        acc[3] += a0.w * xv[i];
        acc[4] += a1.x * xv[i];
        acc[5] += a1.y * xv[i];
        acc[6] += a1.z * xv[i];
        acc[7] += a1.w * xv[i];
      }
    }
#pragma unroll
    for (int s = 0; s < 8; s++) {
      if (c[s] >= 0) {
        if (ATOMIC)
          atomicAdd(y + c[s], (double)acc[s]);
        else
          y[c[s]] += (double)acc[s];
      }
    }
  }
}

// The FP32 operator on FP32 vectors (the mixed solve's inner BiCGStab):
// y += A x with x gathered as float and the outputs scattered with FP32
// atomics (or plain adds within a colour) -- no float<->double conversions,
// which GB300 runs on its FP64 pipe.
template <bool ATOMIC, bool STRUCT>
__global__ void __launch_bounds__(256) stored_apply_f32v(
    const float4 *__restrict__ A, const ConnView cv, int E, int p0,
    int p1, const float *__restrict__ x, float *__restrict__ y, const int *skip,
    const int *skip2) {
  if (skip && *(volatile const int *)skip) return;
  if (skip2 && *(volatile const int *)skip2) return;
  for (long p = p0 + (long)blockIdx.x * blockDim.x + threadIdx.x; p < p1;
       p += (long)gridDim.x * blockDim.x) {
    ElemNodes<STRUCT> c;
    float xv[8];
    c.load(cv, E, p);
#pragma unroll
    for (int s = 0; s < 8; s++) xv[s] = c[s] < 0 ? 0.f : __ldg(x + c[s]);
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const float4 a0 = __ldcs(A + (size_t)(2 * i) * E + p);
      const float4 a1 = __ldcs(A + (size_t)(2 * i + 1) * E + p);
      const float o = a0.x * xv[0] + a0.y * xv[1] + a0.z * xv[2] + a0.w * xv[3] +
                      a1.x * xv[4] + a1.y * xv[5] + a1.z * xv[6] + a1.w * xv[7];
      if (c[i] >= 0) {
        if (ATOMIC)
          atomicAdd(y + c[i], o);
        else
          y[c[i]] += o;
      }
    }
  }
}

// Double-float store: entry (i,j) = hi + lo with hi in Ahi, lo in Alo, both
// float4 [(2i + j/4)*E + p].  x is split into FP32 pairs with integer bit
// operations; the 64-term contraction is FP32 two-products + TwoSum; each
// output is merged to FP64 with one FP64 add.  FP64-pipe work per element
// drops from 64 FMA to 8 adds, so the kernel is bound by HBM.
// Elements whose gathered x leaves the FP32 exponent range (|x| >= 2^128)
// are redone here in FP64 from the merged pairs, gather and scatter included.
template <typename Nodes>
__device__ __forceinline__ void df_element_fallback_core(
    const float4 *__restrict__ Ahi, const float4 *__restrict__ Alo,
    const Nodes &c, int E, long p, bool trans, bool atomic,
    const double *__restrict__ x, double *__restrict__ y) {
  double xv[8], out[8];
  for (int s = 0; s < 8; s++) {
    xv[s] = c[s] < 0 ? 0.0 : x[c[s]];
    out[s] = 0.0;
  }
  for (int i = 0; i < 8; i++)
    for (int h = 0; h < 2; h++) {
      const float4 vh = Ahi[(size_t)(2 * i + h) * E + p];
      const float4 vl = Alo[(size_t)(2 * i + h) * E + p];
      const double a[4] = {df_to_double(vh.x, vl.x), df_to_double(vh.y, vl.y),
                           df_to_double(vh.z, vl.z), df_to_double(vh.w, vl.w)};
      for (int k = 0; k < 4; k++) {
        const int j = 4 * h + k;
        if (trans)
          out[j] += a[k] * xv[i];
        else
          out[i] += a[k] * xv[j];
      }
    }
  for (int s = 0; s < 8; s++)
    if (c[s] >= 0) {
      if (atomic)
        atomicAdd(y + c[s], out[s]);
      else
        y[c[s]] += out[s];
    }
}

template <typename Nodes>
__device__ __noinline__ void df_element_fallback(
    const float4 *__restrict__ Ahi, const float4 *__restrict__ Alo,
    const Nodes &c, int E, long p, bool trans, bool atomic,
    const double *__restrict__ x, double *__restrict__ y) {
  df_element_fallback_core(Ahi, Alo, c, E, p, trans, atomic, x, y);
}

template <bool TRANS, bool ATOMIC, bool STRUCT>
__global__ void __launch_bounds__(256, 4) stored_apply_df(
    const float4 *__restrict__ Ahi, const float4 *__restrict__ Alo,
    const ConnView cv, int E, int p0, int p1,
    const double *__restrict__ x, double *__restrict__ y, const int *skip,
    const int *skip2, ElemGate gate) {
  if (skip && *(volatile const int *)skip) return;
  if (skip2 && *(volatile const int *)skip2) return;
  for (long p = p0 + (long)blockIdx.x * blockDim.x + threadIdx.x; p < p1;
       p += (long)gridDim.x * blockDim.x) {
    if (gate.active && !gate.active[__ldg(gate.eseg + p)]) continue;
    ElemNodes<STRUCT> c;
    double xv[8];
    float xh[8], xl[8];
    bool bad = false;
    int emax = 0;
    c.load(cv, E, p);
#pragma unroll
    for (int s = 0; s < 8; s++) {
      xv[s] = c[s] < 0 ? 0.0 : __ldg(x + c[s]);
      emax = max(emax, df_exp(xv[s]));
    }
    // x is scaled per element by 2^-shift so that its largest entry lies in
    // [1,2); entries 2^126 below it are dropped (relative 1e-38).
    const int shift = emax - 1023;
#pragma unroll
    for (int s = 0; s < 8; s++) df_split(xv[s], xh[s], xl[s], bad, shift);
    if (bad) {
      df_element_fallback(Ahi, Alo, c, E, p, TRANS, ATOMIC, x, y);
      continue;
    }
    if (!TRANS) {
      // each row is scattered as soon as it is complete (fewer live
      // registers: 4 blocks of 256 threads per SM)
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const float4 h0 = __ldcs(Ahi + (size_t)(2 * i) * E + p);
        const float4 h1 = __ldcs(Ahi + (size_t)(2 * i + 1) * E + p);
        const float4 l0 = __ldcs(Alo + (size_t)(2 * i) * E + p);
        const float4 l1 = __ldcs(Alo + (size_t)(2 * i + 1) * E + p);
        DfAcc acc{0.0f, 0.0f};
        df_fma_acc(acc, h0.x, l0.x, xh[0], xl[0]);
        df_fma_acc(acc, h0.y, l0.y, xh[1], xl[1]);
        df_fma_acc(acc, h0.z, l0.z, xh[2], xl[2]);
        df_fma_acc(acc, h0.w, l0.w, xh[3], xl[3]);
        df_fma_acc(acc, h1.x, l1.x, xh[4], xl[4]);
        df_fma_acc(acc, h1.y, l1.y, xh[5], xl[5]);
        df_fma_acc(acc, h1.z, l1.z, xh[6], xl[6]);
        df_fma_acc(acc, h1.w, l1.w, xh[7], xl[7]);
        double o = df_to_double(acc.s, acc.c);
        if (!df_scale(o, shift)) o = ldexp(o, shift);
        if (c[i] >= 0) {
          if (ATOMIC)
            atomicAdd(y + c[i], o);
          else
            y[c[i]] += o;
        }
      }
      continue;
    }
    double out[8];
    {
      DfAcc acc[8];
#pragma unroll
      for (int j = 0; j < 8; j++) acc[j] = DfAcc{0.0f, 0.0f};
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const float4 h0 = __ldcs(Ahi + (size_t)(2 * i) * E + p);
        const float4 h1 = __ldcs(Ahi + (size_t)(2 * i + 1) * E + p);
        const float4 l0 = __ldcs(Alo + (size_t)(2 * i) * E + p);
        const float4 l1 = __ldcs(Alo + (size_t)(2 * i + 1) * E + p);
        df_fma_acc(acc[0], h0.x, l0.x, xh[i], xl[i]);
        df_fma_acc(acc[1], h0.y, l0.y, xh[i], xl[i]);
        df_fma_acc(acc[2], h0.z, l0.z, xh[i], xl[i]);
        df_fma_acc(acc[3], h0.w, l0.w, xh[i], xl[i]);
        df_fma_acc(acc[4], h1.x, l1.x, xh[i], xl[i]);
        df_fma_acc(acc[5], h1.y, l1.y, xh[i], xl[i]);
        df_fma_acc(acc[6], h1.z, l1.z, xh[i], xl[i]);
        df_fma_acc(acc[7], h1.w, l1.w, xh[i], xl[i]);
      }
#pragma unroll
      for (int j = 0; j < 8; j++) out[j] = df_to_double(acc[j].s, acc[j].c);
    }
#pragma unroll
    for (int s = 0; s < 8; s++) {
      if (!df_scale(out[s], shift)) out[s] = ldexp(out[s], shift);
      if (c[s] >= 0) {
        if (ATOMIC)
          atomicAdd(y + c[s], out[s]);
        else
          y[c[s]] += out[s];
      }
    }
  }
}

// The double-float apply with warp-aggregated atomics (VDR_SCATTER_WARP), on
// the canonical structured numbering: lanes of a warp hold consecutive
// elements, and element p and p + 1 of one x row share the four nodes of
// their common face (local nodes 1,2,5,6 of p are 0,3,4,7 of p + 1).  Each
// lane computes its 8 outputs, hands its +x face's four to the next lane
// with shuffles, and issues four FP64 atomics instead of eight (lanes whose
// right neighbour is not in the same row, not in the warp, gated off or
// redone in FP64 issue all eight).  The loop runs whole warps so that every
// shuffle sees all 32 lanes.
template <bool TRANS>
__global__ void __launch_bounds__(256, 3) stored_apply_df_warp(
    const float4 *__restrict__ Ahi, const float4 *__restrict__ Alo,
    const ConnView cv, int E, int p0, int p1,
    const double *__restrict__ x, double *__restrict__ y, const int *skip,
    const int *skip2, ElemGate gate) {
  if (skip && *(volatile const int *)skip) return;
  if (skip2 && *(volatile const int *)skip2) return;
  const int lane = threadIdx.x & 31;
  const unsigned FULLW = 0xffffffffu;
  for (long w0 = p0 + (long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); w0 < p1;
       w0 += (long)gridDim.x * blockDim.x) {
    const long p = w0 + lane;
    bool normal = p < p1;
    if (normal && gate.active && !gate.active[__ldg(gate.eseg + p)]) normal = false;
    ElemNodes<true> c;
    double out[8];
#pragma unroll
    for (int s = 0; s < 8; s++) out[s] = 0.0;
    int ix = 0;
    bool redo = false;  // x outside the FP32 range: the FP64 fallback
    if (normal) {
      c.load(cv, E, p);
      ix = (int)(p % cv.nex);
      double xv[8];
      float xh[8], xl[8];
      bool bad = false;
      int emax = 0;
#pragma unroll
      for (int s = 0; s < 8; s++) {
        xv[s] = c[s] < 0 ? 0.0 : __ldg(x + c[s]);
        emax = max(emax, df_exp(xv[s]));
      }
      const int shift = emax - 1023;
#pragma unroll
      for (int s = 0; s < 8; s++) df_split(xv[s], xh[s], xl[s], bad, shift);
      if (bad) {
        redo = true;
        normal = false;
      } else if (TRANS) {
        DfAcc acc[8];
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j] = DfAcc{0.0f, 0.0f};
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const float4 h0 = __ldcs(Ahi + (size_t)(2 * i) * E + p);
          const float4 h1 = __ldcs(Ahi + (size_t)(2 * i + 1) * E + p);
          const float4 l0 = __ldcs(Alo + (size_t)(2 * i) * E + p);
          const float4 l1 = __ldcs(Alo + (size_t)(2 * i + 1) * E + p);
          df_fma_acc(acc[0], h0.x, l0.x, xh[i], xl[i]);
          df_fma_acc(acc[1], h0.y, l0.y, xh[i], xl[i]);
          df_fma_acc(acc[2], h0.z, l0.z, xh[i], xl[i]);
          df_fma_acc(acc[3], h0.w, l0.w, xh[i], xl[i]);
          df_fma_acc(acc[4], h1.x, l1.x, xh[i], xl[i]);
          df_fma_acc(acc[5], h1.y, l1.y, xh[i], xl[i]);
          df_fma_acc(acc[6], h1.z, l1.z, xh[i], xl[i]);
          df_fma_acc(acc[7], h1.w, l1.w, xh[i], xl[i]);
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
          out[j] = df_to_double(acc[j].s, acc[j].c);
          if (!df_scale(out[j], shift)) out[j] = ldexp(out[j], shift);
        }
      } else {
        // row by row: one accumulator pair live at a time
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const float4 h0 = __ldcs(Ahi + (size_t)(2 * i) * E + p);
          const float4 h1 = __ldcs(Ahi + (size_t)(2 * i + 1) * E + p);
          const float4 l0 = __ldcs(Alo + (size_t)(2 * i) * E + p);
          const float4 l1 = __ldcs(Alo + (size_t)(2 * i + 1) * E + p);
          DfAcc acc{0.0f, 0.0f};
          df_fma_acc(acc, h0.x, l0.x, xh[0], xl[0]);
          df_fma_acc(acc, h0.y, l0.y, xh[1], xl[1]);
          df_fma_acc(acc, h0.z, l0.z, xh[2], xl[2]);
          df_fma_acc(acc, h0.w, l0.w, xh[3], xl[3]);
          df_fma_acc(acc, h1.x, l1.x, xh[4], xl[4]);
          df_fma_acc(acc, h1.y, l1.y, xh[5], xl[5]);
          df_fma_acc(acc, h1.z, l1.z, xh[6], xl[6]);
          df_fma_acc(acc, h1.w, l1.w, xh[7], xl[7]);
          out[i] = df_to_double(acc.s, acc.c);
          if (!df_scale(out[i], shift)) out[i] = ldexp(out[i], shift);
        }
      }
    }
    // hand the +x face to the next lane where both are normal elements of
    // one x row; masked outputs (Dirichlet rows) are never added
    const unsigned nm = __ballot_sync(FULLW, normal);
    const bool hand = normal && lane < 31 && ((nm >> (lane + 1)) & 1u) &&
                      ix + 1 < cv.nex;
    const unsigned hm = __ballot_sync(FULLW, hand);
    const double r1 = __shfl_up_sync(FULLW, out[1], 1);
    const double r2 = __shfl_up_sync(FULLW, out[2], 1);
    const double r5 = __shfl_up_sync(FULLW, out[5], 1);
    const double r6 = __shfl_up_sync(FULLW, out[6], 1);
    if (redo) df_element_fallback_core(Ahi, Alo, c, E, p, TRANS, true, x, y);
    if (!normal) continue;
    if (lane > 0 && ((hm >> (lane - 1)) & 1u)) {
      out[0] += r1;
      out[3] += r2;
      out[4] += r5;
      out[7] += r6;
    }
#pragma unroll
    for (int s = 0; s < 8; s++) {
      const bool plusx = (s == 1 || s == 2 || s == 5 || s == 6);
      if (plusx && hand) continue;
      if (c[s] >= 0) atomicAdd(y + c[s], out[s]);
    }
  }
}

// BiCG's two products in one pass over the double-float store: y1 += A x1
// and y2 += A^T x2 (A p and A^T p~ of one iteration), each element matrix
// read once.  Both inputs are split per element as in stored_apply_df; rows
// of A x1 are scattered as they complete, the columns of A^T x2 accumulate
// in registers.  Elements with an input outside the FP32 range take the
// FP64 fallback for both products.
template <bool ATOMIC, bool STRUCT>
__global__ void __launch_bounds__(256, 2) stored_apply_df_both(
    const float4 *__restrict__ Ahi, const float4 *__restrict__ Alo,
    const ConnView cv, int E, int p0, int p1,
    const double *__restrict__ x1, double *__restrict__ y1,
    const double *__restrict__ x2, double *__restrict__ y2, const int *skip) {
  if (skip && *(volatile const int *)skip) return;
  for (long p = p0 + (long)blockIdx.x * blockDim.x + threadIdx.x; p < p1;
       p += (long)gridDim.x * blockDim.x) {
    ElemNodes<STRUCT> c;
    float ah[8], al[8], bh[8], bl[8];
    bool bad = false;
    int sa, sb;
    {
      double va[8], vb[8];
      int ea = 0, eb = 0;
      c.load(cv, E, p);
#pragma unroll
      for (int s = 0; s < 8; s++) {
        va[s] = c[s] < 0 ? 0.0 : __ldg(x1 + c[s]);
        vb[s] = c[s] < 0 ? 0.0 : __ldg(x2 + c[s]);
        ea = max(ea, df_exp(va[s]));
        eb = max(eb, df_exp(vb[s]));
      }
      sa = ea - 1023;
      sb = eb - 1023;
#pragma unroll
      for (int s = 0; s < 8; s++) {
        df_split(va[s], ah[s], al[s], bad, sa);
        df_split(vb[s], bh[s], bl[s], bad, sb);
      }
    }
    if (bad) {
      df_element_fallback(Ahi, Alo, c, E, p, false, ATOMIC, x1, y1);
      df_element_fallback(Ahi, Alo, c, E, p, true, ATOMIC, x2, y2);
      continue;
    }
    DfAcc acc2[8];
#pragma unroll
    for (int j = 0; j < 8; j++) acc2[j] = DfAcc{0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const float4 h0 = __ldcs(Ahi + (size_t)(2 * i) * E + p);
      const float4 h1 = __ldcs(Ahi + (size_t)(2 * i + 1) * E + p);
      const float4 l0 = __ldcs(Alo + (size_t)(2 * i) * E + p);
      const float4 l1 = __ldcs(Alo + (size_t)(2 * i + 1) * E + p);
      DfAcc acc{0.0f, 0.0f};
      df_fma_acc(acc, h0.x, l0.x, ah[0], al[0]);
      df_fma_acc(acc, h0.y, l0.y, ah[1], al[1]);
      df_fma_acc(acc, h0.z, l0.z, ah[2], al[2]);
      df_fma_acc(acc, h0.w, l0.w, ah[3], al[3]);
      df_fma_acc(acc, h1.x, l1.x, ah[4], al[4]);
      df_fma_acc(acc, h1.y, l1.y, ah[5], al[5]);
      df_fma_acc(acc, h1.z, l1.z, ah[6], al[6]);
      df_fma_acc(acc, h1.w, l1.w, ah[7], al[7]);
      df_fma_acc(acc2[0], h0.x, l0.x, bh[i], bl[i]);
      df_fma_acc(acc2[1], h0.y, l0.y, bh[i], bl[i]);
      df_fma_acc(acc2[2], h0.z, l0.z, bh[i], bl[i]);
      df_fma_acc(acc2[3], h0.w, l0.w, bh[i], bl[i]);
      df_fma_acc(acc2[4], h1.x, l1.x, bh[i], bl[i]);
      df_fma_acc(acc2[5], h1.y, l1.y, bh[i], bl[i]);
      df_fma_acc(acc2[6], h1.z, l1.z, bh[i], bl[i]);
      df_fma_acc(acc2[7], h1.w, l1.w, bh[i], bl[i]);
      double o = df_to_double(acc.s, acc.c);
      if (!df_scale(o, sa)) o = ldexp(o, sa);
      if (c[i] >= 0) {
        if (ATOMIC)
          atomicAdd(y1 + c[i], o);
        else
          y1[c[i]] += o;
      }
    }
#pragma unroll
    for (int j = 0; j < 8; j++) {
      double o = df_to_double(acc2[j].s, acc2[j].c);
      if (!df_scale(o, sb)) o = ldexp(o, sb);
      if (c[j] >= 0) {
        if (ATOMIC)
          atomicAdd(y2 + c[j], o);
        else
          y2[c[j]] += o;
      }
    }
  }
}

// Reference BB (BB[64e + 8i + j], sklad_wd) -> pair store A64[(4i+j/2)*E+e];
// reference ISS (iss(E,8) column-major, 1-based) -> masked 0-based conn.
__global__ void legacy_convert_kernel(const double2 *__restrict__ bb, int E,
                                      double2 *__restrict__ A) {
  const long total = (long)E * 32;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t >> 5;
    const int k = (int)(t & 31);
    A[(size_t)k * E + e] = bb[t];
  }
}

// Reference BB -> double-float store Ahi/Alo[(2i + j/4)*E + e] (chunk c =
// 2i + j/4 holds BB[64e + 4c .. 4c+3]).  Entries outside the store window
// (nonzero with magnitude outside [2^-100, 2^120], inf, NaN) set bit 2 of
// *bad: the caller then uses the FP64 store.
__global__ void legacy_convert_df_kernel(const double *__restrict__ bb, int E,
                                         float4 *__restrict__ Ahi,
                                         float4 *__restrict__ Alo, int *bad) {
  const long total = (long)E * 16;
  bool out = false;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t >> 4;
    const int c = (int)(t & 15);
    const double2 v0 = __ldg(reinterpret_cast<const double2 *>(bb) + 2 * t);
    const double2 v1 = __ldg(reinterpret_cast<const double2 *>(bb) + 2 * t + 1);
    const double v[4] = {v0.x, v0.y, v1.x, v1.y};
    float hi[4], lo[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int ex = df_exp(v[k]);
      if (ex != 0 && (ex < 1023 - 100 || ex > 1023 + 120)) out = true;
      df_split(v[k], hi[k], lo[k], out);
    }
    Ahi[(size_t)c * E + e] = make_float4(hi[0], hi[1], hi[2], hi[3]);
    Alo[(size_t)c * E + e] = make_float4(lo[0], lo[1], lo[2], lo[3]);
  }
  if (out) atomicOr(bad, 2);
}

// Element matrices -> the reference's BB layout, FP64: BB[64 e + 8i + j] =
// A_e(i,j), e the caller's element at storage position p (perm, or the
// identity).  Chunk c = 2i + j/4 of a storage element holds entries
// 8i + 4(j/4) .. +3 = 4c .. 4c+3 (double-float or FP64 pair store).
__global__ void export_bb_kernel(const float4 *__restrict__ Ahi,
                                 const float4 *__restrict__ Alo,
                                 const double2 *__restrict__ A64,
                                 const int *__restrict__ perm, int E,
                                 double *__restrict__ bb) {
  const long total = (long)E * 16;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long p = t >> 4;
    const int c = (int)(t & 15);
    const long e = perm ? __ldg(perm + p) : p;
    double2 v0, v1;
    if (Ahi) {
      const float4 h = Ahi[(size_t)c * E + p], l = Alo[(size_t)c * E + p];
      v0 = make_double2(df_to_double(h.x, l.x), df_to_double(h.y, l.y));
      v1 = make_double2(df_to_double(h.z, l.z), df_to_double(h.w, l.w));
    } else {
      v0 = A64[(size_t)(2 * c) * E + p];
      v1 = A64[(size_t)(2 * c + 1) * E + p];
    }
    double2 *o = reinterpret_cast<double2 *>(bb + 64 * e + 4 * c);
    o[0] = v0;
    o[1] = v1;
  }
}

__global__ void legacy_conn_kernel(const int *__restrict__ iss, int E, int N,
                                   const int *__restrict__ bc,
                                   int *__restrict__ conn, int *bad) {
  const long total = (long)E * 8;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const int n = iss[t] - 1;
    if (n < 0 || n >= N) {
      atomicOr(bad, 1);
      conn[t] = MASK_BIT;  // node 0, masked: never read or written
      continue;
    }
    conn[t] = (bc && bc[n] == 1) ? (n | MASK_BIT) : n;
  }
}

__global__ void mask_conn_kernel(int *__restrict__ conn, long total,
                                 const unsigned char *__restrict__ mask) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const int n = conn[t] & NODE_BITS;
    conn[t] = mask[n] ? (n | MASK_BIT) : n;
  }
}

// Per-element Dirichlet bits from the connectivity table's flags.
__global__ void emask_kernel(const int *__restrict__ conn, int E,
                             unsigned char *__restrict__ emask) {
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < E;
       p += (long)gridDim.x * blockDim.x) {
    unsigned m = 0u;
#pragma unroll
    for (int s = 0; s < 8; s++)
      if (__ldg(conn + (size_t)s * E + p) < 0) m |= 1u << s;
    emask[p] = (unsigned char)m;
  }
}

__global__ void diag_fix_kernel(double *__restrict__ d, double *__restrict__ dinv,
                                const unsigned char *__restrict__ m, int N) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long)gridDim.x * blockDim.x) {
    double di = d[i];
    if (m && m[i]) {
      di = 1.0;
      d[i] = di;
    }
    dinv[i] = 1.0 / di;
  }
}

__global__ void mask_vec_kernel(double *__restrict__ v,
                                const unsigned char *__restrict__ m, int N) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long)gridDim.x * blockDim.x)
    if (m[i]) v[i] = 0.0;
}

// v = 0 on masked entries; *all_zero = 0 if any entry stays nonzero (every
// writer stores the same 0).
__global__ void mask_vec_flag_kernel(double *__restrict__ v,
                                     const unsigned char *__restrict__ m, int N,
                                     int *all_zero) {
  bool nz = false;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long)gridDim.x * blockDim.x) {
    if (m && m[i])
      v[i] = 0.0;
    else if (v[i] != 0.0)
      nz = true;
  }
  if (__syncthreads_or(nz) && threadIdx.x == 0) *all_zero = 0;
}

__global__ void bc_to_mask_kernel(const int *__restrict__ bc,
                                  unsigned char *__restrict__ m, int N) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long)gridDim.x * blockDim.x)
    m[i] = bc[i] == 1 ? 1 : 0;
}

int grid_for(long n, int threads, int per_sm) {
  const long need = (n + threads - 1) / threads;
  return (int)std::max<long>(1, std::min<long>(need, (long)device_sm_count() * per_sm));
}

}  // namespace

cudaError_t launch_stored_apply32v(const Handle &h, const float *x, float *y,
                                   const int *skip, const int *skip2,
                                   cudaStream_t s) {
  const bool color = h.scatter == VDR_SCATTER_COLOR;
  const ConnView cv = conn_view(h);
  const int nranges = color ? h.ncolors : 1;
  for (int r = 0; r < nranges; r++) {
    const int p0 = color ? h.color_off[r] : 0;
    const int p1 = color ? h.color_off[r + 1] : h.E;
    if (p1 <= p0) continue;
    const int grid = grid_for(p1 - p0, 256, h.apply_per_sm);
    if (color)
      stored_apply_f32v<false, false><<<grid, 256, 0, s>>>(h.A32v, cv, h.E, p0, p1, x, y,
                                                           skip, skip2);
    else if (cv.emask)
      stored_apply_f32v<true, true><<<grid, 256, 0, s>>>(h.A32v, cv, h.E, p0, p1, x, y,
                                                         skip, skip2);
    else
      stored_apply_f32v<true, false><<<grid, 256, 0, s>>>(h.A32v, cv, h.E, p0, p1, x, y,
                                                          skip, skip2);
    count_launches(1);
  }
  return cudaGetLastError();
}

bool can_apply_both(const Handle &h) {
  return h.apply_mode == VDR_APPLY_STORED && !h.apply_fp32 &&
         h.storage == VDR_STORE_DF && h.Ahi && h.Alo;
}

cudaError_t launch_apply_both(const Handle &h, const double *x1, double *y1,
                              const double *x2, double *y2, const int *skip,
                              cudaStream_t s) {
  const bool color = h.scatter == VDR_SCATTER_COLOR;
  const ConnView cv = conn_view(h);
  const int nranges = color ? h.ncolors : 1;
  for (int r = 0; r < nranges; r++) {
    const int p0 = color ? h.color_off[r] : 0;
    const int p1 = color ? h.color_off[r + 1] : h.E;
    if (p1 <= p0) continue;
    const int grid = grid_for(p1 - p0, 256, 6);
    // the connectivity table, as the double-float single apply reads it
    if (color)
      stored_apply_df_both<false, false><<<grid, 256, 0, s>>>(h.Ahi, h.Alo, cv, h.E, p0,
                                                              p1, x1, y1, x2, y2, skip);
    else
      stored_apply_df_both<true, false><<<grid, 256, 0, s>>>(h.Ahi, h.Alo, cv, h.E, p0,
                                                             p1, x1, y1, x2, y2, skip);
    count_launches(1);
  }
  return cudaGetLastError();
}

namespace {
// b = cf F - a1 y1 + a2 y2 (y1 = A T, y2 = M T; F, y1, y2 are zero on
// Dirichlet nodes, so b is too).
__global__ void rhs_combine_kernel(const double *__restrict__ F,
                                   const double *__restrict__ y1,
                                   const double *__restrict__ y2, double cf,
                                   double a1, double a2, double *__restrict__ b,
                                   long N) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long)gridDim.x * blockDim.x)
    b[i] = cf * F[i] - a1 * y1[i] + a2 * y2[i];
}
}  // namespace

cudaError_t launch_rhs_from_mass(Handle &h, double cf, double rM, const double *t,
                                 double *b, cudaStream_t s) {
  // H - rM M = A/aH - (aM/aH + rM) M
  double *y1 = h.rhs_tmp, *y2 = h.rhs_tmp + h.N;
  cudaError_t e;
  if ((e = cudaMemsetAsync(h.rhs_tmp, 0, sizeof(double) * 2 * (size_t)h.N, s))) return e;
  if ((e = launch_apply(h, false, t, y1, nullptr, nullptr, s))) return e;
  const bool color = h.scatter == VDR_SCATTER_COLOR;
  const ConnView cv = conn_view(h);
  const int nranges = color ? h.ncolors : 1;
  for (int r = 0; r < nranges; r++) {
    const int p0 = color ? h.color_off[r] : 0;
    const int p1 = color ? h.color_off[r + 1] : h.E;
    if (p1 <= p0) continue;
    const int grid = grid_for(p1 - p0, 256, 8);
    if (color)
      stored_apply_df<false, false, false><<<grid, 256, 0, s>>>(
          h.Mhi, h.Mlo, cv, h.E, p0, p1, t, y2, nullptr, nullptr, ElemGate{});
    else
      stored_apply_df<false, true, false><<<grid, 256, 0, s>>>(
          h.Mhi, h.Mlo, cv, h.E, p0, p1, t, y2, nullptr, nullptr, ElemGate{});
    count_launches(1);
  }
  rhs_combine_kernel<<<grid_for(h.N, 256, 8), 256, 0, s>>>(
      h.Fvec, y1, y2, cf, 1.0 / h.aH, h.aM / h.aH + rM, b, h.N);
  count_launches(1);
  return cudaGetLastError();
}

int apply_launches(const Handle &h) {
  if (h.apply_mode == VDR_APPLY_MATRIX_FREE || h.scatter != VDR_SCATTER_COLOR)
    return 1;
  int n = 0;
  for (int r = 0; r < h.ncolors; r++) n += h.color_off[r + 1] > h.color_off[r];
  return n;
}

cudaError_t launch_stored_apply(const Handle &h, bool fp32, bool transpose,
                                const double *x, double *y, const int *skip,
                                const int *skip2, cudaStream_t s) {
  const bool color = h.scatter == VDR_SCATTER_COLOR;
  const ConnView cv = conn_view(h);
  const int nranges = color ? h.ncolors : 1;
  for (int r = 0; r < nranges; r++) {
    const int p0 = color ? h.color_off[r] : 0;
    const int p1 = color ? h.color_off[r + 1] : h.E;
    if (p1 <= p0) continue;
    const int grid = grid_for(p1 - p0, 256, h.apply_per_sm);
#define VDR_LAUNCH(K, AP)                                                     \
  K<<<grid, 256, 0, s>>>(AP, h.conn, h.E, p0, p1, x, y, skip, skip2)
    if (!fp32 && h.storage == VDR_STORE_DF) {
#define VDR_LAUNCH_DF(K)                                                      \
  K<<<grid, 256, 0, s>>>(h.Ahi, h.Alo, cv, h.E, p0, p1, x, y, skip, skip2,      \
                         ElemGate{h.gate_eseg, h.gate_active})
      // The double-float apply reads the connectivity table even on the
      // structured numbering: without its 32 B per element the kernel kept
      // the same time (0.782 vs 0.786 ms at 8.4M elements) -- fewer bytes in
      // flight per element, lower bandwidth -- while the FP32 applies gain.
      if (h.warp_agg && cv.emask) {
        if (transpose) VDR_LAUNCH_DF((stored_apply_df_warp<true>));
        else VDR_LAUNCH_DF((stored_apply_df_warp<false>));
      } else if (transpose) {
        if (color) VDR_LAUNCH_DF((stored_apply_df<true, false, false>));
        else VDR_LAUNCH_DF((stored_apply_df<true, true, false>));
      } else {
        if (color) VDR_LAUNCH_DF((stored_apply_df<false, false, false>));
        else VDR_LAUNCH_DF((stored_apply_df<false, true, false>));
      }
#undef VDR_LAUNCH_DF
    } else if (!fp32) {
      if (transpose) {
        if (color) VDR_LAUNCH((stored_apply_f64<true, false>), h.A64);
        else VDR_LAUNCH((stored_apply_f64<true, true>), h.A64);
      } else {
        if (color) VDR_LAUNCH((stored_apply_f64<false, false>), h.A64);
        else VDR_LAUNCH((stored_apply_f64<false, true>), h.A64);
      }
    } else {
      if (transpose) {
        if (color) VDR_LAUNCH((stored_apply_f32<true, false>), h.A32v);
        else VDR_LAUNCH((stored_apply_f32<true, true>), h.A32v);
      } else {
        if (color) VDR_LAUNCH((stored_apply_f32<false, false>), h.A32v);
        else VDR_LAUNCH((stored_apply_f32<false, true>), h.A32v);
      }
    }
#undef VDR_LAUNCH
    count_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_legacy_bb(const double *bb_ref, int E, double2 *A64,
                             cudaStream_t s) {
  legacy_convert_kernel<<<grid_for((long)E * 32, 256, 16), 256, 0, s>>>(
      reinterpret_cast<const double2 *>(bb_ref), E, A64);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_legacy_bb_df(const double *bb_ref, int E, float4 *Ahi, float4 *Alo,
                                int *bad, cudaStream_t s) {
  legacy_convert_df_kernel<<<grid_for((long)E * 16, 256, 16), 256, 0, s>>>(
      bb_ref, E, Ahi, Alo, bad);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_export_bb(const Handle &h, double *bb, cudaStream_t s) {
  const bool df = h.storage == VDR_STORE_DF && h.Ahi;
  const int *perm = h.scatter == VDR_SCATTER_COLOR ? h.perm_d : nullptr;
  export_bb_kernel<<<grid_for((long)h.E * 16, 256, 16), 256, 0, s>>>(
      df ? h.Ahi : nullptr, df ? h.Alo : nullptr, df ? nullptr : h.A64, perm, h.E, bb);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_legacy_conn(const int *iss_ref, int E, int N, const int *bc,
                               int *conn, int *bad, cudaStream_t s) {
  legacy_conn_kernel<<<grid_for((long)E * 8, 256, 16), 256, 0, s>>>(
      iss_ref, E, N, bc, conn, bad);
  count_launches(1);
  return cudaGetLastError();
}

ConnView conn_view(const Handle &h) {
  ConnView v;
  v.conn = h.conn;
  if (h.emask && h.nax > 1 && h.nay > 1 && h.naz > 1 && !h.perm_d &&
      h.scatter != VDR_SCATTER_COLOR) {
    v.emask = h.emask;
    v.nex = h.nax - 1;
    v.ney = h.nay - 1;
    v.nax = h.nax;
    v.pl = h.nax * h.nay;
  }
  return v;
}

// The per-element Dirichlet bits of a mesh in the canonical structured
// numbering (natural order), rebuilt with every operator build so that
// they follow vdr_set_dirichlet.
cudaError_t launch_emask(Handle &h) {
  if (!(h.nax > 1 && h.nay > 1 && h.naz > 1) || h.perm_d ||
      h.scatter == VDR_SCATTER_COLOR || !h.conn)
    return cudaSuccess;
  cudaError_t e;
  if (!h.emask && (e = cudaMalloc(&h.emask, (size_t)h.E))) return e;
  emask_kernel<<<grid_for(h.E, 256, 8), 256, 0, h.stream>>>(h.conn, h.E, h.emask);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mask_conn(int *conn, int E, const unsigned char *mask,
                             cudaStream_t s) {
  mask_conn_kernel<<<grid_for((long)E * 8, 256, 16), 256, 0, s>>>(
      conn, (long)E * 8, mask);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_diag_fix(double *diag, double *dinv,
                            const unsigned char *mask, int N, cudaStream_t s) {
  diag_fix_kernel<<<grid_for(N, 256, 8), 256, 0, s>>>(diag, dinv, mask, N);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mask_vec_flag(double *v, const unsigned char *mask, int N,
                                 int *all_zero, cudaStream_t s) {
  mask_vec_flag_kernel<<<grid_for(N, 256, 8), 256, 0, s>>>(v, mask, N, all_zero);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_mask_vec(double *v, const unsigned char *mask, int N,
                            cudaStream_t s) {
  mask_vec_kernel<<<grid_for(N, 256, 8), 256, 0, s>>>(v, mask, N);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_bc_to_mask(const int *bc, unsigned char *mask, int N,
                              cudaStream_t s) {
  bc_to_mask_kernel<<<grid_for(N, 256, 8), 256, 0, s>>>(bc, mask, N);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_apply(const Handle &h, bool transpose, const double *x,
                         double *y, const int *skip, const int *skip2,
                         cudaStream_t s) {
  if (h.apply_mode == VDR_APPLY_MATRIX_FREE)
    return launch_mf_apply(op_args(h), h.apply_fp32, transpose, x, y, skip, skip2, s);
  return launch_stored_apply(h, h.apply_fp32, transpose, x, y, skip, skip2, s);
}

}  // namespace vdr
