// unet.cu -- the learned preconditioner.
//
// A 3-level 3D U-Net on the structured nodal grid (x fastest, the
// reference's node numbering), channels 16 / 32 / 64, 3x3x3 convolutions
// with zero padding, ReLU, 2x2x2 average pooling (partial cells at odd
// edges average the children that exist), nearest upsampling, skip
// concatenation, and a 1x1 head to one channel.  Activations and weights
// are BF16, accumulation FP32; training keeps FP32 master weights (Adam).
//
// Input channels (padded to 16): residual r / rms(r), nodal u_x, u_y, u_z
// (element velocities averaged over the elements sharing the node) and
// ln(lambda) - ln(1e-4) (averaged the same way).  As a right
// preconditioner the network corrects Jacobi:
//   M(r) = D^-1 r + (rms(r) / dbar) * net(r / rms(r), features)
// with dbar the mean assembled diagonal over free nodes, zero on Dirichlet
// nodes; an untrained (zero-output) network is plain Jacobi.  It is
// trained on pairs (r_k, e_k) = (b - A x_k, x* - x_k) of the solver's own
// iterates, target (e - D^-1 r) dbar / rms(r), relative squared error over
// free nodes.
//
// Kernels:
//   conv3_kernel   implicit GEMM on the tensor cores (mma.sync m16n8k16
//                  BF16, FP32 accumulate): M = 16-voxel x-row segments, N =
//                  output channels, K = 27 taps x input channels, the A
//                  operand staged per (dy, dz) row in shared memory and read
//                  by ldmatrix for the three x-taps (the wide layers' weights
//                  staged the same way).  The nearest upsampling and
//                  concatenation of the decoder inputs are fused into the
//                  operand staging.  The same kernel computes the backward
//                  data pass (flipped, transposed weights; FP32 gradient
//                  input with the ReLU mask of the layer output fused into
//                  the staging).
//   conv3_wgrad_tc weight and bias gradients on mma.sync, K = voxels: per
//                  (dy, dz) pair an 18-voxel row segment of the inputs
//                  staged in shared memory serves the three x-taps (B by
//                  ldmatrix.trans), the masked output gradient transposed
//                  into x rows padded to 16 voxels (A); FP32 atomics.
//   conv3_tc_kernel (conv_tc.cuh) the forward convolutions on the fifth-
//                  generation tensor cores: tcgen05.mma from TMA-staged
//                  halo slabs into tensor memory (VDR_NET_CONV_TCGEN05,
//                  the default where the tensor maps can be made); the
//                  decoder's upsampled input is first copied to the fine
//                  grid (upsample_bf16).
//   pooling, head, loss, Adam, BF16 packing, features, normalisation.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "conv_tc.cuh"
#include "vdr_internal.h"

namespace vdr {
namespace {

typedef __nv_bfloat16 bf16;
constexpr unsigned FULLM = 0xffffffffu;

enum { L_E0A, L_E0B, L_E1A, L_E1B, L_BTA, L_BTB, L_D1A, L_D1B, L_D0A, L_D0B,
       L_HEAD, NLAYER };
struct LayerDef {
  int cin1, cin2, cout, level;
};
// d1a / d0a read [skip | upsampled coarser output]; the head is 1x1.
constexpr LayerDef DEFS[NLAYER] = {
    {16, 0, 16, 0},  {16, 0, 16, 0}, {16, 0, 32, 1}, {32, 0, 32, 1},
    {32, 0, 64, 2},  {64, 0, 64, 2}, {32, 64, 32, 1}, {32, 0, 32, 1},
    {16, 32, 16, 0}, {16, 0, 16, 0}, {16, 0, 1, 0}};
constexpr int IN_REAL = 5;  // real input channels of layer 0 (of 16)

constexpr long layer_wsize(int l) {
  return l == L_HEAD ? 16 : 27L * DEFS[l].cout * (DEFS[l].cin1 + DEFS[l].cin2);
}

int grid_for(long n, int threads, int per_sm = 8) {
  const long need = (n + threads - 1) / threads;
  return (int)std::max<long>(1, std::min<long>(need, (long)device_sm_count() * per_sm));
}

__device__ __forceinline__ bool skipped(const int *s1, const int *s2) {
  return (s1 && *(volatile const int *)s1) || (s2 && *(volatile const int *)s2);
}

// ------------------------------------------------------------ BF16 pairs
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }
__device__ __forceinline__ bool bf_pos(uint32_t h16) {  // bf16 bits > 0
  return !(h16 & 0x8000u) && (h16 & 0x7fffu);
}
__device__ __forceinline__ uint32_t ld2(const bf16 *p) {
  return *reinterpret_cast<const uint32_t *>(p);
}
template <bool F32>
__device__ __forceinline__ uint32_t ld_pair(const void *base, long i) {
  if (F32) {
    const float2 v = *reinterpret_cast<const float2 *>(static_cast<const float *>(base) + i);
    return pack2(v.x, v.y);
  }
  return ld2(static_cast<const bf16 *>(base) + i);
}
__device__ __forceinline__ uint32_t apply_mask(uint32_t v, uint32_t m) {
  return (bf_pos(m & 0xffffu) ? (v & 0xffffu) : 0u) |
         (bf_pos(m >> 16) ? (v & 0xffff0000u) : 0u);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1,
                                         uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ------------------------------------------------------- convolution
struct ConvArgs {
  const void *in1;    // [V][CIN1] (BF16, or FP32 for the backward pass)
  const bf16 *mask1;  // [V][CIN1] or null: in1 used only where mask1 > 0
  const bf16 *in2;    // [Vc][CIN2] coarser level, read upsampled, or null
  const bf16 *w;      // [27][COUT][CIN]
  const float *bias;  // [COUT] or null
  void *out;          // [V][COUT] (BF16, or FP32)
  int W, H, D, Wc, Hc;
  long V;
  int relu;
  const int *skip, *skip2;
};

// Four 8x8 b16 matrices from shared memory (ldmatrix): lane l supplies the
// address of row l & 7 of matrix l >> 3.
__device__ __forceinline__ void ldsm_x4(const bf16 *p, uint32_t &r0, uint32_t &r1,
                                        uint32_t &r2, uint32_t &r3) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(sa)
               : "memory");
}

// 3x3x3 convolution by x-row segments: out[v][co] = bias + sum over taps
// t = (dz+1)*9 + (dy+1)*3 + (dx+1) of W[t][co][.] . X[v + off(t)][.],
// X = [in1 (zero where mask1 <= 0) | up(in2)].  A warp takes MS segments of
// 16 voxels of x rows (MS m-tiles), the block's four warps four such groups
// together.  For each (dy, dz) pair each warp copies the 18 voxels
// xs-1 .. xs+16 of the shifted row of each of its segments into a padded
// shared tile (BF16; FP32 inputs converted; zero outside the volume), and
// the three x-taps read their A fragments from tile rows dx+1 .. dx+16 with
// ldmatrix.  With one m-tile per warp (the wide layers) the block also
// copies the pair's three taps of weights into shared memory and the B
// fragments come from there by ldmatrix; with two, the m-tiles share 32-bit
// weight loads through L1 (measured faster for those layers).
template <int CIN1, int CIN2, int COUT, int MS, bool F32IN, bool F32OUT>
__global__ void __launch_bounds__(128) conv3_kernel(ConvArgs a) {
  if (skipped(a.skip, a.skip2)) return;
  constexpr int CIN = CIN1 + CIN2, KC = CIN / 16, NT = COUT / 8;
  static_assert(CIN1 % 16 == 0 && CIN2 % 16 == 0 && COUT % 16 == 0, "shape");
  constexpr int RSTR = CIN + 8;  // bf16 per tile / weight row (16 bytes of padding)
  constexpr int UNITS = CIN / 8, ITEMS = MS * 18 * UNITS, PER_LANE = (ITEMS + 31) / 32;
  constexpr bool WSM = MS == 1;              // weights staged in shared memory
  constexpr int WUNITS = 3 * COUT * UNITS;  // 16-byte units of a pair's weights
  __shared__ __align__(16) bf16 tile[4][MS * 18 * RSTR];
  __shared__ __align__(16) bf16 wsm[WSM ? 3 * COUT * RSTR : 8];  // [tx][co][ci]
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, warp = threadIdx.x >> 5;
  bf16 *tw = tile[warp];
  const int W = a.W, H = a.H, D = a.D;
  const int segs = (W + 15) >> 4;
  const long nseg = (long)H * D * segs;
  const long ngroup = (nseg + MS - 1) / MS;
  for (long bgi = blockIdx.x; bgi * 4 < ngroup; bgi += gridDim.x) {
    // segment m of this warp's group: flat segment MS gi + m = (row, xs)
    const long gi = bgi * 4 + warp;
    long rowm[MS];
    int xsm[MS], ym[MS], zm[MS];
    bool segok[MS];
#pragma unroll
    for (int m = 0; m < MS; m++) {
      const long sg = MS * gi + m;
      segok[m] = sg < nseg;
      const long sgc = segok[m] ? sg : 0;
      rowm[m] = sgc / segs;
      xsm[m] = (int)(sgc - rowm[m] * segs) << 4;
      ym[m] = (int)(rowm[m] % H);
      zm[m] = (int)(rowm[m] / H);
    }
    float acc[MS][NT][4];
#pragma unroll
    for (int m = 0; m < MS; m++)
#pragma unroll
      for (int nt = 0; nt < NT; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[m][nt][q] = 0.f;
#pragma unroll 1
    for (int pair = 0; pair < 9; pair++) {
      const int dyy = pair % 3 - 1, dz = pair / 3 - 1;
      if constexpr (WSM) {
        __syncthreads();  // every warp has read the previous pair's weights and tile
        const bf16 *wsrc = a.w + (size_t)3 * pair * COUT * CIN;  // taps 3 pair .. + 2
        for (int u = threadIdx.x; u < WUNITS; u += blockDim.x) {
          const int rowc = u / UNITS, c8 = (u - rowc * UNITS) * 8;  // row = tx COUT + co
          *reinterpret_cast<uint4 *>(wsm + rowc * RSTR + c8) =
              *reinterpret_cast<const uint4 *>(wsrc + (size_t)rowc * CIN + c8);
        }
      } else {
        __syncwarp();  // the previous pair's ldmatrix reads of the tile are done
      }
#pragma unroll
      for (int k = 0; k < PER_LANE; k++) {
        const int idx = lane + 32 * k;
        if (idx >= ITEMS) break;
        const int m = idx / (18 * UNITS), rem = idx - m * 18 * UNITS;
        const int r = rem / UNITS, ch = (rem - r * UNITS) * 8;
        const int x = xsm[m] - 1 + r, yn = ym[m] + dyy, zn = zm[m] + dz;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (segok[m] && x >= 0 && x < W && yn >= 0 && yn < H && zn >= 0 && zn < D) {
          if (ch < CIN1) {
            const long i = ((long)W * (yn + (long)H * zn) + x) * CIN1 + ch;
            if (F32IN) {
              const float4 f0 = *reinterpret_cast<const float4 *>(static_cast<const float *>(a.in1) + i);
              const float4 f1 =
                  *reinterpret_cast<const float4 *>(static_cast<const float *>(a.in1) + i + 4);
              v = make_uint4(pack2(f0.x, f0.y), pack2(f0.z, f0.w), pack2(f1.x, f1.y),
                             pack2(f1.z, f1.w));
            } else {
              v = *reinterpret_cast<const uint4 *>(static_cast<const bf16 *>(a.in1) + i);
            }
            if (a.mask1) {
              const uint4 mk = *reinterpret_cast<const uint4 *>(a.mask1 + i);
              v = make_uint4(apply_mask(v.x, mk.x), apply_mask(v.y, mk.y),
                             apply_mask(v.z, mk.z), apply_mask(v.w, mk.w));
            }
          } else if (CIN2 > 0) {
            v = *reinterpret_cast<const uint4 *>(
                a.in2 +
                ((long)(x >> 1) + (long)a.Wc * ((yn >> 1) + (long)a.Hc * (zn >> 1))) *
                    (CIN2 > 0 ? CIN2 : 1) +
                (ch - CIN1));
          }
        }
        *reinterpret_cast<uint4 *>(tw + (m * 18 + r) * RSTR + ch) = v;
      }
      if constexpr (WSM)
        __syncthreads();  // the weights and this warp's tile are in place
      else
        __syncwarp();
      const int mi = lane >> 3;  // ldmatrix matrix of this lane's address
#pragma unroll
      for (int tx = 0; tx < 3; tx++) {
#pragma unroll
        for (int kc = 0; kc < KC; kc++) {
          // B: matrices (n-tile nt, k 0-7), (nt, k 8-15), (nt+1, k 0-7), (nt+1, k 8-15)
          uint32_t bfr[NT][2];
          if constexpr (WSM) {
#pragma unroll
            for (int nt = 0; nt < NT; nt += 2)
              ldsm_x4(wsm + (tx * COUT + (nt + (mi >> 1)) * 8 + (lane & 7)) * RSTR + kc * 16 +
                          (mi & 1) * 8,
                      bfr[nt][0], bfr[nt][1], bfr[nt + 1][0], bfr[nt + 1][1]);
          } else {
            const bf16 *wt = a.w + (size_t)(3 * pair + tx) * COUT * CIN;
#pragma unroll
            for (int nt = 0; nt < NT; nt++) {
              const bf16 *wp = wt + (size_t)(nt * 8 + g) * CIN + kc * 16 + 2 * t;
              bfr[nt][0] = ld2(wp);
              bfr[nt][1] = ld2(wp + 8);
            }
          }
#pragma unroll
          for (int m = 0; m < MS; m++) {
            uint32_t a0, a1, a2, a3;
            ldsm_x4(tw + (m * 18 + tx + (mi & 1) * 8 + (lane & 7)) * RSTR + kc * 16 + (mi >> 1) * 8,
                    a0, a1, a2, a3);
#pragma unroll
            for (int nt = 0; nt < NT; nt++)
              mma_bf16(acc[m][nt], a0, a1, a2, a3, bfr[nt][0], bfr[nt][1]);
          }
        }
      }
    }
    // D fragments: rows g, g + 8 (voxels xs + g, xs + g + 8), cols co = 8 nt + 2t, +1
#pragma unroll
    for (int m = 0; m < MS; m++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int x = xsm[m] + g + 8 * h;
        if (!segok[m] || x >= W) continue;
        const long r = rowm[m] * W + x;
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
          const int co = nt * 8 + 2 * t;
          float v0 = acc[m][nt][2 * h], v1 = acc[m][nt][2 * h + 1];
          if (a.bias) {
            v0 += a.bias[co];
            v1 += a.bias[co + 1];
          }
          if (a.relu) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
          }
          if (F32OUT) {
            *reinterpret_cast<float2 *>(static_cast<float *>(a.out) + r * COUT + co) =
                make_float2(v0, v1);
          } else {
            *reinterpret_cast<uint32_t *>(static_cast<bf16 *>(a.out) + r * COUT + co) =
                pack2(v0, v1);
          }
        }
      }
  }
}

// Weight and bias gradients of one 3x3x3 layer on the tensor cores:
// dW[tap][co][ci] += sum_v dY'[v][co] X[v + off(tap)][ci], an implicit GEMM
// with M = output channels, N = input channels, K = voxels (16 per MMA),
// X = [in1 | up(in2)].  dY' (the ReLU-masked output gradient) is first
// written transposed in BF16, dyt[co][row][x] with x rows padded to Wp, a
// multiple of 16 voxels (zero past W), so that A fragments load as aligned
// pairs of consecutive voxels; B fragments come from the shifted inputs
// staged in shared memory.  Grid: (voxel chunks, 9 (dy, dz) pairs, groups
// of NG input-channel tiles); a block's chunk is a range of 16-voxel x-row
// segments, each warp takes every fourth one, and the three x-taps of the
// pair share its staging and its A fragments; the tiles go to dW with
// atomics.  db accumulates in the centre-pair blocks.
struct WgArgs {
  const bf16 *in1, *in2;
  const bf16 *dyt;  // [COUT][H D][Wp]
  float *dw, *db;
  int W, H, D, Wc, Hc, Wp;
  long V, Vp, chunk;  // Vp = H D Wp
};

// dyt[c][row][x] = dY[v][c] where Y[v][c] > 0 (the ReLU's derivative), v =
// row W + x; zero in the rows' padding x in [W, Wp) (the buffer is shared
// by layers of other shapes).  One block per x row, one thread per padded
// voxel: its C channels in 16-byte loads, and per channel a coalesced store
// across the row.
template <int C>
__global__ void mask_transpose(const float *__restrict__ dy, const bf16 *__restrict__ y,
                               bf16 *__restrict__ dyt, int W, int Wp, long Vp) {
  static_assert(C % 8 == 0, "channels");
  const long row = blockIdx.x;
  for (int x = threadIdx.x; x < Wp; x += blockDim.x) {
    bf16 *out = dyt + row * Wp + x;
    if (x >= W) {
#pragma unroll
      for (int c = 0; c < C; c++) out[(long)c * Vp] = __float2bfloat16_rn(0.f);
      continue;
    }
    const long v = row * W + x;
    const float4 *dp = reinterpret_cast<const float4 *>(dy + v * C);
    const uint4 *yp = reinterpret_cast<const uint4 *>(y + v * C);
#pragma unroll
    for (int c8 = 0; c8 < C / 8; c8++) {
      const uint4 ym = yp[c8];
      const float4 d0 = dp[2 * c8], d1 = dp[2 * c8 + 1];
      const uint32_t yw[4] = {ym.x, ym.y, ym.z, ym.w};
      const float dv[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const uint32_t h16 = (k & 1) ? (yw[k >> 1] >> 16) : (yw[k >> 1] & 0xffffu);
        out[(long)(8 * c8 + k) * Vp] =
            __float2bfloat16_rn(__uint_as_float(h16 << 16) > 0.f ? dv[k] : 0.f);
      }
    }
  }
}

// Four 8x8 b16 matrices from shared memory, transposed (ldmatrix .trans):
// lane l supplies the address of row l & 7 of matrix l >> 3.
__device__ __forceinline__ void ldsm_x4_trans(const bf16 *p, uint32_t &r0, uint32_t &r1,
                                              uint32_t &r2, uint32_t &r3) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(sa)
               : "memory");
}

// Weight gradient of the three x-taps of one (dy, dz) pair:
// dW[tap][co][ci] = sum_v dY[co][v] X[v + off(tap)][ci] as MMAs with K =
// voxels.  A k-step is a 16-voxel segment of one x row; per k-step a warp
// copies the 18 voxels xs-1 .. xs+16 of the shifted row (zero outside the
// volume), NG units of 8 channels each (16-byte loads of channels-last
// rows), into a padded shared tile, and tap dx reads its B fragments from
// tile rows 1 + dx .. 16 + dx with ldmatrix .trans: one staging and one set
// of A fragments for three taps.  The next k-step's rows are loaded while
// the current one multiplies.
template <int CIN1, int CIN2, int COUT, int NG>
__global__ void __launch_bounds__(128) conv3_wgrad_tc(WgArgs a) {
  constexpr int CIN = CIN1 + CIN2, MT = COUT / 16, NT = CIN / 8;
  static_assert(COUT % 16 == 0 && CIN % 8 == 0 && CIN1 % 8 == 0 && NG % 2 == 0, "shape");
  // B tile per warp: 18 rows (voxels) x NG units, rows padded by one unit so
  // that the 8 rows of one ldmatrix matrix fall on distinct banks
  constexpr int RSTR = NG * 8 + 8;  // bf16 per row
  constexpr int TROWS = 18, ITEMS = TROWS * NG, PER_LANE = (ITEMS + 31) / 32;
  __shared__ __align__(16) bf16 tile[4][TROWS * RSTR];
  const int pair = blockIdx.y;  // 3 (dz + 1) + (dy + 1)
  const int dyy = pair % 3 - 1, dz = pair / 3 - 1;
  const int ntile0 = blockIdx.z * NG;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int warp = threadIdx.x >> 5;
  bf16 *tw = tile[warp];
  const int W = a.W, H = a.H, D = a.D;
  const int segs = a.Wp >> 4;  // 16-voxel segments per (padded) x row
  const long nks = (long)H * D * segs;
  const long ks0 = (long)blockIdx.x * a.chunk;
  const long ks1 = nks < ks0 + a.chunk ? nks : ks0 + a.chunk;
  float acc[3][MT][NG][4];
#pragma unroll
  for (int tx = 0; tx < 3; tx++)
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
      for (int j = 0; j < NG; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[tx][mt][j][q] = 0.f;
  float dbs[MT][2] = {};
  // the warp's k-step as (segment, y, z), advanced by 4 segments per step
  // without divisions
  long ks = ks0 + warp;
  int seg = 0, y = 0, z = 0;
  if (ks < ks1) {
    const long row = ks / segs;
    seg = (int)(ks - row * segs);
    y = (int)(row % H);
    z = (int)(row / H);
  }
  // the B rows of a k-step: item idx = lane + 32 k is tile row idx / NG
  // (input x = 16 sg - 1 + row), unit idx % NG of the group (zero outside
  // the volume and past CIN)
  auto load_rows = [&](int sg, int yy, int zz, uint4 (&sv)[PER_LANE]) {
    const int yn = yy + dyy, zn = zz + dz;
    const bool rowok = yn >= 0 && yn < H && zn >= 0 && zn < D;
    const long frow = (long)W * (yn + (long)H * zn);
    const long crow = (long)a.Wc * ((yn >> 1) + (long)a.Hc * (zn >> 1));
#pragma unroll
    for (int k = 0; k < PER_LANE; k++) {
      const int idx = lane + 32 * k;
      const int r = idx / NG, u = idx % NG;
      const int x = (sg << 4) - 1 + r, ch = (ntile0 + u) * 8;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (idx < ITEMS && rowok && x >= 0 && x < W && ch < CIN) {
        if (ch < CIN1)
          v = *reinterpret_cast<const uint4 *>(a.in1 + (frow + x) * CIN1 + ch);
        else if (CIN2 > 0)
          v = *reinterpret_cast<const uint4 *>(
              a.in2 + ((long)(x >> 1) + crow) * (CIN2 > 0 ? CIN2 : 1) + (ch - CIN1));
      }
      sv[k] = v;
    }
  };
  uint4 sv[PER_LANE];
  if (ks < ks1) load_rows(seg, y, z, sv);
  for (; ks < ks1; ks += 4) {
    // the k-step's first voxel in the padded gradient rows
    const long vb = ((long)y + (long)H * z) * a.Wp + ((long)seg << 4);
    __syncwarp();  // the previous k-step's ldmatrix reads are done
#pragma unroll
    for (int k = 0; k < PER_LANE; k++) {
      const int idx = lane + 32 * k;
      if (idx < ITEMS)
        *reinterpret_cast<uint4 *>(tw + (idx / NG) * RSTR + (idx % NG) * 8) = sv[k];
    }
    __syncwarp();
    seg += 4;
    while (seg >= segs) {
      seg -= segs;
      if (++y >= H) {
        y = 0;
        ++z;
      }
    }
    if (ks + 4 < ks1) load_rows(seg, y, z, sv);  // in flight during the MMAs
    // A fragments: dyt[co][vb + (2t, 2t+1)] and [vb + (2t+8, 2t+9)], aligned
    // pairs (zero in the rows' padding)
    uint32_t af[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
      for (int h = 0; h < 2; h++) {  // rows g, g+8
        const bf16 *rp = a.dyt + (long)(mt * 16 + g + 8 * h) * a.Vp + vb;
        const uint32_t lo = ld2(rp + 2 * t), hi = ld2(rp + 2 * t + 8);
        af[mt][h] = lo;      // a0 (row g) / a1 (row g+8): k = 2t, 2t+1
        af[mt][2 + h] = hi;  // a2 / a3: k = 2t+8, 2t+9
        if (pair == 4 && blockIdx.z == 0)
          dbs[mt][h] += bf_lo(lo) + bf_hi(lo) + bf_lo(hi) + bf_hi(hi);
      }
    // tap dx = tx - 1: B rows tx .. tx + 15; matrices (rows 0-7, j),
    // (rows 8-15, j), (rows 0-7, j+1), (rows 8-15, j+1)
#pragma unroll
    for (int tx = 0; tx < 3; tx++)
#pragma unroll
      for (int j = 0; j < NG; j += 2) {
        if (ntile0 + j >= NT) break;
        const int m = lane >> 3;
        uint32_t b0, b1, b2, b3;
        ldsm_x4_trans(tw + ((m & 1) * 8 + (lane & 7) + tx) * RSTR + (j + (m >> 1)) * 8, b0, b1,
                      b2, b3);
#pragma unroll
        for (int mt = 0; mt < MT; mt++)
          mma_bf16(acc[tx][mt][j], af[mt][0], af[mt][1], af[mt][2], af[mt][3], b0, b1);
        if (ntile0 + j + 1 < NT) {
#pragma unroll
          for (int mt = 0; mt < MT; mt++)
            mma_bf16(acc[tx][mt][j + 1], af[mt][0], af[mt][1], af[mt][2], af[mt][3], b2, b3);
        }
      }
  }
  // D fragments: rows co = g (c0, c1), g+8 (c2, c3); cols ci = 2t, 2t+1
#pragma unroll
  for (int tx = 0; tx < 3; tx++) {
    const int tap = 3 * pair + tx;
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
      for (int j = 0; j < NG; j++) {
        const int nt = ntile0 + j;
        if (nt >= NT) break;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int co = mt * 16 + g + 8 * (q >> 1), ci = nt * 8 + 2 * t + (q & 1);
          atomicAdd(a.dw + ((size_t)tap * COUT + co) * CIN + ci, acc[tx][mt][j][q]);
        }
      }
  }
  if (pair == 4 && blockIdx.z == 0) {
#pragma unroll
    for (int mt = 0; mt < MT; mt++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        float x = dbs[mt][h];
        x += __shfl_xor_sync(FULLM, x, 1);
        x += __shfl_xor_sync(FULLM, x, 2);
        if (t == 0) atomicAdd(a.db + mt * 16 + g + 8 * h, x);
      }
  }
}

// --------------------------------------------------------- pooling
struct Dims {
  int W, H, D;
  long V;
};
// Voxels of a level's transposed output gradient with x rows padded to 16.
inline long padded_rows(const Dims &f) { return (long)f.H * f.D * ((f.W + 15) & ~15); }
__host__ __device__ inline Dims coarse_of(const Dims &f) {
  Dims c;
  c.W = (f.W + 1) / 2;
  c.H = (f.H + 1) / 2;
  c.D = (f.D + 1) / 2;
  c.V = (long)c.W * c.H * c.D;
  return c;
}

__global__ void pool_fwd(const bf16 *in, bf16 *out, Dims f, Dims c, int C,
                         const int *skip, const int *skip2) {
  if (skipped(skip, skip2)) return;
  const long total = c.V * C;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int ch = (int)(idx % C);
    const long vc = idx / C;
    const int X = (int)(vc % c.W), Y = (int)((vc / c.W) % c.H),
              Z = (int)(vc / ((long)c.W * c.H));
    float s = 0.f;
    int cnt = 0;
    for (int k = 0; k < 2; k++)
      for (int j = 0; j < 2; j++)
        for (int i = 0; i < 2; i++) {
          const int x = 2 * X + i, y = 2 * Y + j, z = 2 * Z + k;
          if (x < f.W && y < f.H && z < f.D) {
            s += __bfloat162float(in[((long)x + (long)f.W * (y + (long)f.H * z)) * C + ch]);
            cnt++;
          }
        }
    out[idx] = __float2bfloat16_rn(s / (float)cnt);
  }
}

__device__ __forceinline__ int child_count(int X, int Y, int Z, const Dims &f) {
  return (2 * X + 1 < f.W ? 2 : 1) * (2 * Y + 1 < f.H ? 2 : 1) * (2 * Z + 1 < f.D ? 2 : 1);
}

// gf[v][c] += gc[parent(v)][c] / count(parent)
__global__ void pool_bwd_add(const float *gc, float *gf, Dims f, Dims c, int C) {
  const long total = f.V * C;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int ch = (int)(idx % C);
    const long v = idx / C;
    const int x = (int)(v % f.W), y = (int)((v / f.W) % f.H),
              z = (int)(v / ((long)f.W * f.H));
    const int X = x >> 1, Y = y >> 1, Z = z >> 1;
    const long P = (long)X + (long)c.W * (Y + (long)c.H * Z);
    gf[idx] += gc[P * C + ch] / (float)child_count(X, Y, Z, f);
  }
}

// Splits the gradient of a [skip | up(coarse)] input: gskip = first C1
// channels; gcoarse[P] = sum over the children of the last C2 channels.
__global__ void upcat_bwd_skip(const float *gcat, float *gskip, long V, int C1, int C2) {
  const long total = V * C1;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const long v = idx / C1;
    const int ch = (int)(idx % C1);
    gskip[idx] = gcat[v * (C1 + C2) + ch];
  }
}
__global__ void upcat_bwd_coarse(const float *gcat, float *gc, Dims f, Dims c,
                                 int C1, int C2) {
  const long total = c.V * C2;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long)gridDim.x * blockDim.x) {
    const int ch = (int)(idx % C2);
    const long vc = idx / C2;
    const int X = (int)(vc % c.W), Y = (int)((vc / c.W) % c.H),
              Z = (int)(vc / ((long)c.W * c.H));
    float s = 0.f;
    for (int k = 0; k < 2; k++)
      for (int j = 0; j < 2; j++)
        for (int i = 0; i < 2; i++) {
          const int x = 2 * X + i, y = 2 * Y + j, z = 2 * Z + k;
          if (x < f.W && y < f.H && z < f.D)
            s += gcat[((long)x + (long)f.W * (y + (long)f.H * z)) * (C1 + C2) + C1 + ch];
        }
    gc[idx] = s;
  }
}

// ---------------------------------------------------------- head / loss
__global__ void head_fwd(const bf16 *u0, const float *wh, float *c, long V,
                         const int *skip, const int *skip2) {
  if (skipped(skip, skip2)) return;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x) {
    float s = wh[16];
    const uint4 *p = reinterpret_cast<const uint4 *>(u0 + v * 16);
    const uint4 q0 = p[0], q1 = p[1];
    const uint32_t w8[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
    for (int k = 0; k < 8; k++)
      s += wh[2 * k] * bf_lo(w8[k]) + wh[2 * k + 1] * bf_hi(w8[k]);
    c[v] = s;
  }
}

// Relative loss L = sum_free (c - t)^2 / sum_free t^2 (tt = the
// denominator, device); gu0 = dL/du0; dwh += dL/dwh; loss += L.
__global__ void __launch_bounds__(256) head_bwd(const bf16 *u0, const float *wh,
                                                const float *c, const float *tg,
                                                const unsigned char *mask,
                                                const double *tt, float *gu0,
                                                float *dwh, double *loss, long V) {
  const float inv_n = (float)(*tt > 0.0 ? 1.0 / *tt : 1.0 / (double)V);
  float lw[17];
#pragma unroll
  for (int k = 0; k < 17; k++) lw[k] = 0.f;
  double ls = 0.0;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x) {
    const float d = mask[v] ? 0.f : c[v] - tg[v];
    ls += (double)d * d;
    const float dc = 2.f * d * inv_n;
#pragma unroll
    for (int k = 0; k < 16; k++) {
      const float u = __bfloat162float(u0[v * 16 + k]);
      gu0[v * 16 + k] = dc * wh[k];
      lw[k] += dc * u;
    }
    lw[16] += dc;
  }
  __shared__ float sw[8][17];
  __shared__ double sl[8];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 17; k++) {
    float x = lw[k];
    for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(FULLM, x, off);
    if (l == 0) sw[w][k] = x;
  }
  for (int off = 16; off; off >>= 1) ls += __shfl_xor_sync(FULLM, ls, off);
  if (l == 0) sl[w] = ls;
  __syncthreads();
  if (threadIdx.x < 17) {
    float x = 0.f;
    for (int j = 0; j < 8; j++) x += sw[j][threadIdx.x];
    atomicAdd(dwh + threadIdx.x, x);
  }
  if (threadIdx.x == 0) {
    double x = 0.0;
    for (int j = 0; j < 8; j++) x += sl[j];
    atomicAdd(loss, x * (double)inv_n);
  }
}

// ------------------------------------------------------- optimizer
__global__ void adam_kernel(float *th, const float *g, float *m, float *v, long n,
                            float lr, float b1, float b2, float eps, float bc1,
                            float bc2) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    th[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// BF16 copies of a conv layer's weights: wb (same layout) and wbt =
// [27][CIN][COUT] with the tap flipped (the backward data pass).
// wb[tap][co][ci] (forward), wbt[26 - tap][ci][co] (backward data pass) and
// wtc[tap][ci/8][co][ci%8] (the tensor-core kernel's core-matrix order).
__global__ void pack_weights(const float *th, bf16 *wb, bf16 *wbt, bf16 *wtc, int cin,
                             int cout) {
  const long total = 27L * cin * cout;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long)gridDim.x * blockDim.x) {
    const int tap = (int)(i / ((long)cin * cout));
    const int rem = (int)(i % ((long)cin * cout));
    const int co = rem / cin, ci = rem % cin;
    const bf16 b = __float2bfloat16_rn(th[i]);
    wb[i] = b;
    wbt[((long)(26 - tap) * cin + ci) * cout + co] = b;
    wtc[(((long)tap * (cin / 8) + ci / 8) * cout + co) * 8 + (ci & 7)] = b;
  }
}

// Nearest upsampling of a coarse [Vc][C] BF16 tensor to the fine grid
// (fine voxel (x, y, z) reads coarse (x/2, y/2, z/2)), 16 bytes a thread.
__global__ void upsample_bf16(const bf16 *__restrict__ in, bf16 *__restrict__ out,
                              int W, int H, long V, int Wc, int Hc, int C,
                              const int *skip, const int *skip2) {
  if (skipped(skip, skip2)) return;
  const int c8 = C / 8;
  const long total = V * c8;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long)gridDim.x * blockDim.x) {
    const long v = i / c8;
    const int k = (int)(i - v * c8);
    const int x = (int)(v % W);
    const long r = v / W;
    const int y = (int)(r % H), z = (int)(r / H);
    const long vc = (long)(x >> 1) + (long)Wc * ((long)(y >> 1) + (long)Hc * (z >> 1));
    reinterpret_cast<uint4 *>(out)[v * c8 + k] =
        __ldg(reinterpret_cast<const uint4 *>(in) + vc * c8 + k);
  }
}

// ------------------------------------------------ features / inputs
// acc[v][0..3] += (u_x, u_y, u_z, ln lambda - ln 1e-4) of each element at
// node v; acc[v][4] counts the elements.
__global__ void node_feature_acc(const int *conn, const double *vel,
                                 const double *lam, int E, float *acc) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < 8L * E;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t % E;
    const int n = conn[t] & NODE_BITS;
    const float f[4] = {(float)vel[e], (float)vel[E + e], (float)vel[2L * E + e],
                        (float)(log(lam[e]) - log(1e-4))};
#pragma unroll
    for (int k = 0; k < 4; k++) atomicAdd(acc + (long)n * 5 + k, f[k]);
    atomicAdd(acc + (long)n * 5 + 4, 1.f);
  }
}
__global__ void node_feature_fin(const float *acc, float *feat, long N) {
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < N;
       v += (long)gridDim.x * blockDim.x) {
    const float c = fmaxf(acc[v * 5 + 4], 1.f);
#pragma unroll
    for (int k = 0; k < 4; k++) feat[v * 4 + k] = acc[v * 5 + k] / c;
  }
}

// Deterministic sum over free nodes of f(v), f = x^2 (RMS) or diag (mean).
template <int MODE, typename T = double>  // 0: rms over free nodes; 1: mean; 2: sum x^2
__global__ void __launch_bounds__(256) free_sum(const T *x,
                                                const unsigned char *mask, long N,
                                                double *partials, unsigned *ticket,
                                                double *out, const int *skip,
                                                const int *skip2) {
  if (skipped(skip, skip2)) return;
  double s = 0.0, c = 0.0;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < N;
       v += (long)gridDim.x * blockDim.x) {
    if (!mask[v]) {
      const double xv = (double)x[v];
      s += MODE == 1 ? xv : xv * xv;
      c += 1.0;
    }
  }
  __shared__ double sm[2][8];
  __shared__ bool last;
  for (int off = 16; off; off >>= 1) {
    s += __shfl_xor_sync(FULLM, s, off);
    c += __shfl_xor_sync(FULLM, c, off);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sm[0][w] = s;
    sm[1][w] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = 0.0, a1 = 0.0;
    for (int j = 0; j < 8; j++) {
      a0 += sm[0][j];
      a1 += sm[1][j];
    }
    partials[2 * blockIdx.x] = a0;
    partials[2 * blockIdx.x + 1] = a1;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double a0 = 0.0, a1 = 0.0;
  for (unsigned b = 0; b < gridDim.x; b++) {
    a0 += __ldcg(partials + 2 * b);
    a1 += __ldcg(partials + 2 * b + 1);
  }
  *ticket = 0u;
  if (MODE == 0) {
    out[0] = a1 > 0.0 ? sqrt(a0 / a1) : 0.0;  // rms
  } else if (MODE == 1) {
    out[0] = a1 > 0.0 ? a0 / a1 : 1.0;  // mean
  } else {
    out[0] = a0;  // sum of squares
  }
}

// Network input: channel 0 = r / rms (FP64 or FP32 source), 1..4 features.
template <typename T>
__global__ void prep_input(const T *r, const double *rms, const float *feat,
                           bf16 *x0, long V, const int *skip, const int *skip2) {
  if (skipped(skip, skip2)) return;
  const double rm = rms ? *rms : 1.0;
  const double inv = rm > 0.0 ? 1.0 / rm : 0.0;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x) {
    const float f0 = (float)((double)r[v] * inv);
    const float4 f = *reinterpret_cast<const float4 *>(feat + v * 4);
    uint4 q0, q1;
    q0.x = pack2(f0, f.x);
    q0.y = pack2(f.y, f.z);
    q0.z = pack2(f.w, 0.f);
    q0.w = 0u;
    q1.x = q1.y = q1.z = q1.w = 0u;
    uint4 *p = reinterpret_cast<uint4 *>(x0 + v * 16);
    p[0] = q0;
    p[1] = q1;
  }
}

// out += (rms / dbar) * c on free nodes.
__global__ void combine_out(const float *c, const double *rms, const double *dbar,
                            const unsigned char *mask, double *out, long V,
                            const int *skip, const int *skip2) {
  if (skipped(skip, skip2)) return;
  const double sc = *rms / *dbar;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x)
    if (!mask[v]) out[v] += sc * (double)c[v];
}

// r = b - r (r holds A x_k).
__global__ void residual_inplace(const double *b, double *r, long V) {
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x)
    r[v] = b[v] - r[v];
}

// Training pair: rhat = r / rms(r); target = (e - D^-1 r) dbar / rms(r)
// with e = x* - x_k, zero on Dirichlet nodes.
__global__ void make_pair(const double *r, const double *xs, const double *xk,
                          const double *dinv, const unsigned char *mask,
                          const double *rms, const double *dbar, float *rhat,
                          float *tg, long V) {
  const double rm = *rms;
  const double inv = rm > 0.0 ? 1.0 / rm : 0.0;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x) {
    rhat[v] = (float)(r[v] * inv);
    tg[v] = mask[v] ? 0.f
                    : (float)(((xs[v] - xk[v]) - dinv[v] * r[v]) * *dbar * inv);
  }
}

// Residual loss: z = D^-1 rhat + c / dbar (0 on Dirichlet nodes).
__global__ void res_z(const float *rhat, const float *c, const double *dinv,
                      const unsigned char *mask, const double *dbar, double *z,
                      long V) {
  const double inv = 1.0 / *dbar;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x)
    z[v] = mask[v] ? 0.0 : dinv[v] * (double)rhat[v] + inv * (double)c[v];
}

// rho = rhat - A z on free nodes (q holds A z); sums ||rho||^2, ||rhat||^2
// (deterministic: per-block partials, last block adds in order) ->
// out[0] = ||rho||^2 / ||rhat||^2 (the loss), out[1] = ||rhat||^2.
__global__ void __launch_bounds__(256) res_rho(const float *rhat, const double *q,
                                               const unsigned char *mask, double *rho,
                                               long V, double *partials,
                                               unsigned *ticket, double *out) {
  double a0 = 0.0, a1 = 0.0;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x) {
    const double rv = mask[v] ? 0.0 : (double)rhat[v];
    const double pv = mask[v] ? 0.0 : rv - q[v];
    rho[v] = pv;
    a0 += pv * pv;
    a1 += rv * rv;
  }
  __shared__ double sm[2][8];
  __shared__ bool last;
  for (int off = 16; off; off >>= 1) {
    a0 += __shfl_xor_sync(FULLM, a0, off);
    a1 += __shfl_xor_sync(FULLM, a1, off);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sm[0][w] = a0;
    sm[1][w] = a1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int j = 0; j < 8; j++) {
      s0 += sm[0][j];
      s1 += sm[1][j];
    }
    partials[2 * blockIdx.x] = s0;
    partials[2 * blockIdx.x + 1] = s1;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double s0 = 0.0, s1 = 0.0;
  for (unsigned b = 0; b < gridDim.x; b++) {
    s0 += __ldcg(partials + 2 * b);
    s1 += __ldcg(partials + 2 * b + 1);
  }
  *ticket = 0u;
  out[0] = s1 > 0.0 ? s0 / s1 : 0.0;
  out[1] = s1;
}

// dL/dc = -2 (A^T rho) / (dbar ||rhat||^2) on free nodes (g holds A^T rho).
__global__ void res_dc(const double *g, const unsigned char *mask, const double *dbar,
                       const double *rr, float *dc, long V) {
  const double sc = *rr > 0.0 ? -2.0 / (*dbar * *rr) : 0.0;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x)
    dc[v] = mask[v] ? 0.f : (float)(sc * g[v]);
}

// Head backward from a given dL/dc: gu0 = dc wh, dwh += sum dc u0, dbh +=
// sum dc.
__global__ void __launch_bounds__(256) head_bwd_dc(const bf16 *u0, const float *wh,
                                                   const float *dc, float *gu0,
                                                   float *dwh, long V) {
  float lw[17];
#pragma unroll
  for (int k = 0; k < 17; k++) lw[k] = 0.f;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x) {
    const float d = dc[v];
#pragma unroll
    for (int k = 0; k < 16; k++) {
      gu0[v * 16 + k] = d * wh[k];
      lw[k] += d * __bfloat162float(u0[v * 16 + k]);
    }
    lw[16] += d;
  }
  __shared__ float sw[8][17];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < 17; k++) {
    float x = lw[k];
    for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(FULLM, x, off);
    if (l == 0) sw[w][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < 17) {
    float x = 0.f;
    for (int j = 0; j < 8; j++) x += sw[j][threadIdx.x];
    atomicAdd(dwh + threadIdx.x, x);
  }
}

// Post-smoothing: out += omega D^-1 (in - A out) (ax holds A out).
__global__ void smooth_out(const double *in, const double *ax, const double *dinv,
                           const unsigned char *mask, double omega, double *out,
                           long V, const int *skip, const int *skip2) {
  if (skipped(skip, skip2)) return;
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x)
    if (!mask[v]) out[v] += omega * dinv[v] * (in[v] - ax[v]);
}

// Jacobi part of the preconditioner (used by the standalone apply).
__global__ void jacobi_out(const double *in, const double *dinv,
                           const unsigned char *mask, double *out, long V) {
  for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < V;
       v += (long)gridDim.x * blockDim.x)
    out[v] = mask[v] ? 0.0 : in[v] * dinv[v];
}

}  // namespace

// ================================================================ host
struct Net {
  Handle *h = nullptr;
  Dims d[3];
  long woff[NLAYER], boff[NLAYER];
  long nparam = 0;
  float *theta = nullptr, *grad = nullptr, *am = nullptr, *av = nullptr;
  bf16 *wb = nullptr, *wbt = nullptr;
  // activations [V][C]
  bf16 *x0 = nullptr, *a0 = nullptr, *s0 = nullptr, *p0 = nullptr, *a1 = nullptr,
       *s1 = nullptr, *p1 = nullptr, *a2 = nullptr, *b2 = nullptr, *a3 = nullptr,
       *u1 = nullptr, *a4 = nullptr, *u0 = nullptr;
  float *c = nullptr;
  // gradients [V][C], FP32
  float *g_u0 = nullptr, *g_a4 = nullptr, *g_cat0 = nullptr, *g_s0 = nullptr,
        *g_u1 = nullptr, *g_a3 = nullptr, *g_cat1 = nullptr, *g_s1 = nullptr,
        *g_b2 = nullptr, *g_a2 = nullptr, *g_p1 = nullptr, *g_a1 = nullptr,
        *g_p0 = nullptr, *g_a0 = nullptr;
  float *feat = nullptr, *facc = nullptr;
  double *rbuf = nullptr;     // [N] residual scratch (training pairs)
  double *zbuf = nullptr, *qbuf = nullptr, *pbuf = nullptr, *gbuf = nullptr;  // residual loss
  float *dc = nullptr;
  bf16 *dyt = nullptr;  // [C][V] masked transposed output gradient (wgrad)
  double *scal = nullptr;  // [0] rms [1] loss [2] dbar [3] sum t^2 [4] residual loss [5] ||rhat||^2
  double *partials = nullptr;
  unsigned *ticket = nullptr;
  int red_grid = 0;
  int adam_t = 0;
  int smooth_steps = 1;   // Jacobi post-smoothing steps after the network
  double smooth_omega = 1.0;
  bool features_set = false;
  // tcgen05 forward convolutions: packed weights, the decoders' upsampled
  // inputs on the fine grid, and per layer the TMA maps of its inputs
  bf16 *wtc = nullptr;
  bf16 *up0 = nullptr, *up1 = nullptr;  // up(u1) on level 0, up(b2) on level 1
  int *tc_err = nullptr;                // bit 0: a tcgen05 kernel wait ran out
  int conv_mode = VDR_NET_CONV_MMA;
  bool tc_ok = false;                   // every map could be made
  CUtensorMap tmap[NLAYER][2];
  std::vector<void *> allocs;
};

namespace {

template <typename T>
cudaError_t nalloc(Net &n, T **p, size_t count) {
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(count, 1));
  if (!e) n.allocs.push_back((void *)*p);
  return e;
}

// host RNG for the initial weights (SplitMix64 + Box-Muller)
struct HostRng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uni() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double normal() {
    const double u1 = uni(), u2 = uni();
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  }
};

template <int CIN1, int CIN2, int COUT, bool F32IN, bool F32OUT>
cudaError_t conv_launch(const ConvArgs &a, cudaStream_t s) {
  // segments (m-tiles) per warp: two where the accumulators and the
  // staged rows of both fit the registers
  constexpr int MS = (COUT >= 64 || CIN1 + CIN2 >= 96) ? 1 : 2;
  const long nseg = (long)a.H * a.D * ((a.W + 15) / 16);
  const long groups = (nseg + MS - 1) / MS;
  const long blocks = std::min<long>((groups + 3) / 4, (long)device_sm_count() * 16);
  conv3_kernel<CIN1, CIN2, COUT, MS, F32IN, F32OUT><<<(unsigned)blocks, 128, 0, s>>>(a);
  count_launches(1);
  return cudaGetLastError();
}

template <int CIN1, int CIN2, int COUT>
cudaError_t wgrad_launch(const Net &n, WgArgs a, const float *dy, const bf16 *y,
                         cudaStream_t s) {
  constexpr int CIN = CIN1 + CIN2, NT = CIN / 8, MT = COUT / 16;
  // n-tiles per block (3 taps x MT x NG accumulator tiles, at most 24):
  // groups of 6 where they divide the channels evenly (no zero-filled units
  // staged), else 4 where they divide, else 2
  constexpr int NG = (MT == 1 && NT % 6 == 0) ? 6 : (MT <= 2 && NT % 4 == 0) ? 4 : 2;
  constexpr int NGROUPS = (NT + NG - 1) / NG;
  // masked, transposed BF16 output gradient with x rows padded to 16 voxels
  // (scratch sized for the largest layer)
  a.Wp = (a.W + 15) & ~15;
  a.Vp = (long)a.H * a.D * a.Wp;
  mask_transpose<COUT><<<(unsigned)((long)a.H * a.D), 128, 0, s>>>(dy, y, n.dyt, a.W, a.Wp, a.Vp);
  a.dyt = n.dyt;
  const long nks = (long)a.H * a.D * (a.Wp / 16);  // 16-voxel x-row segments
  const long target = std::max<long>(1, (long)device_sm_count() * 8 / (9 * NGROUPS));
  long chunk = (nks + target - 1) / target;
  chunk = std::max<long>(16, ((chunk + 3) / 4) * 4);
  a.chunk = chunk;
  const long nchunk = (nks + chunk - 1) / chunk;
  conv3_wgrad_tc<CIN1, CIN2, COUT, NG><<<dim3((unsigned)nchunk, 9, NGROUPS), 128, 0, s>>>(a);
  count_launches(2);
  return cudaGetLastError();
}

ConvArgs conv_args(const Net &n, int level, const void *in1, const bf16 *mask1,
                   const bf16 *in2, const bf16 *w, const float *bias, void *out,
                   bool relu, const int *skip, const int *skip2) {
  ConvArgs a{};
  const Dims &f = n.d[level];
  a.in1 = in1;
  a.mask1 = mask1;
  a.in2 = in2;
  a.w = w;
  a.bias = bias;
  a.out = out;
  a.W = f.W;
  a.H = f.H;
  a.D = f.D;
  if (level < 2) {
    a.Wc = n.d[level + 1].W;
    a.Hc = n.d[level + 1].H;
  }
  a.V = f.V;
  a.relu = relu ? 1 : 0;
  a.skip = skip;
  a.skip2 = skip2;
  return a;
}

WgArgs wg_args(const Net &n, int l, const bf16 *in1, const bf16 *in2) {
  WgArgs a{};
  const Dims &f = n.d[DEFS[l].level];
  a.in1 = in1;
  a.in2 = in2;
  a.dw = n.grad + n.woff[l];
  a.db = n.grad + n.boff[l];
  a.W = f.W;
  a.H = f.H;
  a.D = f.D;
  if (DEFS[l].level < 2) {
    a.Wc = n.d[DEFS[l].level + 1].W;
    a.Hc = n.d[DEFS[l].level + 1].H;
  }
  a.V = f.V;
  return a;
}

const bf16 *wf(const Net &n, int l) { return n.wb + n.woff[l]; }
const bf16 *wt(const Net &n, int l) { return n.wbt + n.woff[l]; }
const float *bs(const Net &n, int l) { return n.theta + n.boff[l]; }

// kernels of one forward pass: 10 convolutions, 2 pools, the head, and on
// the tensor-core path the 2 upsampled copies
int fwd_launches(const Net &n) {
  return (n.conv_mode == VDR_NET_CONV_TCGEN05 && n.tc_ok) ? 15 : 13;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *,
                                  const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// The map of a channels-last [V][C] BF16 tensor on grid d: dimensions (C,
// x, y, z), box (C channels, 10 x 18 x `planes` voxels) -- a tile's halo
// slab, swizzled for the tensor cores by its row width 2C; out-of-grid
// voxels read as zero.
bool make_tmap(CUtensorMap *m, const bf16 *base, int C, int planes, const Dims &d) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !base) return false;
  if (C != 16 && C != 32 && C != 64) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)d.W, (cuuint64_t)d.H,
                              (cuuint64_t)d.D};
  const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)C * 2 * d.W,
                                 (cuuint64_t)C * 2 * d.W * d.H};
  const cuuint32_t box[4] = {(cuuint32_t)C, convtc::SX, convtc::SY, (cuuint32_t)planes};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  const CUtensorMapSwizzle sw = C == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                                        : (C == 32 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                   : CU_TENSOR_MAP_SWIZZLE_32B);
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(base), dims,
            strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Every forward layer's input maps (in1, and the upsampled copy for the two
// decoder layers that concatenate); false if any cannot be made.
bool make_tmaps(Net &n) {
  struct In {
    int l;
    const bf16 *in1, *in2;
  };
  const In ins[] = {{L_E0A, n.x0, nullptr}, {L_E0B, n.a0, nullptr},
                    {L_E1A, n.p0, nullptr}, {L_E1B, n.a1, nullptr},
                    {L_BTA, n.p1, nullptr}, {L_BTB, n.a2, nullptr},
                    {L_D1A, n.s1, n.up1},   {L_D1B, n.a3, nullptr},
                    {L_D0A, n.s0, n.up0},   {L_D0B, n.a4, nullptr}};
  for (const In &i : ins) {
    const LayerDef &L = DEFS[i.l];
    const Dims &d = n.d[L.level];
    const int planes = convtc::group_of(L.cin1, L.cin2, L.cout) + 2;  // G + halo
    if (!make_tmap(&n.tmap[i.l][0], i.in1, L.cin1, planes, d)) return false;
    n.tmap[i.l][1] = n.tmap[i.l][0];
    if (i.in2 && !make_tmap(&n.tmap[i.l][1], i.in2, L.cin2, planes, d)) return false;
  }
  return true;
}

template <int CIN1, int CIN2, int COUT>
cudaError_t conv_tc_launch(const Net &n, int l, bf16 *out, const int *sk,
                           const int *sk2, cudaStream_t s) {
  using Sh = convtc::Shape<CIN1, CIN2, COUT>;
  auto kern = convtc::conv3_tc_kernel<CIN1, CIN2, COUT>;
  static const cudaError_t attr =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Sh::SMEM);
  if (attr) return attr;
  const Dims &d = n.d[DEFS[l].level];
  convtc::Args a;
  a.W = d.W;
  a.H = d.H;
  a.D = d.D;
  a.tiles_x = (d.W + convtc::TX - 1) / convtc::TX;
  a.tiles_y = (d.H + convtc::TY - 1) / convtc::TY;
  a.ntiles = a.tiles_x * a.tiles_y * ((d.D + Sh::G - 1) / Sh::G);
  a.wpk = n.wtc + n.woff[l];
  a.bias = n.theta + n.boff[l];
  a.out = out;
  a.relu = 1;
  a.err = n.tc_err;
  a.skip = sk;
  a.skip2 = sk2;
  const int grid = std::min(a.ntiles, device_sm_count());
  kern<<<grid, convtc::THREADS, Sh::SMEM, s>>>(n.tmap[l][0], n.tmap[l][1], a);
  count_launches(1);
  return cudaGetLastError();
}

// The forward pass's ten convolutions on the tensor cores (tcgen05).
cudaError_t net_forward_tc(Net &n, const int *sk, const int *sk2, cudaStream_t s) {
  cudaError_t e;
  const Dims &f0 = n.d[0], &f1 = n.d[1], &f2 = n.d[2];
  if ((e = conv_tc_launch<16, 0, 16>(n, L_E0A, n.a0, sk, sk2, s)) ||
      (e = conv_tc_launch<16, 0, 16>(n, L_E0B, n.s0, sk, sk2, s)))
    return e;
  pool_fwd<<<grid_for(f1.V * 16, 256), 256, 0, s>>>(n.s0, n.p0, f0, f1, 16, sk, sk2);
  if ((e = conv_tc_launch<16, 0, 32>(n, L_E1A, n.a1, sk, sk2, s)) ||
      (e = conv_tc_launch<32, 0, 32>(n, L_E1B, n.s1, sk, sk2, s)))
    return e;
  pool_fwd<<<grid_for(f2.V * 32, 256), 256, 0, s>>>(n.s1, n.p1, f1, f2, 32, sk, sk2);
  if ((e = conv_tc_launch<32, 0, 64>(n, L_BTA, n.a2, sk, sk2, s)) ||
      (e = conv_tc_launch<64, 0, 64>(n, L_BTB, n.b2, sk, sk2, s)))
    return e;
  upsample_bf16<<<grid_for(f1.V * 8, 256), 256, 0, s>>>(n.b2, n.up1, f1.W, f1.H, f1.V,
                                                         f2.W, f2.H, 64, sk, sk2);
  if ((e = conv_tc_launch<32, 64, 32>(n, L_D1A, n.a3, sk, sk2, s)) ||
      (e = conv_tc_launch<32, 0, 32>(n, L_D1B, n.u1, sk, sk2, s)))
    return e;
  upsample_bf16<<<grid_for(f0.V * 4, 256), 256, 0, s>>>(n.u1, n.up0, f0.W, f0.H, f0.V,
                                                         f1.W, f1.H, 32, sk, sk2);
  if ((e = conv_tc_launch<16, 32, 16>(n, L_D0A, n.a4, sk, sk2, s)) ||
      (e = conv_tc_launch<16, 0, 16>(n, L_D0B, n.u0, sk, sk2, s)))
    return e;
  head_fwd<<<grid_for(f0.V, 256), 256, 0, s>>>(n.u0, n.theta + n.woff[L_HEAD], n.c, f0.V,
                                                sk, sk2);
  count_launches(5);
  return cudaGetLastError();
}

// Forward pass from the prepared input x0 to the head output c.
cudaError_t net_forward(Net &n, const int *sk, const int *sk2, cudaStream_t s) {
  if (n.conv_mode == VDR_NET_CONV_TCGEN05 && n.tc_ok) return net_forward_tc(n, sk, sk2, s);
  cudaError_t e;
#define VDR_CONV(CI1, CI2, CO, LVL, IN1, IN2, L, OUT)                              \
  if ((e = conv_launch<CI1, CI2, CO, false, false>(                                \
           conv_args(n, LVL, IN1, nullptr, IN2, wf(n, L), bs(n, L), OUT, true, sk, \
                     sk2),                                                         \
           s)))                                                                    \
    return e;
  VDR_CONV(16, 0, 16, 0, n.x0, nullptr, L_E0A, n.a0)
  VDR_CONV(16, 0, 16, 0, n.a0, nullptr, L_E0B, n.s0)
  pool_fwd<<<grid_for(n.d[1].V * 16, 256), 256, 0, s>>>(n.s0, n.p0, n.d[0], n.d[1], 16, sk, sk2);
  VDR_CONV(16, 0, 32, 1, n.p0, nullptr, L_E1A, n.a1)
  VDR_CONV(32, 0, 32, 1, n.a1, nullptr, L_E1B, n.s1)
  pool_fwd<<<grid_for(n.d[2].V * 32, 256), 256, 0, s>>>(n.s1, n.p1, n.d[1], n.d[2], 32, sk, sk2);
  VDR_CONV(32, 0, 64, 2, n.p1, nullptr, L_BTA, n.a2)
  VDR_CONV(64, 0, 64, 2, n.a2, nullptr, L_BTB, n.b2)
  VDR_CONV(32, 64, 32, 1, n.s1, n.b2, L_D1A, n.a3)
  VDR_CONV(32, 0, 32, 1, n.a3, nullptr, L_D1B, n.u1)
  VDR_CONV(16, 32, 16, 0, n.s0, n.u1, L_D0A, n.a4)
  VDR_CONV(16, 0, 16, 0, n.a4, nullptr, L_D0B, n.u0)
#undef VDR_CONV
  head_fwd<<<grid_for(n.d[0].V, 256), 256, 0, s>>>(n.u0, n.theta + n.woff[L_HEAD],
                                                   n.c, n.d[0].V, sk, sk2);
  count_launches(3);
  return cudaGetLastError();
}

// Backward pass: the loss gradient of the head output is already in g_u0
// (and the head's weight gradient in grad); accumulates every layer's
// weight and bias gradients into grad.
cudaError_t net_backward(Net &n, cudaStream_t s) {
  cudaError_t e;
  const Dims &f0 = n.d[0], &f1 = n.d[1], &f2 = n.d[2];
  // d0b: u0 = relu(conv(a4))
  if ((e = wgrad_launch<16, 0, 16>(n, wg_args(n, L_D0B, n.a4, nullptr), n.g_u0, n.u0, s))) return e;
  if ((e = conv_launch<16, 0, 16, true, true>(
           conv_args(n, 0, n.g_u0, n.u0, nullptr, wt(n, L_D0B), nullptr, n.g_a4, false,
                     nullptr, nullptr), s))) return e;
  // d0a: a4 = relu(conv([s0 | up(u1)]))
  if ((e = wgrad_launch<16, 32, 16>(n, wg_args(n, L_D0A, n.s0, n.u1), n.g_a4, n.a4, s))) return e;
  if ((e = conv_launch<16, 0, 48, true, true>(
           conv_args(n, 0, n.g_a4, n.a4, nullptr, wt(n, L_D0A), nullptr, n.g_cat0, false,
                     nullptr, nullptr), s))) return e;
  upcat_bwd_skip<<<grid_for(f0.V * 16, 256), 256, 0, s>>>(n.g_cat0, n.g_s0, f0.V, 16, 32);
  upcat_bwd_coarse<<<grid_for(f1.V * 32, 256), 256, 0, s>>>(n.g_cat0, n.g_u1, f0, f1, 16, 32);
  count_launches(2);
  // d1b: u1 = relu(conv(a3))
  if ((e = wgrad_launch<32, 0, 32>(n, wg_args(n, L_D1B, n.a3, nullptr), n.g_u1, n.u1, s))) return e;
  if ((e = conv_launch<32, 0, 32, true, true>(
           conv_args(n, 1, n.g_u1, n.u1, nullptr, wt(n, L_D1B), nullptr, n.g_a3, false,
                     nullptr, nullptr), s))) return e;
  // d1a: a3 = relu(conv([s1 | up(b2)]))
  if ((e = wgrad_launch<32, 64, 32>(n, wg_args(n, L_D1A, n.s1, n.b2), n.g_a3, n.a3, s))) return e;
  if ((e = conv_launch<32, 0, 96, true, true>(
           conv_args(n, 1, n.g_a3, n.a3, nullptr, wt(n, L_D1A), nullptr, n.g_cat1, false,
                     nullptr, nullptr), s))) return e;
  upcat_bwd_skip<<<grid_for(f1.V * 32, 256), 256, 0, s>>>(n.g_cat1, n.g_s1, f1.V, 32, 64);
  upcat_bwd_coarse<<<grid_for(f2.V * 64, 256), 256, 0, s>>>(n.g_cat1, n.g_b2, f1, f2, 32, 64);
  count_launches(2);
  // btb: b2 = relu(conv(a2))
  if ((e = wgrad_launch<64, 0, 64>(n, wg_args(n, L_BTB, n.a2, nullptr), n.g_b2, n.b2, s))) return e;
  if ((e = conv_launch<64, 0, 64, true, true>(
           conv_args(n, 2, n.g_b2, n.b2, nullptr, wt(n, L_BTB), nullptr, n.g_a2, false,
                     nullptr, nullptr), s))) return e;
  // bta: a2 = relu(conv(p1))
  if ((e = wgrad_launch<32, 0, 64>(n, wg_args(n, L_BTA, n.p1, nullptr), n.g_a2, n.a2, s))) return e;
  if ((e = conv_launch<64, 0, 32, true, true>(
           conv_args(n, 2, n.g_a2, n.a2, nullptr, wt(n, L_BTA), nullptr, n.g_p1, false,
                     nullptr, nullptr), s))) return e;
  pool_bwd_add<<<grid_for(f1.V * 32, 256), 256, 0, s>>>(n.g_p1, n.g_s1, f1, f2, 32);
  count_launches(1);
  // e1b: s1 = relu(conv(a1))
  if ((e = wgrad_launch<32, 0, 32>(n, wg_args(n, L_E1B, n.a1, nullptr), n.g_s1, n.s1, s))) return e;
  if ((e = conv_launch<32, 0, 32, true, true>(
           conv_args(n, 1, n.g_s1, n.s1, nullptr, wt(n, L_E1B), nullptr, n.g_a1, false,
                     nullptr, nullptr), s))) return e;
  // e1a: a1 = relu(conv(p0))
  if ((e = wgrad_launch<16, 0, 32>(n, wg_args(n, L_E1A, n.p0, nullptr), n.g_a1, n.a1, s))) return e;
  if ((e = conv_launch<32, 0, 16, true, true>(
           conv_args(n, 1, n.g_a1, n.a1, nullptr, wt(n, L_E1A), nullptr, n.g_p0, false,
                     nullptr, nullptr), s))) return e;
  pool_bwd_add<<<grid_for(f0.V * 16, 256), 256, 0, s>>>(n.g_p0, n.g_s0, f0, f1, 16);
  count_launches(1);
  // e0b: s0 = relu(conv(a0))
  if ((e = wgrad_launch<16, 0, 16>(n, wg_args(n, L_E0B, n.a0, nullptr), n.g_s0, n.s0, s))) return e;
  if ((e = conv_launch<16, 0, 16, true, true>(
           conv_args(n, 0, n.g_s0, n.s0, nullptr, wt(n, L_E0B), nullptr, n.g_a0, false,
                     nullptr, nullptr), s))) return e;
  // e0a: a0 = relu(conv(x0)); the input needs no gradient
  if ((e = wgrad_launch<16, 0, 16>(n, wg_args(n, L_E0A, n.x0, nullptr), n.g_a0, n.a0, s))) return e;
  return cudaGetLastError();
}

cudaError_t pack_all(Net &n, cudaStream_t s) {
  for (int l = 0; l < L_HEAD; l++) {
    const int cin = DEFS[l].cin1 + DEFS[l].cin2, cout = DEFS[l].cout;
    pack_weights<<<grid_for(layer_wsize(l), 256), 256, 0, s>>>(
        n.theta + n.woff[l], n.wb + n.woff[l], n.wbt + n.woff[l], n.wtc + n.woff[l], cin,
        cout);
  }
  count_launches(L_HEAD);
  return cudaGetLastError();
}

// Loss and gradients of one (rhat, target) pair into n.grad (zeroed first).
cudaError_t net_loss_grad(Net &n, const float *rhat, const float *tg, cudaStream_t s) {
  cudaError_t e;
  const long V = n.d[0].V;
  prep_input<float><<<grid_for(V, 256), 256, 0, s>>>(rhat, nullptr, n.feat, n.x0, V,
                                                       nullptr, nullptr);
  count_launches(1);
  if ((e = net_forward(n, nullptr, nullptr, s))) return e;
  if ((e = cudaMemsetAsync(n.grad, 0, sizeof(float) * n.nparam, s))) return e;
  if ((e = cudaMemsetAsync(n.scal + 1, 0, sizeof(double), s))) return e;
  free_sum<2, float><<<n.red_grid, 256, 0, s>>>(tg, n.h->mask, V, n.partials, n.ticket,
                                                n.scal + 3, nullptr, nullptr);
  head_bwd<<<grid_for(V, 256, 4), 256, 0, s>>>(n.u0, n.theta + n.woff[L_HEAD], n.c, tg,
                                               n.h->mask, n.scal + 3, n.g_u0,
                                               n.grad + n.woff[L_HEAD], n.scal + 1, V);
  count_launches(2);
  return net_backward(n, s);
}

// Residual loss of one normalised residual rhat with the handle's current
// operator: z = D^-1 rhat + c/dbar, L = ||rhat - A z||^2 / ||rhat||^2 (free
// nodes); gradients of every parameter into n.grad (zeroed first).
cudaError_t net_residual_loss_grad(Net &n, const float *rhat, cudaStream_t s) {
  cudaError_t e;
  Handle &h = *n.h;
  const long V = n.d[0].V;
  prep_input<float><<<grid_for(V, 256), 256, 0, s>>>(rhat, nullptr, n.feat, n.x0, V,
                                                       nullptr, nullptr);
  count_launches(1);
  if ((e = net_forward(n, nullptr, nullptr, s))) return e;
  res_z<<<grid_for(V, 256), 256, 0, s>>>(rhat, n.c, h.dinv, h.mask, n.scal + 2, n.zbuf, V);
  count_launches(1);
  if ((e = cudaMemsetAsync(n.qbuf, 0, sizeof(double) * V, s)) ||
      (e = launch_apply(h, false, n.zbuf, n.qbuf, nullptr, nullptr, s)))
    return e;
  res_rho<<<n.red_grid, 256, 0, s>>>(rhat, n.qbuf, h.mask, n.pbuf, V, n.partials,
                                     n.ticket, n.scal + 4);
  count_launches(1);
  if ((e = cudaMemsetAsync(n.gbuf, 0, sizeof(double) * V, s)) ||
      (e = launch_apply(h, true, n.pbuf, n.gbuf, nullptr, nullptr, s)))
    return e;
  res_dc<<<grid_for(V, 256), 256, 0, s>>>(n.gbuf, h.mask, n.scal + 2, n.scal + 5, n.dc, V);
  count_launches(1);
  if ((e = cudaMemsetAsync(n.grad, 0, sizeof(float) * n.nparam, s))) return e;
  head_bwd_dc<<<grid_for(V, 256, 4), 256, 0, s>>>(n.u0, n.theta + n.woff[L_HEAD], n.dc,
                                                  n.g_u0, n.grad + n.woff[L_HEAD], V);
  count_launches(1);
  return net_backward(n, s);
}

// Preconditioner hook: out += (rms(in)/dbar) net(in/rms(in)).
cudaError_t net_enqueue(void *ctx, const double *in, double *out, const int *skip,
                        const int *skip2, cudaStream_t s) {
  Net &n = *static_cast<Net *>(ctx);
  const long V = n.d[0].V;
  free_sum<0><<<n.red_grid, 256, 0, s>>>(in, n.h->mask, V, n.partials, n.ticket,
                                         n.scal, skip, skip2);
  prep_input<double><<<grid_for(V, 256), 256, 0, s>>>(in, n.scal, n.feat, n.x0, V,
                                                        skip, skip2);
  count_launches(2);
  cudaError_t e = net_forward(n, skip, skip2, s);
  if (e) return e;
  combine_out<<<grid_for(V, 256), 256, 0, s>>>(n.c, n.scal, n.scal + 2, n.h->mask,
                                               out, V, skip, skip2);
  count_launches(1);
  // The network's output is accurate at long wavelengths only (BF16
  // activations leave noise that A amplifies); Jacobi steps remove the
  // short-wavelength error of the combined estimate.
  for (int k = 0; k < n.smooth_steps; k++) {
    if ((e = cudaMemsetAsync(n.rbuf, 0, sizeof(double) * V, s)) ||
        (e = launch_apply(*n.h, false, out, n.rbuf, skip, skip2, s)))
      return e;
    smooth_out<<<grid_for(V, 256), 256, 0, s>>>(in, n.rbuf, n.h->dinv, n.h->mask,
                                                n.smooth_omega, out, V, skip, skip2);
    count_launches(1);
  }
  return cudaGetLastError();
}

int net_enqueue_launches(const Net &n) {
  return fwd_launches(n) + 4 + n.smooth_steps * (1 + apply_launches(*n.h));
}

}  // namespace
}  // namespace vdr

// ============================================================ C ABI
struct vdr_net {
  vdr::Net n;
};

using namespace vdr;

extern "C" int vdr_net_adam_step(vdr_net *N, float lr, float beta1, float beta2,
                                 float eps);

static int net_check(vdr_net *N) {
  if (!N || !N->n.h) {
    set_error("null network");
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e = cudaSetDevice(N->n.h->device);
  return e ? cuda_fail(e, "cudaSetDevice") : VDR_OK;
}

extern "C" int vdr_net_create(vdr_handle *H, unsigned long long seed, vdr_net **out) {
  if (!H || !out) {
    set_error("vdr_net_create: null argument");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = handle_of(H);
  if (h.nax <= 0) {
    set_error("vdr_net_create: the network needs the structured node numbering");
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e = cudaSetDevice(h.device);
  if (e) return cuda_fail(e, "cudaSetDevice");
  vdr_net *N = new vdr_net();
  Net &n = N->n;
  n.h = &h;
  n.d[0] = Dims{h.nax, h.nay, h.naz, (long)h.N};
  n.d[1] = coarse_of(n.d[0]);
  n.d[2] = coarse_of(n.d[1]);
  long off = 0;
  for (int l = 0; l < NLAYER; l++) {
    n.woff[l] = off;
    off += layer_wsize(l);
    n.boff[l] = off;
    off += DEFS[l].cout;
    off = (off + 7) & ~7L;  // keep BF16 pair loads aligned
  }
  n.nparam = off;
  const long V0 = n.d[0].V, V1 = n.d[1].V, V2 = n.d[2].V;
  n.red_grid = grid_for(V0, 256, 4);
  int st = VDR_OK;
  do {
    if ((e = nalloc(n, &n.theta, off)) || (e = nalloc(n, &n.grad, off)) ||
        (e = nalloc(n, &n.am, off)) || (e = nalloc(n, &n.av, off)) ||
        (e = nalloc(n, &n.wb, off)) || (e = nalloc(n, &n.wbt, off)) ||
        (e = nalloc(n, &n.x0, V0 * 16)) || (e = nalloc(n, &n.a0, V0 * 16)) ||
        (e = nalloc(n, &n.s0, V0 * 16)) || (e = nalloc(n, &n.p0, V1 * 16)) ||
        (e = nalloc(n, &n.a1, V1 * 32)) || (e = nalloc(n, &n.s1, V1 * 32)) ||
        (e = nalloc(n, &n.p1, V2 * 32)) || (e = nalloc(n, &n.a2, V2 * 64)) ||
        (e = nalloc(n, &n.b2, V2 * 64)) || (e = nalloc(n, &n.a3, V1 * 32)) ||
        (e = nalloc(n, &n.u1, V1 * 32)) || (e = nalloc(n, &n.a4, V0 * 16)) ||
        (e = nalloc(n, &n.u0, V0 * 16)) || (e = nalloc(n, &n.c, V0)) ||
        (e = nalloc(n, &n.g_u0, V0 * 16)) || (e = nalloc(n, &n.g_a4, V0 * 16)) ||
        (e = nalloc(n, &n.g_cat0, V0 * 48)) || (e = nalloc(n, &n.g_s0, V0 * 16)) ||
        (e = nalloc(n, &n.g_u1, V1 * 32)) || (e = nalloc(n, &n.g_a3, V1 * 32)) ||
        (e = nalloc(n, &n.g_cat1, V1 * 96)) || (e = nalloc(n, &n.g_s1, V1 * 32)) ||
        (e = nalloc(n, &n.g_b2, V2 * 64)) || (e = nalloc(n, &n.g_a2, V2 * 64)) ||
        (e = nalloc(n, &n.g_p1, V2 * 32)) || (e = nalloc(n, &n.g_a1, V1 * 32)) ||
        (e = nalloc(n, &n.g_p0, V1 * 16)) || (e = nalloc(n, &n.g_a0, V0 * 16)) ||
        (e = nalloc(n, &n.feat, V0 * 4)) || (e = nalloc(n, &n.facc, V0 * 5)) ||
        (e = nalloc(n, &n.rbuf, V0)) || (e = nalloc(n, &n.zbuf, V0)) ||
        (e = nalloc(n, &n.qbuf, V0)) || (e = nalloc(n, &n.pbuf, V0)) ||
        (e = nalloc(n, &n.gbuf, V0)) || (e = nalloc(n, &n.dc, V0)) ||
        (e = nalloc(n, &n.dyt, std::max(std::max(padded_rows(n.d[0]) * 16,
                                                  padded_rows(n.d[1]) * 32),
                                         padded_rows(n.d[2]) * 64))) ||
        (e = nalloc(n, &n.scal, 8)) || (e = nalloc(n, &n.partials, 2L * n.red_grid)) ||
        (e = nalloc(n, &n.ticket, 1)) || (e = nalloc(n, &n.wtc, off)) ||
        (e = nalloc(n, &n.up0, V0 * 32)) || (e = nalloc(n, &n.up1, V1 * 64)) ||
        (e = nalloc(n, &n.tc_err, 1))) {
      st = cuda_fail(e, "network allocation");
      break;
    }
    // the tensor-core path where every input's tensor map can be made
    n.tc_ok = make_tmaps(n);
    n.conv_mode = n.tc_ok ? VDR_NET_CONV_TCGEN05 : VDR_NET_CONV_MMA;
    if ((e = cudaMemsetAsync(n.tc_err, 0, sizeof(int), h.stream))) {
      st = cuda_fail(e, "network initialisation");
      break;
    }
    // Kaiming-normal weights (real fan-in), zero biases; the head starts at
    // zero so the untrained preconditioner is Jacobi.
    std::vector<float> th(off, 0.f);
    HostRng rng{seed ^ 0x5eed5eedull};
    for (int l = 0; l < L_HEAD; l++) {
      const int cin = DEFS[l].cin1 + DEFS[l].cin2, cout = DEFS[l].cout;
      const int real_in = l == L_E0A ? IN_REAL : cin;
      const double sd = sqrt(2.0 / (27.0 * real_in));
      for (int tap = 0; tap < 27; tap++)
        for (int co = 0; co < cout; co++)
          for (int ci = 0; ci < cin; ci++)
            th[n.woff[l] + ((long)tap * cout + co) * cin + ci] =
                ci < real_in ? (float)(sd * rng.normal()) : 0.f;
    }
    if ((e = cudaMemcpyAsync(n.theta, th.data(), sizeof(float) * off,
                             cudaMemcpyHostToDevice, h.stream)) ||
        (e = cudaMemsetAsync(n.am, 0, sizeof(float) * off, h.stream)) ||
        (e = cudaMemsetAsync(n.av, 0, sizeof(float) * off, h.stream)) ||
        (e = cudaMemsetAsync(n.grad, 0, sizeof(float) * off, h.stream)) ||
        (e = cudaMemsetAsync(n.feat, 0, sizeof(float) * V0 * 4, h.stream)) ||
        (e = cudaMemsetAsync(n.ticket, 0, sizeof(unsigned), h.stream)) ||
        (e = cudaMemsetAsync(n.scal, 0, sizeof(double) * 8, h.stream)) ||
        (e = pack_all(n, h.stream)) || (e = cudaStreamSynchronize(h.stream))) {
      st = cuda_fail(e, "network initialisation");
      break;
    }
  } while (0);
  if (st) {
    for (void *p : n.allocs) cudaFree(p);
    delete N;
    return st;
  }
  *out = N;
  return VDR_OK;
}

extern "C" int vdr_net_set_conv(vdr_net *N, int mode) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  if (mode != VDR_NET_CONV_MMA && mode != VDR_NET_CONV_TCGEN05) {
    set_error("vdr_net_set_conv: unknown mode");
    return VDR_BAD_ARGUMENT;
  }
  if (mode == VDR_NET_CONV_TCGEN05 && !n.tc_ok) {
    set_error("vdr_net_set_conv: the tensor maps of the tcgen05 path could not be made");
    return VDR_BAD_ARGUMENT;
  }
  n.conv_mode = mode;
  return VDR_OK;
}

extern "C" int vdr_net_conv_status(vdr_net *N, int *mode) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  if (mode) *mode = (n.conv_mode == VDR_NET_CONV_TCGEN05 && n.tc_ok) ? VDR_NET_CONV_TCGEN05
                                                                       : VDR_NET_CONV_MMA;
  int err = 0;
  cudaError_t e = cudaMemcpyAsync(&err, n.tc_err, sizeof(int), cudaMemcpyDeviceToHost,
                                  n.h->stream);
  if (!e) e = cudaStreamSynchronize(n.h->stream);
  if (!e) e = cudaMemsetAsync(n.tc_err, 0, sizeof(int), n.h->stream);
  if (e) return cuda_fail(e, "vdr_net_conv_status");
  if (err) {
    set_error("a tcgen05 convolution gave up waiting for its operands");
    return VDR_TIMEOUT;
  }
  return VDR_OK;
}

extern "C" int vdr_net_destroy(vdr_net *N) {
  if (!N) return VDR_OK;
  if (N->n.h) {
    cudaSetDevice(N->n.h->device);
    cudaStreamSynchronize(N->n.h->stream);
  }
  for (void *p : N->n.allocs) cudaFree(p);
  delete N;
  return VDR_OK;
}

extern "C" int vdr_net_param_count(vdr_net *N, long long *count) {
  int st = net_check(N);
  if (st) return st;
  if (!count) return VDR_BAD_ARGUMENT;
  *count = N->n.nparam;
  return VDR_OK;
}

static int copy_params(vdr_net *N, float *host, const float *src_dev, bool to_host) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  if (!host) {
    set_error("null host buffer");
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e;
  if (to_host) {
    e = cudaMemcpyAsync(host, src_dev, sizeof(float) * n.nparam, cudaMemcpyDeviceToHost,
                        n.h->stream);
  } else {
    e = cudaMemcpyAsync(n.theta, host, sizeof(float) * n.nparam, cudaMemcpyHostToDevice,
                        n.h->stream);
    if (!e) e = pack_all(n, n.h->stream);
  }
  if (!e) e = cudaStreamSynchronize(n.h->stream);
  return e ? cuda_fail(e, "parameter copy") : VDR_OK;
}

extern "C" int vdr_net_get_params(vdr_net *N, float *host) {
  return copy_params(N, host, N ? N->n.theta : nullptr, true);
}
extern "C" int vdr_net_set_params(vdr_net *N, const float *host) {
  return copy_params(N, const_cast<float *>(host), nullptr, false);
}
extern "C" int vdr_net_get_grads(vdr_net *N, float *host) {
  return copy_params(N, host, N ? N->n.grad : nullptr, true);
}

extern "C" int vdr_net_update_features(vdr_net *N, float *d_feat_out, double *dbar_out) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  Handle &h = *n.h;
  if ((st = prepare_operator(h))) return st;
  cudaStream_t s = h.stream;
  const long V = n.d[0].V;
  cudaError_t e;
  if ((e = cudaMemsetAsync(n.facc, 0, sizeof(float) * V * 5, s))) return cuda_fail(e, "memset");
  node_feature_acc<<<grid_for(8L * h.E, 256), 256, 0, s>>>(h.conn, h.vel, h.lam, h.E, n.facc);
  node_feature_fin<<<grid_for(V, 256), 256, 0, s>>>(n.facc, n.feat, V);
  free_sum<1><<<n.red_grid, 256, 0, s>>>(h.diag, h.mask, V, n.partials, n.ticket,
                                         n.scal + 2, nullptr, nullptr);
  count_launches(3);
  if ((e = cudaGetLastError())) return cuda_fail(e, "features");
  if (d_feat_out &&
      (e = cudaMemcpyAsync(d_feat_out, n.feat, sizeof(float) * V * 4,
                           cudaMemcpyDeviceToDevice, s)))
    return cuda_fail(e, "features copy");
  double dbar = 0.0;
  if ((e = cudaMemcpyAsync(&dbar, n.scal + 2, sizeof(double), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "features");
  if (dbar_out) *dbar_out = dbar;
  n.features_set = true;
  return VDR_OK;
}

extern "C" int vdr_net_set_features_device(vdr_net *N, const float *d_feat, double dbar) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  if (!d_feat || !(dbar > 0.0)) {
    set_error("vdr_net_set_features_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  cudaError_t e;
  if ((e = cudaMemcpyAsync(n.feat, d_feat, sizeof(float) * n.d[0].V * 4,
                           cudaMemcpyDeviceToDevice, n.h->stream)) ||
      (e = cudaMemcpyAsync(n.scal + 2, &dbar, sizeof(double), cudaMemcpyHostToDevice,
                           n.h->stream)) ||
      (e = cudaStreamSynchronize(n.h->stream)))
    return cuda_fail(e, "features");
  n.features_set = true;
  return VDR_OK;
}

extern "C" int vdr_net_make_pair_device(vdr_net *N, const double *d_b,
                                        const double *d_xk, const double *d_xstar,
                                        float *d_rhat, float *d_target) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  Handle &h = *n.h;
  if (!d_b || !d_xk || !d_xstar || !d_rhat || !d_target || !n.features_set) {
    set_error("vdr_net_make_pair_device: bad arguments or features not set");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = prepare_operator(h))) return st;
  const long V = n.d[0].V;
  cudaStream_t s = h.stream;
  cudaError_t e;
  if ((e = cudaMemsetAsync(n.rbuf, 0, sizeof(double) * V, s)) ||
      (e = launch_apply(h, false, d_xk, n.rbuf, nullptr, nullptr, s)))
    return cuda_fail(e, "pair residual");
  residual_inplace<<<grid_for(V, 256), 256, 0, s>>>(d_b, n.rbuf, V);
  free_sum<0><<<n.red_grid, 256, 0, s>>>(n.rbuf, h.mask, V, n.partials, n.ticket, n.scal,
                                         nullptr, nullptr);
  make_pair<<<grid_for(V, 256), 256, 0, s>>>(n.rbuf, d_xstar, d_xk, h.dinv, h.mask, n.scal,
                                             n.scal + 2, d_rhat, d_target, V);
  count_launches(3);
  e = cudaGetLastError();
  return e ? cuda_fail(e, "pair") : VDR_OK;
}

extern "C" int vdr_net_forward_device(vdr_net *N, const float *d_rhat, float *d_out) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  if (!d_rhat || !d_out) {
    set_error("vdr_net_forward_device: null argument");
    return VDR_BAD_ARGUMENT;
  }
  const long V = n.d[0].V;
  cudaStream_t s = n.h->stream;
  prep_input<float><<<grid_for(V, 256), 256, 0, s>>>(d_rhat, nullptr, n.feat, n.x0, V,
                                                       nullptr, nullptr);
  count_launches(1);
  cudaError_t e = net_forward(n, nullptr, nullptr, s);
  if (!e) e = cudaMemcpyAsync(d_out, n.c, sizeof(float) * V, cudaMemcpyDeviceToDevice, s);
  return e ? cuda_fail(e, "network forward") : VDR_OK;
}

extern "C" int vdr_net_loss_grad_device(vdr_net *N, const float *d_rhat,
                                        const float *d_target, double *loss) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  if (!d_rhat || !d_target) {
    set_error("vdr_net_loss_grad_device: null argument");
    return VDR_BAD_ARGUMENT;
  }
  cudaStream_t s = n.h->stream;
  cudaError_t e = net_loss_grad(n, d_rhat, d_target, s);
  if (!e && loss) {
    e = cudaMemcpyAsync(loss, n.scal + 1, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
  }
  return e ? cuda_fail(e, "network loss/gradient") : VDR_OK;
}

extern "C" int vdr_net_residual_loss_grad_device(vdr_net *N, const float *d_rhat,
                                                 double *loss) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  if (!d_rhat || !n.features_set) {
    set_error("vdr_net_residual_loss_grad_device: null argument or features not set");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = prepare_operator(*n.h))) return st;
  cudaStream_t s = n.h->stream;
  cudaError_t e = net_residual_loss_grad(n, d_rhat, s);
  if (!e && loss) {
    e = cudaMemcpyAsync(loss, n.scal + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
  }
  return e ? cuda_fail(e, "network residual loss/gradient") : VDR_OK;
}

extern "C" int vdr_net_train_step_residual_device(vdr_net *N, const float *d_rhat,
                                                  float lr, double *loss) {
  int st = vdr_net_residual_loss_grad_device(N, d_rhat, nullptr);
  if (st) return st;
  st = vdr_net_adam_step(N, lr, 0.9f, 0.999f, 1e-8f);
  if (st) return st;
  if (loss) {
    cudaError_t e = cudaMemcpyAsync(loss, N->n.scal + 4, sizeof(double),
                                    cudaMemcpyDeviceToHost, N->n.h->stream);
    if (!e) e = cudaStreamSynchronize(N->n.h->stream);
    if (e) return cuda_fail(e, "loss");
  }
  return VDR_OK;
}

extern "C" int vdr_net_adam_step(vdr_net *N, float lr, float beta1, float beta2, float eps) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  cudaStream_t s = n.h->stream;
  n.adam_t += 1;
  const float bc1 = 1.f - powf(beta1, (float)n.adam_t);
  const float bc2 = 1.f - powf(beta2, (float)n.adam_t);
  adam_kernel<<<grid_for(n.nparam, 256), 256, 0, s>>>(n.theta, n.grad, n.am, n.av, n.nparam,
                                                      lr, beta1, beta2, eps, bc1, bc2);
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (!e) e = pack_all(n, s);
  return e ? cuda_fail(e, "adam") : VDR_OK;
}

// One optimizer step on one pair: forward, backward, Adam.  loss (host,
// nullable) is read back only when given.
extern "C" int vdr_net_train_step_device(vdr_net *N, const float *d_rhat,
                                         const float *d_target, float lr, double *loss) {
  int st = vdr_net_loss_grad_device(N, d_rhat, d_target, nullptr);
  if (st) return st;
  st = vdr_net_adam_step(N, lr, 0.9f, 0.999f, 1e-8f);
  if (st) return st;
  if (loss) {
    cudaError_t e = cudaMemcpyAsync(loss, N->n.scal + 1, sizeof(double),
                                    cudaMemcpyDeviceToHost, N->n.h->stream);
    if (!e) e = cudaStreamSynchronize(N->n.h->stream);
    if (e) return cuda_fail(e, "loss");
  }
  return VDR_OK;
}

extern "C" int vdr_net_set_smoothing(vdr_net *N, int steps, double omega) {
  int st = net_check(N);
  if (st) return st;
  if (steps < 0 || steps > 8 || !(omega > 0.0) || !(omega <= 2.0)) {
    set_error("vdr_net_set_smoothing: steps 0..8, omega in (0, 2]");
    return VDR_BAD_ARGUMENT;
  }
  N->n.smooth_steps = steps;
  N->n.smooth_omega = omega;
  return VDR_OK;
}

extern "C" int vdr_net_precondition_device(vdr_net *N, const double *d_in, double *d_out) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  Handle &h = *n.h;
  if (!d_in || !d_out || !n.features_set) {
    set_error("vdr_net_precondition_device: bad arguments or features not set");
    return VDR_BAD_ARGUMENT;
  }
  if ((st = prepare_operator(h))) return st;
  jacobi_out<<<grid_for(h.N, 256), 256, 0, h.stream>>>(d_in, h.dinv, h.mask, d_out, h.N);
  count_launches(1);
  cudaError_t e = net_enqueue(&n, d_in, d_out, nullptr, nullptr, h.stream);
  return e ? cuda_fail(e, "precondition") : VDR_OK;
}

extern "C" int vdr_solve_learned_device(vdr_handle *H, vdr_net *N, const double *d_b,
                                        double *d_x, double tol, int itmax,
                                        int stall_window, int *iter, double *err,
                                        int *fell_back) {
  int st = net_check(N);
  if (st) return st;
  Net &n = N->n;
  if (!H || &handle_of(H) != n.h || !d_b || !d_x || !n.features_set) {
    set_error("vdr_solve_learned_device: bad arguments or features not set");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = *n.h;
  if ((st = prepare_operator(h))) return st;
  Precond pc{net_enqueue, &n, net_enqueue_launches(n)};
  int it1 = 0;
  double e1 = 0.0;
  st = solve_device(h, VDR_SOLVER_BICGSTAB, d_b, d_x, tol, itmax, &it1, &e1, &pc,
                    stall_window);
  if (fell_back) *fell_back = 0;
  if ((st == VDR_NOT_CONVERGED || st == VDR_BREAKDOWN) && it1 < itmax) {
    // stalled or broke down: plain Jacobi-BiCGStab from the current iterate
    int it2 = 0;
    double e2 = 0.0;
    const int rest = itmax - it1;
    st = solve_device(h, VDR_SOLVER_BICGSTAB, d_b, d_x, tol, rest, &it2, &e2);
    it1 += it2;
    e1 = e2;
    if (fell_back) *fell_back = 1;
  }
  if (iter) *iter = it1;
  if (err) *err = e1;
  return st;
}

extern "C" int vdr_solve_gcr_device(vdr_handle *H, vdr_net *N, const double *d_b,
                                    double *d_x, double tol, int itmax, int restart,
                                    int stall_window, int *iter, double *err,
                                    int *fell_back) {
  if (!H || !d_b || !d_x) {
    set_error("vdr_solve_gcr_device: null argument");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = handle_of(H);
  cudaError_t e = cudaSetDevice(h.device);
  if (e) return cuda_fail(e, "cudaSetDevice");
  if (N && (N->n.h != &h || !N->n.features_set)) {
    set_error("vdr_solve_gcr_device: network of another handle, or features not set");
    return VDR_BAD_ARGUMENT;
  }
  int st = prepare_operator(h);
  if (st) return st;
  Precond pc{net_enqueue, N ? &N->n : nullptr, N ? net_enqueue_launches(N->n) : 0};
  int it1 = 0;
  double e1 = 0.0;
  st = solve_gcr_device(h, d_b, d_x, tol, itmax, restart, N ? &pc : nullptr,
                        stall_window, &it1, &e1);
  if (fell_back) *fell_back = 0;
  if (N && (st == VDR_NOT_CONVERGED || st == VDR_BREAKDOWN) && it1 < itmax) {
    int it2 = 0;
    double e2 = 0.0;
    st = solve_device(h, VDR_SOLVER_BICGSTAB, d_b, d_x, tol, itmax - it1, &it2, &e2);
    it1 += it2;
    e1 = e2;
    if (fell_back) *fell_back = 1;
  }
  if (iter) *iter = it1;
  if (err) *err = e1;
  return st;
}

extern "C" int vdr_solve_learned_hybrid_device(vdr_handle *H, vdr_net *N,
                                               const double *d_b, double *d_x,
                                               double tol, int itmax, int learned_steps,
                                               int *iter, double *err) {
  if (!H || !N || !d_b || !d_x || learned_steps < 1 ||
      learned_steps > GCR_MAX_RESTART) {
    set_error("vdr_solve_learned_hybrid_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = handle_of(H);
  cudaError_t e = cudaSetDevice(h.device);
  if (e) return cuda_fail(e, "cudaSetDevice");
  if (N->n.h != &h || !N->n.features_set) {
    set_error("vdr_solve_learned_hybrid_device: network of another handle, or features not set");
    return VDR_BAD_ARGUMENT;
  }
  int st = prepare_operator(h);
  if (st) return st;
  Precond pc{net_enqueue, &N->n, net_enqueue_launches(N->n)};
  int it1 = 0, it2 = 0;
  double e1 = 0.0;
  st = solve_gcr_device(h, d_b, d_x, tol, std::min(learned_steps, itmax), learned_steps,
                        &pc, 0, &it1, &e1);
  if (st == VDR_NOT_CONVERGED || st == VDR_BREAKDOWN) {
    st = solve_device(h, VDR_SOLVER_BICGSTAB, d_b, d_x, tol, std::max(0, itmax - it1),
                      &it2, &e1);
  }
  if (iter) *iter = it1 + it2;
  if (err) *err = e1;
  return st;
}

extern "C" int vdr_solve_gcr_record_device(vdr_handle *H, vdr_net *N, const double *d_b,
                                           double *d_x, double tol, int itmax, int restart,
                                           double *d_hist, int max_hist, int *n_hist,
                                           int *iter, double *err) {
  if (!H || !d_b || !d_x || !d_hist || max_hist < 1 || !n_hist) {
    set_error("vdr_solve_gcr_record_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = handle_of(H);
  cudaError_t e = cudaSetDevice(h.device);
  if (e) return cuda_fail(e, "cudaSetDevice");
  if (N && (N->n.h != &h || !N->n.features_set)) {
    set_error("vdr_solve_gcr_record_device: network of another handle, or features not set");
    return VDR_BAD_ARGUMENT;
  }
  int st = prepare_operator(h);
  if (st) return st;
  Precond pc{net_enqueue, N ? &N->n : nullptr, N ? net_enqueue_launches(N->n) : 0};
  return solve_gcr_device(h, d_b, d_x, tol, itmax, restart, N ? &pc : nullptr, 0, iter,
                          err, d_hist, max_hist, n_hist);
}

extern "C" int vdr_solve_record_device(vdr_handle *H, const double *d_b, double *d_x,
                                       double tol, int itmax, double *d_hist,
                                       int max_hist, int *n_hist, int *iter,
                                       double *err) {
  if (!H || !d_b || !d_x || !d_hist || max_hist < 1 || !n_hist) {
    set_error("vdr_solve_record_device: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  Handle &h = handle_of(H);
  cudaError_t e = cudaSetDevice(h.device);
  if (e) return cuda_fail(e, "cudaSetDevice");
  int st = prepare_operator(h);
  if (st) return st;
  const int saved = h.opt.iters_per_graph;
  h.opt.iters_per_graph = 1;  // one iterate per graph launch
  *n_hist = 0;
  st = solve_device(h, VDR_SOLVER_BICGSTAB, d_b, d_x, tol, itmax, iter, err, nullptr, 0,
                    d_hist, max_hist, n_hist);
  h.opt.iters_per_graph = saved;
  return st;
}
