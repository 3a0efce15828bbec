// conv_tc.cuh -- 3x3x3 convolution (zero padding, bias, ReLU) as an
// implicit GEMM on the fifth-generation tensor cores: tcgen05.mma (BF16
// operands, FP32 accumulator in tensor memory), operands staged in shared
// memory by TMA and bulk copies, one elected thread issuing the MMAs.
//
// Tile: 128 voxels = 8 consecutive x by 16 consecutive y at one z; GEMM
// M = 128 (voxels), N = COUT, K = 27 taps x CIN.  For a tile the kernel
// loads, per 16-byte chunk of 8 input channels, the halo slab x0-1..x0+8,
// y0-1..y0+16, z-1..z+1 with one 4-D TMA box (10 x 18 x 3 voxels x 16
// bytes); voxels outside the grid are filled with zeros by the TMA unit,
// which is the convolution's zero padding.  In shared memory the slab is
// [chunk][z][y][x][8 channels], i.e. the canonical no-swizzle K-major
// layout with 16-byte rows: the 8 x-voxels of one y row form a core matrix
// and consecutive y rows are 160 bytes apart (the descriptor's stride
// offset), so every one of the 27 taps is the same slab read from a start
// address shifted by 16 dx + 160 dy + 2880 dz bytes -- no im2col copy.
// Decoder layers read [skip | upsampled coarser output]: the second part
// comes from its own tensor (the upsampled copy) through a second map.
//
// Weights: [tap][chunk][COUT][8] BF16 (core matrices of 8 output channels
// x 8 input channels), resident in shared memory when all 27 taps fit next
// to two slab stages, else streamed one tap at a time through a ring.
//
// Warp roles (192 threads): warp 0 = TMA / bulk-copy producer, warp 1 =
// TMEM owner and MMA issuer, warps 2-5 = epilogue (TMEM -> registers ->
// bias, ReLU, BF16 -> global).  Slabs are double-buffered when they fit,
// the accumulator always (two COUT-column halves of the TMEM allocation),
// so loading tile i+1 and the epilogue of tile i-1 overlap the MMAs of
// tile i.  Every mbarrier wait is bounded; a wait that runs out sets *err,
// the roles stop, outstanding copies and MMAs are drained (bounded too) and
// the TMEM is released before the kernel returns.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tc_ptx.cuh"

namespace vdr {
namespace convtc {

constexpr int TX = 8, TY = 16;             // tile: 8 x 16 voxels at one z
constexpr int SX = TX + 2, SY = TY + 2;    // halo slab extents
constexpr int SLAB_ROW = 16;               // bytes per voxel per chunk
constexpr int SLAB_Y = SX * SLAB_ROW;      // 160: y stride (descriptor SBO)
constexpr int SLAB_Z = SY * SLAB_Y;        // 2880: z stride
constexpr int SLAB_CHUNK_TX = 3 * SLAB_Z;  // 8640 bytes a TMA box writes
constexpr int SLAB_CHUNK = 8704;           // chunk stride, 128-byte aligned
constexpr int THREADS = 192;
constexpr long long WAIT_LIMIT = 2000000000LL;  // ~1 s of clocks per wait

struct Args {
  int W, H, D;
  int tiles_x, tiles_y, ntiles;
  const __nv_bfloat16 *wpk;  // [27][KC][COUT][8]
  const float *bias;         // [COUT]
  __nv_bfloat16 *out;        // [V][COUT]
  int relu;
  int *err;                  // bit 0: a wait ran out
  const int *skip, *skip2;
};

template <int CIN1, int CIN2, int COUT>
struct Shape {
  static constexpr int KC1 = CIN1 / 8, KC2 = CIN2 / 8, KC = KC1 + KC2;
  static constexpr int SLAB = KC * SLAB_CHUNK;
  static constexpr int WTAP = KC * COUT * 16;  // bytes of one tap's weights
  static constexpr int BUDGET = 200 * 1024;
  static constexpr bool RES = 27 * WTAP + 2 * SLAB <= BUDGET;
  static constexpr int NW = RES ? 27 : 8;       // weight slots
  static constexpr int NS = (RES || 2 * SLAB + NW * WTAP <= BUDGET) ? 2 : 1;
  static constexpr int TMEM_COLS = 2 * COUT < 32 ? 32 : 2 * COUT;
  static constexpr int NBAR = 2 * NS + (RES ? 1 : 2 * NW) + 4 + 1;
  static constexpr int SMEM = 1024 + NS * SLAB + NW * WTAP + NBAR * 8 + 16;
  static_assert(CIN1 % 16 == 0 && CIN2 % 16 == 0, "K steps of 16 channels");
  static_assert(COUT % 16 == 0 && COUT >= 16 && COUT <= 256, "M = 128 needs N % 16 == 0");
  static_assert(SMEM <= 227 * 1024, "shared memory");
};

template <int CIN1, int CIN2, int COUT>
__global__ void __launch_bounds__(THREADS, 1)
    conv3_tc_kernel(const __grid_constant__ CUtensorMap map1,
                    const __grid_constant__ CUtensorMap map2, Args a) {
  using S = Shape<CIN1, CIN2, COUT>;
  if ((a.skip && *(volatile const int *)a.skip) ||
      (a.skip2 && *(volatile const int *)a.skip2))
    return;
  extern __shared__ unsigned char dyn_smem[];
  // 1024-aligned base for the slabs and weights
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(dyn_smem) + 1023) & ~(uintptr_t)1023);
  unsigned char *slab = base;
  unsigned char *wbuf = base + S::NS * S::SLAB;
  uint64_t *bars = reinterpret_cast<uint64_t *>(wbuf + S::NW * S::WTAP);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + S::NBAR);
  // barrier indices
  const int B_SFULL = 0, B_SEMPTY = S::NS;
  const int B_WFULL = 2 * S::NS;
  const int B_WEMPTY = B_WFULL + (S::RES ? 1 : S::NW);
  const int B_AFULL = B_WEMPTY + (S::RES ? 0 : S::NW);
  const int B_AEMPTY = B_AFULL + 2;
  const int B_DRAIN = B_AEMPTY + 2;
  auto bar = [&](int i) { return tc::smem_u32(bars + i); };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < S::NS; i++) {
      tc::mbar_init(bar(B_SFULL + i), 1);
      tc::mbar_init(bar(B_SEMPTY + i), 1);
    }
    if (S::RES) {
      tc::mbar_init(bar(B_WFULL), 1);
    } else {
      for (int i = 0; i < S::NW; i++) {
        tc::mbar_init(bar(B_WFULL + i), 1);
        tc::mbar_init(bar(B_WEMPTY + i), 1);
      }
    }
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(bar(B_AFULL + i), 1);
      tc::mbar_init(bar(B_AEMPTY + i), 128);
    }
    tc::mbar_init(bar(B_DRAIN), 1);
    tc::mbar_init_fence();
  }
  if (warp == 1) tc::tmem_alloc(tc::smem_u32(tslot), S::TMEM_COLS);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    // ------------------------------------------------ producer
    if (lane == 0) {
      tc::prefetch_tensormap(&map1);
      if (CIN2 > 0) tc::prefetch_tensormap(&map2);
      bool ok = true;
      if (S::RES) {
        tc::mbar_arrive_expect_tx(bar(B_WFULL), 27 * S::WTAP);
        tc::bulk_load(tc::smem_u32(wbuf), a.wpk, 27 * S::WTAP, bar(B_WFULL));
      }
      int it = 0;
      long wc = 0;
      for (int t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x, it++) {
        const int s = it % S::NS;
        const uint32_t ph = (uint32_t)(it / S::NS) & 1u;
        if (!tc::mbar_wait(bar(B_SEMPTY + s), ph ^ 1u, WAIT_LIMIT)) {
          ok = false;
          break;
        }
        const int tx = t % a.tiles_x, r = t / a.tiles_x;
        const int ty = r % a.tiles_y, z = r / a.tiles_y;
        const int x0 = tx * TX - 1, y0 = ty * TY - 1, z0 = z - 1;
        tc::mbar_arrive_expect_tx(bar(B_SFULL + s), S::KC * SLAB_CHUNK_TX);
        const uint32_t dst = tc::smem_u32(slab + s * S::SLAB);
#pragma unroll 1
        for (int kc = 0; kc < S::KC1; kc++)
          tc::tma_load_4d(dst + kc * SLAB_CHUNK, &map1, 8 * kc, x0, y0, z0, bar(B_SFULL + s));
#pragma unroll 1
        for (int kc = 0; kc < S::KC2; kc++)
          tc::tma_load_4d(dst + (S::KC1 + kc) * SLAB_CHUNK, &map2, 8 * kc, x0, y0, z0,
                          bar(B_SFULL + s));
        if (!S::RES) {
#pragma unroll 1
          for (int tap = 0; tap < 27; tap++, wc++) {
            const int w = (int)(wc % S::NW);
            const uint32_t wph = (uint32_t)(wc / S::NW) & 1u;
            if (!tc::mbar_wait(bar(B_WEMPTY + w), wph ^ 1u, WAIT_LIMIT)) {
              ok = false;
              break;
            }
            tc::mbar_arrive_expect_tx(bar(B_WFULL + w), S::WTAP);
            tc::bulk_load(tc::smem_u32(wbuf + w * S::WTAP),
                          reinterpret_cast<const unsigned char *>(a.wpk) + (size_t)tap * S::WTAP,
                          S::WTAP, bar(B_WFULL + w));
          }
        }
      }
      if (!ok) atomicOr(a.err, 1);
      // drain: every copy issued has landed before the block may exit
      for (int k = (it > S::NS ? it - S::NS : 0); k < it; k++)
        tc::mbar_wait(bar(B_SFULL + k % S::NS), (uint32_t)(k / S::NS) & 1u, WAIT_LIMIT);
      if (S::RES) {
        tc::mbar_wait(bar(B_WFULL), 0u, WAIT_LIMIT);
      } else {
        for (long k = (wc > S::NW ? wc - S::NW : 0); k < wc; k++)
          tc::mbar_wait(bar(B_WFULL + (int)(k % S::NW)), (uint32_t)(k / S::NW) & 1u,
                        WAIT_LIMIT);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t IDESC = tc::idesc_bf16_f32(128, COUT);
      bool ok = true;
      if (S::RES && !tc::mbar_wait(bar(B_WFULL), 0u, WAIT_LIMIT)) ok = false;
      int it = 0;
      long wc = 0;
      for (int t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x, it++) {
        const int s = it % S::NS;
        const uint32_t ph = (uint32_t)(it / S::NS) & 1u;
        const int b = it & 1;
        const uint32_t bph = (uint32_t)(it >> 1) & 1u;
        if (!tc::mbar_wait(bar(B_AEMPTY + b), bph ^ 1u, WAIT_LIMIT) ||
            !tc::mbar_wait(bar(B_SFULL + s), ph, WAIT_LIMIT)) {
          ok = false;
          break;
        }
        tc::fence_after();
        const uint32_t sbase = tc::smem_u32(slab + s * S::SLAB);
        const uint32_t dtm = tmem + (uint32_t)(b * COUT);
#pragma unroll 1
        for (int tap = 0; tap < 27; tap++) {
          int w = tap;
          if (!S::RES) {
            w = (int)(wc % S::NW);
            if (!tc::mbar_wait(bar(B_WFULL + w), (uint32_t)(wc / S::NW) & 1u, WAIT_LIMIT)) {
              ok = false;
              break;
            }
            tc::fence_after();
          }
          const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;  // 0..2
          const uint32_t a0 = sbase + dz * SLAB_Z + dy * SLAB_Y + dx * SLAB_ROW;
          const uint32_t b0 = tc::smem_u32(wbuf + w * S::WTAP);
#pragma unroll
          for (int j = 0; j < S::KC / 2; j++) {
            const uint64_t ad = tc::smem_desc(a0 + 2 * j * SLAB_CHUNK, SLAB_CHUNK, SLAB_Y);
            const uint64_t bd = tc::smem_desc(b0 + 2 * j * COUT * 16, COUT * 16, 128);
            tc::mma_bf16(dtm, ad, bd, IDESC, (tap > 0 || j > 0) ? 1u : 0u);
          }
          if (!S::RES) {
            tc::commit(bar(B_WEMPTY + w));
            wc++;
          }
        }
        if (!ok) break;
        tc::commit(bar(B_SEMPTY + s));
        tc::commit(bar(B_AFULL + b));
      }
      if (!ok) atomicOr(a.err, 1);
      // drain: every MMA issued has completed before the TMEM is released
      tc::commit(bar(B_DRAIN));
      tc::mbar_wait(bar(B_DRAIN), 0u, WAIT_LIMIT);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------ epilogue
    const int q = warp & 3;  // TMEM sub-partition: lanes 32q .. 32q + 31
    const int row = 32 * q + lane;
    float bias[COUT];
#pragma unroll
    for (int c = 0; c < COUT; c++) bias[c] = a.bias ? __ldg(a.bias + c) : 0.f;
    int it = 0;
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x, it++) {
      const int b = it & 1;
      const uint32_t bph = (uint32_t)(it >> 1) & 1u;
      // the whole warp waits, so that the collective TMEM load below is
      // reached by all 32 lanes or by none
      const bool got = tc::mbar_wait(bar(B_AFULL + b), bph, WAIT_LIMIT);
      if (!__all_sync(0xffffffffu, got)) {
        if (lane == 0) atomicOr(a.err, 1);
        break;
      }
      tc::fence_after();
      uint32_t v[COUT];
#pragma unroll
      for (int c0 = 0; c0 < COUT; c0 += 16) {
        uint32_t r16[16];
        tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * COUT + c0), r16);
        tc::tmem_wait_ld();
#pragma unroll
        for (int k = 0; k < 16; k++) v[c0 + k] = r16[k];
      }
      tc::fence_before();
      tc::mbar_arrive(bar(B_AEMPTY + b));
      const int tx = t % a.tiles_x, r = t / a.tiles_x;
      const int ty = r % a.tiles_y, z = r / a.tiles_y;
      const int x = tx * TX + (row & 7), y = ty * TY + (row >> 3);
      if (x < a.W && y < a.H) {
        const long vox = (long)x + (long)a.W * ((long)y + (long)a.H * z);
        uint4 *o = reinterpret_cast<uint4 *>(a.out + vox * COUT);
#pragma unroll
        for (int c8 = 0; c8 < COUT / 8; c8++) {
          uint32_t pk[4];
#pragma unroll
          for (int k = 0; k < 4; k++) {
            float f0 = __uint_as_float(v[8 * c8 + 2 * k]) + bias[8 * c8 + 2 * k];
            float f1 = __uint_as_float(v[8 * c8 + 2 * k + 1]) + bias[8 * c8 + 2 * k + 1];
            if (a.relu) {
              f0 = fmaxf(f0, 0.f);
              f1 = fmaxf(f1, 0.f);
            }
            __nv_bfloat162 h = __floats2bfloat162_rn(f0, f1);
            pk[k] = *reinterpret_cast<uint32_t *>(&h);
          }
          o[c8] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, S::TMEM_COLS);
  }
}

}  // namespace convtc
}  // namespace vdr
