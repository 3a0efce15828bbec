// conv_tc.cuh -- 3x3x3 convolution (zero padding, bias, ReLU) as an
// implicit GEMM on the fifth-generation tensor cores: tcgen05.mma (BF16
// operands, FP32 accumulator in tensor memory), operands staged in shared
// memory by TMA and bulk copies, one elected thread issuing the MMAs.
//
// Tile: G stacked planes of 128 voxels = 8 consecutive x by 16 consecutive
// y, at z0 .. z0+G-1; per plane a GEMM with M = 128 (voxels), N = COUT,
// K = 27 taps x CIN and its own FP32 accumulator in TMEM.  For a tile the
// kernel loads, per input part, the halo slab x0-1..x0+8, y0-1..y0+16,
// z0-1..z0+G (10 x 18 x (G+2) voxels, all C channels of a voxel as one row
// of 2C bytes) with one 4-D TMA box; voxels outside the grid are filled
// with zeros by the TMA unit, which is the convolution's zero padding.  The
// box lands in shared memory in the K-major swizzled layout of its row
// width (2C = 32, 64 or 128 bytes: the 32B/64B/128B swizzle modes), rows
// in voxel order [z][y][x].  A tap (dx, dy, dz) of plane g is then the same
// slab read from a start address shifted by ((g + dz) 18 + dy) 10 + dx
// rows: the 8 x-voxels of one y row are 8 consecutive rows, consecutive y
// rows are 10 rows apart (the descriptor's stride offset), and because the
// tensor cores, like the TMA unit, swizzle on absolute shared-memory
// address bits, a shifted start reads the rows the TMA unit wrote -- no
// im2col copy, one TMA box per part per tile.  The MMAs of a tap go to the
// G planes in turn, so consecutive MMAs write different accumulators and
// the tensor pipe overlaps them (one plane's 27 x CIN/16 MMAs alone form a
// dependent chain), and one load serves G planes.  G (8, 4, 2 or 1) is the
// largest that fits the TMEM (512 columns for two sets of G accumulators)
// and the shared memory.  Decoder layers read [skip | upsampled coarser
// output]: the second part comes from its own tensor (the upsampled copy)
// through a second map, into its own slab.
//
// Weights: [tap][chunk][COUT][8] BF16 in the no-swizzle K-major layout
// (core matrices of 8 output channels x 8 input channels), resident in
// shared memory when all 27 taps fit next to the slab stages, else streamed
// one tap at a time through a ring.
//
// Warp roles (192 threads): warp 0 = TMA / bulk-copy producer, warp 1 =
// TMEM owner and MMA issuer, warps 2-5 = epilogue (TMEM -> registers ->
// bias, ReLU, BF16 -> global).  Slabs are double-buffered when they fit,
// the accumulators always (two sets of G x COUT TMEM columns), so loading
// tile i+1 and the epilogue of tile i-1 overlap the MMAs of tile i.  The
// MMA issuer builds each operand descriptor once and advances only its
// start-address field.  Every mbarrier wait is bounded; a wait that runs
// out sets *err, the roles stop, outstanding copies and MMAs are drained
// (bounded too) and the TMEM is released before the kernel returns.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tc_ptx.cuh"

namespace vdr {
namespace convtc {

constexpr int TX = 8, TY = 16;             // plane: 8 x 16 voxels
constexpr int SX = TX + 2, SY = TY + 2;    // halo slab extents in x, y
constexpr int PROWS = SX * SY;             // 180 voxel rows per slab plane
constexpr int THREADS = 192;
constexpr int BUDGET = 200 * 1024;         // shared memory for slabs + weights
constexpr long long WAIT_LIMIT = 2000000000LL;  // ~1 s of clocks per wait

// Slab bytes of a part with C channels for G planes (1024-aligned for the
// swizzle).
__host__ __device__ constexpr int slab_bytes(int C, int G) {
  return C == 0 ? 0 : (PROWS * (G + 2) * 2 * C + 1023) / 1024 * 1024;
}
__host__ __device__ constexpr int tap_bytes(int cin, int cout) { return cin / 8 * cout * 16; }
// Largest G in {8, 4, 2, 1} whose two accumulator sets fit the 512 TMEM
// columns and whose `ns` slab stages plus weights (all 27 taps resident, or
// an 8-tap ring) fit the budget; 0 if none.
__host__ __device__ constexpr int fit_group(int cin1, int cin2, int cout, int ns) {
  for (int G = 8; G >= 1; G /= 2) {
    if (2 * G * cout > 512) continue;
    const int slab = slab_bytes(cin1, G) + slab_bytes(cin2, G);
    const int wt = tap_bytes(cin1 + cin2, cout);
    const int w = (27 * wt + ns * slab <= BUDGET) ? 27 * wt : 8 * wt;
    if (ns * slab + w <= BUDGET) return G;
  }
  return 0;
}
// Double-buffered slabs when they allow G >= 2 (or as large a G as one
// stage would), else one stage with the larger G.  Measured: double
// buffering matters more than a larger G (G = 4 with one stage instead of
// G = 2 with two took the [16 | 32] -> 16 layer from 157 to 227 us, G = 8
// with one stage the 32 -> 32 layer from 22.6 to 30.7 us).
__host__ __device__ constexpr int stages_of(int cin1, int cin2, int cout) {
  return (fit_group(cin1, cin2, cout, 2) >= 2 ||
          fit_group(cin1, cin2, cout, 2) >= fit_group(cin1, cin2, cout, 1))
             ? 2
             : 1;
}
__host__ __device__ constexpr int group_of(int cin1, int cin2, int cout) {
  return fit_group(cin1, cin2, cout, stages_of(cin1, cin2, cout));
}
// Descriptor layout code of a K-major operand whose rows are `row_bytes`
// wide: 32B, 64B or 128B swizzle.
__host__ __device__ constexpr int swizzle_code(int row_bytes) {
  return row_bytes == 128 ? 2 : (row_bytes == 64 ? 4 : 6);
}

struct Args {
  int W, H, D;
  int tiles_x, tiles_y, ntiles;  // ntiles = tiles_x tiles_y ceil(D / G)
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
  static constexpr int NS = stages_of(CIN1, CIN2, COUT);
  static constexpr int G = group_of(CIN1, CIN2, COUT);
  static constexpr int SLAB1 = slab_bytes(CIN1, G), SLAB2 = slab_bytes(CIN2, G);
  static constexpr int SLAB = SLAB1 + SLAB2;
  static constexpr int TXB = PROWS * (G + 2) * 2 * (CIN1 + CIN2);  // bytes the boxes land
  static constexpr int WTAP = tap_bytes(CIN1 + CIN2, COUT);  // one tap's weights
  static constexpr bool RES = 27 * WTAP + NS * SLAB <= BUDGET;
  static constexpr int NW = RES ? 27 : 8;       // weight slots
  static constexpr int ACC = 2 * G * COUT;      // columns of the two accumulator sets
  static constexpr int TMEM_COLS =
      ACC <= 32 ? 32 : (ACC <= 64 ? 64 : (ACC <= 128 ? 128 : (ACC <= 256 ? 256 : 512)));
  static constexpr int NBAR = 2 * NS + (RES ? 1 : 2 * NW) + 4 + 1;
  static constexpr int SMEM = 1024 + NS * SLAB + NW * WTAP + NBAR * 8 + 16;
  static_assert(CIN1 % 16 == 0 && CIN2 % 16 == 0, "K steps of 16 channels");
  static_assert((CIN1 == 16 || CIN1 == 32 || CIN1 == 64) &&
                    (CIN2 == 0 || CIN2 == 16 || CIN2 == 32 || CIN2 == 64),
                "voxel rows of 32, 64 or 128 bytes (one swizzle atom wide)");
  static_assert(COUT % 16 == 0 && COUT >= 16 && COUT <= 256, "M = 128 needs N % 16 == 0");
  static_assert(G >= 1 && ACC <= 512, "a plane group fits the TMEM and shared memory");
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
        const int ty = r % a.tiles_y, tz = r / a.tiles_y;
        const int x0 = tx * TX - 1, y0 = ty * TY - 1, z0 = tz * S::G - 1;
        tc::mbar_arrive_expect_tx(bar(B_SFULL + s), S::TXB);
        const uint32_t dst = tc::smem_u32(slab + s * S::SLAB);
        tc::tma_load_4d(dst, &map1, 0, x0, y0, z0, bar(B_SFULL + s));
        if (CIN2 > 0) tc::tma_load_4d(dst + S::SLAB1, &map2, 0, x0, y0, z0, bar(B_SFULL + s));
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
        const uint32_t dtm = tmem + (uint32_t)(b * S::G * COUT);  // plane g at + g COUT
        // Descriptors are built once; an MMA's operand start is the base
        // descriptor plus the byte offset / 16 in the start-address field
        // (bits 0-13; shared-memory offsets < 256 KB never carry out of it).
        const uint64_t a1d = tc::smem_desc_sw(sbase, SX * 2 * CIN1, swizzle_code(2 * CIN1));
        const uint64_t a2d =
            tc::smem_desc_sw(sbase + S::SLAB1, SX * 2 * (CIN2 > 0 ? CIN2 : 16),
                             swizzle_code(CIN2 > 0 ? 2 * CIN2 : 32));
        const uint64_t bdd = tc::smem_desc(tc::smem_u32(wbuf), COUT * 16, 128);
#pragma unroll 3
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
          const int row0 = (dz * SY + dy) * SX + dx;  // the tap's first slab row
          const uint64_t bt = bdd + (uint64_t)((w * S::WTAP) >> 4);
          // part 1: rows of 2 CIN1 bytes, K steps of 16 channels (32 bytes);
          // plane g's rows start PROWS g rows further into the slab
          const uint64_t at1 = a1d + (uint64_t)((row0 * 2 * CIN1) >> 4);
#pragma unroll
          for (int j = 0; j < CIN1 / 16; j++)
#pragma unroll
            for (int g = 0; g < S::G; g++)
              tc::mma_bf16(dtm + g * COUT,
                           at1 + (uint64_t)((g * PROWS * 2 * CIN1 + 32 * j) >> 4),
                           bt + (uint64_t)((2 * j * COUT * 16) >> 4), IDESC,
                           (tap > 0 || j > 0) ? 1u : 0u);
          if (CIN2 > 0) {
            const uint64_t at2 = a2d + (uint64_t)((row0 * 2 * CIN2) >> 4);
#pragma unroll
            for (int j = 0; j < CIN2 / 16; j++)
#pragma unroll
              for (int g = 0; g < S::G; g++)
                tc::mma_bf16(dtm + g * COUT,
                             at2 + (uint64_t)((g * PROWS * 2 * CIN2 + 32 * j) >> 4),
                             bt + (uint64_t)(((S::KC1 + 2 * j) * COUT * 16) >> 4), IDESC,
                             1u);
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
      // the whole warp waits, so that the collective TMEM loads below are
      // reached by all 32 lanes or by none
      const bool got = tc::mbar_wait(bar(B_AFULL + b), bph, WAIT_LIMIT);
      if (!__all_sync(0xffffffffu, got)) {
        if (lane == 0) atomicOr(a.err, 1);
        break;
      }
      tc::fence_after();
      const int tx = t % a.tiles_x, r = t / a.tiles_x;
      const int ty = r % a.tiles_y, tz = r / a.tiles_y;
      const int x = tx * TX + (row & 7), y = ty * TY + (row >> 3);
#pragma unroll 1
      for (int g = 0; g < S::G; g++) {
        const int z = tz * S::G + g;
        if (z >= a.D) break;  // uniform over the warp
        uint32_t v[COUT];
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
          uint32_t r16[16];
          tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) +
                            (uint32_t)((b * S::G + g) * COUT + c0),
                        r16);
          tc::tmem_wait_ld();
#pragma unroll
          for (int k = 0; k < 16; k++) v[c0 + k] = r16[k];
        }
        if (x >= a.W || y >= a.H) continue;
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
      tc::fence_before();
      tc::mbar_arrive(bar(B_AEMPTY + b));
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
