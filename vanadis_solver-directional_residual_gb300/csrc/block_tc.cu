// block_tc.cu -- the 64-column block apply Y += A X on the fifth-generation
// tensor cores, for meshes in the canonical structured numbering.
//
// The mma.sync applies of block.cu contract each 8 x 8 element matrix with
// its 8 node rows; they are bound by the instructions that gather, split
// and scatter per element.  Here a CTA takes a box of 4 x 4 x 4 elements
// and its 5 x 5 x 5 = 125 node rows, assembles the box operator A_box
// (125 x 125: the couplings of the box's own elements) in tensor memory,
// and computes D = A_box X_box for all 64 columns with tcgen05.mma
// (kind::tf32, M = 128 rows = box nodes, K = 128 box nodes, FP32
// accumulators in TMEM):
//
//   X_box   the 125 node rows (64 floats each) arrive by two 4-D TMA boxes
//           (32 columns x 5 x 5 x 5 nodes, 128-byte swizzle) from the
//           node-major block vector viewed as (64, nax, nay, naz); nodes
//           outside the mesh arrive as zeros.  TF32 operands must be
//           K-major (an MN-major TF32 B operand measured all zeros), so the
//           split pass writes B transposed: row n = column n of X, the 125
//           box nodes along K (lane = node: each store of a warp fills one
//           128-byte row, no bank conflicts).  Heads are truncated to TF32
//           (top 10 mantissa bits), tails are the exact FP32 remainders.
//   A_box   thread r of the four assembly warps owns box node r: it sums
//           node r's rows of the (up to 8) box elements around it into its
//           27 stencil couplings, writes them into its row of a shared
//           staging buffer at columns r + dx + 5 dy + 25 dz (the other
//           columns of the row stay zero), reads back the columns its warp
//           covers and stores them to TMEM lane r (tcgen05.st) as TF32 head
//           and tail.  The MMAs read A from TMEM.
//   split   D = A_hi [X_hi | X_lo] (one N = 128 MMA per K step: head and
//           tail of X side by side in B) + A_lo X_hi (N = 64): the three
//           products of split TF32, FP32-level accuracy.  Plain TF32 issues
//           A_hi X_hi alone.
//   Y       the epilogue adds the two halves of D into a shared tile laid
//           out as the TMA box, and one thread adds the tile to Y with two
//           tensor reduces (cp.reduce.async.bulk.tensor .add.f32: element-
//           wise atomic adds by the TMA unit; nodes outside the mesh are
//           skipped); nodes on box faces receive one add per box sharing
//           them.
//
// The element matrices come from the element-major FP32 copy
// Aaos[p*64 + 8i + j] (Jacobi scale folded into the columns, Dirichlet rows
// and columns zero), a box's 64 elements by two TMA boxes per box.
//
// Warp roles (576 threads, one CTA per SM, boxes strided over the grid):
// warp 0 = TMA producer, warp 1 = TMEM owner and MMA issuer, warps 2-5 = A
// assembly, warps 6-13 = X split and transpose (a 32-node K atom and 32
// columns each), warps 14-17 = epilogue; warp w
// reaches TMEM lanes 32 (w % 4) .. 32 (w % 4) + 31.  The TMA stages and D
// are double-buffered, so the load of box i+1 and the epilogue of box i-1
// overlap the MMAs of box i.  A (256 of the 512 TMEM columns) and B are
// single and handed over in two halves of K: box i's MMAs release the first
// half while the second half multiplies, and box i+1's first half (its A
// columns and its B atoms) is written meanwhile.
// Every mbarrier wait is bounded; a wait that runs out sets *err, the
// roles stop, outstanding copies and MMAs are drained (bounded too) and the
// TMEM is released before the kernel returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "tc_ptx.cuh"
#include "vdr_internal.h"

namespace vdr {
namespace blocktc {

constexpr int BE = 4, BN = 5, ROWS = BN * BN * BN;  // box: 4^3 elements, 125 nodes
// warps: 0 TMA producer, 1 MMA issuer, 2-5 A assembly, 6-13 X split, 14-17
// epilogue
constexpr int W_ASM = 2, W_SPL = 6, W_EPI = 14;
constexpr int THREADS = 32 * (W_EPI + 4);
constexpr int XREG = 16384;         // 128 rows x 128 bytes: 32 columns of the TMA stage
constexpr int XSTAGE = 2 * XREG;    // node rows as the TMA lands them
constexpr int XBYTES = 2 * 32 * 4 * ROWS;  // bytes the two TMA boxes land
constexpr int KATOM = 16384;        // B: 128 rows (columns of X) x 32 nodes x 4 bytes
constexpr int BSTAGE = 4 * KATOM;   // B: rows 0-63 head, 64-127 tail; K = 128 nodes
                                    // (atoms 0-1: first half of K, 2-3: second)
constexpr int SPITCH = 100;         // staging row pitch (floats): conflict-free rows
constexpr int STAGING = ROWS * SPITCH * 4;
constexpr int ETILE = 64 * 128;     // element matrices: 64 box elements x 32 floats
constexpr int ESTAGE = 2 * ETILE;   // [rows 0-3 | rows 4-7] of every box element
constexpr int YSTAGE = 2 * XREG;    // the D tile in the TMA box layout, for the reduce
constexpr int NBAR = 15;
constexpr int SMEM = 1024 + 2 * XSTAGE + BSTAGE + YSTAGE + ESTAGE + STAGING + NBAR * 8 + 8;
static_assert(SMEM <= 232448, "shared memory per block");
constexpr int TMEM_COLS = 512;
constexpr uint32_t A_HI = 0, A_LO = 128, D_BASE = 256;  // TMEM columns
constexpr long long WAIT_LIMIT = 2000000000LL;         // ~1 s of clocks per wait
// barrier indices
// AFULL / AFREE: one per half of K, covering that half's A columns (TMEM)
// and B rows' K atoms (shared memory)
constexpr int B_XFULL = 0, B_XEMPTY = 2, B_AFULL = 4, B_AFREE = 6, B_DFULL = 8,
              B_DEMPTY = 10, B_DRAIN = 12, B_EFULL = 13, B_EEMPTY = 14;

struct Args {
  const float *A;             // Aaos, [E][64]
  float *Y;                   // [N][64], accumulated
  const unsigned char *mask;  // optional: Dirichlet rows of X read as zero, of Y get nothing
  int nax, nay, naz;          // nodes per direction
  int nbx, nby, nbox;         // boxes in x, y; all boxes
  const int *skip;            // nonzero: return at once (a finished inner solve)
  int *err;                   // bit 0: a wait ran out
};

// Instruction descriptor of kind::tf32: FP32 accumulator (bits 4-5), A and
// B TF32 (format 2 in bits 7-9 and 10-12), both K-major, N >> 3 in bits
// 17-22, M >> 4 in 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
// D[tmem] (+)= A[tmem] * B[desc]^T, kind::tf32, one CTA, issued by one thread.
__device__ __forceinline__ void mma_tf32_ts(uint32_t d, uint32_t a, uint64_t bdesc,
                                            uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, q;\n}\n" ::"r"(d),
      "r"(a), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Whole warp: 16 consecutive 32-bit columns of the warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]),
      "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]),
      "r"(r[14]), "r"(r[15])
      : "memory");
}
// Element-wise atomic add of a shared-memory box into the 4-D tensor (out
// of range elements are skipped), tracked by the issuing thread's bulk group.
__device__ __forceinline__ void tma_reduce_add_4d(const CUtensorMap *map, uint32_t src, int c0,
                                                  int c1, int c2, int c3) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.4d.global.shared::cta.add.tile.bulk_group"
      " [%0, {%2, %3, %4, %5}], [%1];" ::"l"((uint64_t)map),
      "r"(src), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Waits until the bulk operations this thread committed have read their
// shared-memory sources.
__device__ __forceinline__ void bulk_wait_read0() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// Named barrier 1 over the four epilogue warps; the _or form returns
// whether `pred` held for any of their threads (so that a timeout seen by
// one warp stops all four at the same point).
__device__ __forceinline__ void epi_sync() {
  asm volatile("bar.sync 1, 128;" ::: "memory");
}
__device__ __forceinline__ bool epi_sync_or(bool pred) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, 128, p;\n"
      " selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)pred)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
// Split TF32 by truncation: the head keeps the top 10 mantissa bits (an
// exact TF32 value), the tail v - head is exact in FP32 and loses at most
// 2^-10 of itself (under 2^-20 of v) when the tensor core reads it as TF32.
__device__ __forceinline__ uint32_t tf32_head(float f) {
  return __float_as_uint(f) & 0xFFFFE000u;
}
__device__ __forceinline__ uint32_t tf32_tail(float f, uint32_t head) {
  return __float_as_uint(f - __uint_as_float(head));
}
// Local index of the HEX8 corner (x, y, z): 0 (0,0,0), 1 (1,0,0), 2 (1,1,0),
// 3 (0,1,0), and + 4 at z = 1.
__host__ __device__ constexpr int corner(int x, int y, int z) {
  return 4 * z + (y ? (x ? 2 : 3) : (x ? 1 : 0));
}
__host__ __device__ constexpr int cx(int j) { return ((j & 3) == 1 || (j & 3) == 2) ? 1 : 0; }
__host__ __device__ constexpr int cy(int j) { return (j & 3) >> 1; }
__host__ __device__ constexpr int cz(int j) { return j >> 2; }

template <bool SPLIT>
__global__ void __launch_bounds__(THREADS, 1)
    block_apply_tc_kernel(const __grid_constant__ CUtensorMap xmap,
                          const __grid_constant__ CUtensorMap ymap,
                          const __grid_constant__ CUtensorMap amap, Args a) {
  if (a.skip && *(volatile const int *)a.skip) return;
  extern __shared__ unsigned char dsm[];
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(dsm) + 1023) &
                                        ~static_cast<uintptr_t>(1023));
  unsigned char *xst = base;                // two TMA stages: node rows
  unsigned char *bst = base + 2 * XSTAGE;   // B (transposed, split)
  unsigned char *yst = bst + BSTAGE;        // D tile for the TMA reduce
  unsigned char *est = yst + YSTAGE;        // element matrices of a box (TMA)
  float *staging = reinterpret_cast<float *>(est + ESTAGE);
  uint64_t *bars = reinterpret_cast<uint64_t *>(est + ESTAGE + STAGING);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + NBAR);
  auto bar = [&](int i) { return tc::smem_u32(bars + i); };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(bar(B_XFULL + i), 1);
      tc::mbar_init(bar(B_XEMPTY + i), 8);
      tc::mbar_init(bar(B_AFULL + i), 4 + 4);  // A assembly warps + split warps of the half
      tc::mbar_init(bar(B_AFREE + i), 1);
      tc::mbar_init(bar(B_DFULL + i), 1);
      tc::mbar_init(bar(B_DEMPTY + i), 4);
    }
    tc::mbar_init(bar(B_DRAIN), 1);
    tc::mbar_init(bar(B_EFULL), 1);
    tc::mbar_init(bar(B_EEMPTY), 4);
    tc::mbar_init_fence();
  }
  if (warp == 1) tc::tmem_alloc(tc::smem_u32(tslot), TMEM_COLS);
  if (warp >= W_ASM && warp < W_ASM + 4) {
    // staging rows zero (only a row's stencil columns are ever written)
    const int r = 32 * (warp & 3) + lane;
    if (r < ROWS) {
      float4 *srow = reinterpret_cast<float4 *>(staging + r * SPITCH);
      for (int i = 0; i < SPITCH / 4; i++) srow[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  } else if (warp >= W_SPL && warp < W_SPL + 4) {
    // K positions 124..127 of every B row zero: 125..127 are never written
    // and the MMA reads them (times zero columns of A)
    const int row = threadIdx.x - 32 * W_SPL;  // 0 .. 127
    *reinterpret_cast<float4 *>(bst + 3 * KATOM + row * 128 + ((7 ^ (row & 7)) << 4)) =
        make_float4(0.f, 0.f, 0.f, 0.f);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    // ------------------------------------------------ producer
    if (lane == 0) {
      tc::prefetch_tensormap(&xmap);
      bool ok = true;
      int it = 0;
      for (int b = blockIdx.x; b < a.nbox; b += gridDim.x, it++) {
        // the split of the box two back has read the stage
        const int s = it & 1;
        if (!tc::mbar_wait_sleep(bar(B_XEMPTY + s), ((uint32_t)(it >> 1) & 1u) ^ 1u, WAIT_LIMIT)) {
          ok = false;
          break;
        }
        const int bx = b % a.nbx, by = (b / a.nbx) % a.nby, bz = b / (a.nbx * a.nby);
        tc::mbar_arrive_expect_tx(bar(B_XFULL + s), XBYTES);
        const uint32_t dst = tc::smem_u32(xst + s * XSTAGE);
        tc::tma_load_4d(dst, &xmap, 0, BE * bx, BE * by, BE * bz, bar(B_XFULL + s));
        tc::tma_load_4d(dst + XREG, &xmap, 32, BE * bx, BE * by, BE * bz, bar(B_XFULL + s));
      }
      if (!ok) atomicOr(a.err, 1);
      // drain: every copy issued has landed before the block may exit
      for (int k = (it > 2 ? it - 2 : 0); k < it; k++)
        tc::mbar_wait_sleep(bar(B_XFULL + (k & 1)), (uint32_t)(k >> 1) & 1u, WAIT_LIMIT);
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t IDESC_N = idesc_tf32(128, SPLIT ? 128 : 64);
      constexpr uint32_t IDESC_64 = idesc_tf32(128, 64);
      bool ok = true;
      int it = 0;
      for (int b = blockIdx.x; b < a.nbox && ok; b += gridDim.x, it++) {
        const int s = it & 1;
        const uint32_t ph = (uint32_t)(it >> 1) & 1u;
        if (!tc::mbar_wait_sleep(bar(B_DEMPTY + s), ph ^ 1u, WAIT_LIMIT)) {
          ok = false;
          break;
        }
        const uint32_t dtm = tmem + D_BASE + 128u * (uint32_t)s;
        // K step k (box nodes 8k .. 8k+7): 32 bytes into K atom k / 4; the
        // 8-row groups of B (columns of X) are 1 KB apart
        const uint64_t b0 = tc::smem_desc_sw(tc::smem_u32(bst), 1024, 2);
        // A and B in two halves of K: the first half is released (and
        // refilled with the next box) while the second half multiplies
#pragma unroll 1
        for (int hf = 0; hf < 2; hf++) {
          if (!tc::mbar_wait_sleep(bar(B_AFULL + hf), (uint32_t)it & 1u, WAIT_LIMIT)) {
            ok = false;
            break;
          }
          tc::fence_after();
#pragma unroll
          for (int k = 8 * hf; k < 8 * hf + 8; k++)
            mma_tf32_ts(dtm, tmem + A_HI + 8 * k,
                        b0 + (uint64_t)(((k >> 2) * KATOM + (k & 3) * 32) >> 4), IDESC_N,
                        k > 0 ? 1u : 0u);
          if (SPLIT) {
#pragma unroll
            for (int k = 8 * hf; k < 8 * hf + 8; k++)
              mma_tf32_ts(dtm, tmem + A_LO + 8 * k,
                          b0 + (uint64_t)(((k >> 2) * KATOM + (k & 3) * 32) >> 4), IDESC_64,
                          1u);
          }
          tc::commit(bar(B_AFREE + hf));
        }
        if (!ok) break;
        tc::commit(bar(B_DFULL + s));
      }
      if (!ok) atomicOr(a.err, 1);
      // drain: every MMA issued has completed before the TMEM is released
      tc::commit(bar(B_DRAIN));
      tc::mbar_wait_sleep(bar(B_DRAIN), 0u, WAIT_LIMIT);
    }
    __syncwarp();
  } else if (warp < W_ASM + 4) {
    // ------------------------------------------------ A assembly
    const int q = warp & 3;        // TMEM lanes 32q .. 32q + 31
    const int r = 32 * q + lane;   // box node of this thread
    const bool rv = r < ROWS;
    const int lx = r % BN, ly = (r / BN) % BN, lz = r / (BN * BN);
    // chunks of 16 columns this warp's rows reach: rows 32q .. 32q+31 couple
    // to columns 32q - 31 .. 32q + 62
    const int c_lo = q == 0 ? 0 : (q == 1 ? 0 : (q == 2 ? 2 : 4));
    const int c_hi = q == 0 ? 4 : (q == 1 ? 6 : 8);
    float *srow = staging + r * SPITCH - 16 * c_lo;  // srow[column]
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    // in-box couplings of this node: bit (dx+1) + 3 (dy+1) + 9 (dz+1)
    unsigned inb = 0u;
#pragma unroll
    for (int o = 0; o < 27; o++) {
      const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dz = o / 9 - 1;
      if (rv && lx + dx >= 0 && lx + dx < BN && ly + dy >= 0 && ly + dy < BN &&
          lz + dz >= 0 && lz + dz < BN)
        inb |= 1u << o;
    }
    // the A region of TMEM starts zero: columns outside a warp's window are
    // never written again
    {
      uint32_t z[16];
#pragma unroll
      for (int i = 0; i < 16; i++) z[i] = 0u;
#pragma unroll 1
      for (int c = 0; c < 256; c += 16) tmem_st16(lane_base + (uint32_t)c, z);
      tmem_wait_st();
    }
    // The box's element matrices arrive by two TMA boxes of Aaos viewed as
    // (64 floats, nex, ney, nez): (32 floats, 4 x 4 x 4 elements) each, rows
    // 0-3 and rows 4-7 of every element; box element le = ex + 4 ey + 16 ez
    // is the 128-byte row le of each tile, its 16-byte chunks permuted by
    // the 128-byte swizzle (le % 8), so the lanes of a warp reading the same
    // corner of different elements hit different banks.  Elements outside
    // the mesh arrive as zeros.  Warp W_ASM issues the next box's copies
    // once all four warps have read the stage.
    auto load_elements = [&](int b) {
      const int bx = b % a.nbx, by = (b / a.nbx) % a.nby, bz = b / (a.nbx * a.nby);
      tc::mbar_arrive_expect_tx(bar(B_EFULL), ESTAGE);
      tc::tma_load_4d(tc::smem_u32(est), &amap, 0, BE * bx, BE * by, BE * bz, bar(B_EFULL));
      tc::tma_load_4d(tc::smem_u32(est + ETILE), &amap, 32, BE * bx, BE * by, BE * bz,
                      bar(B_EFULL));
    };
    const bool eissuer = warp == W_ASM && lane == 0;
    if (eissuer) {
      tc::prefetch_tensormap(&amap);
      load_elements(blockIdx.x);
    }
    int issued = 1;  // element copies issued (box it lands in phase it)
    bool ok = true;
    int it = 0;
    for (int b = blockIdx.x; b < a.nbox; b += gridDim.x, it++) {
      const bool landed = tc::mbar_wait_sleep(bar(B_EFULL), (uint32_t)it & 1u, WAIT_LIMIT);
      if (!__all_sync(0xffffffffu, landed)) {
        ok = false;
        break;
      }
      // the 27 stencil sums: element (e0, e1, e2) around node r (local
      // (lx-1+e0, ly-1+e1, lz-1+e2)) holds the node at its corner (1-e0,
      // 1-e1, 1-e2), row s of its matrix; its input node j sits at offset
      // (e0 - 1 + x_j, e1 - 1 + y_j, e2 - 1 + z_j) from node r
      float sten[27];
#pragma unroll
      for (int o = 0; o < 27; o++) sten[o] = 0.f;
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const int e0 = e & 1, e1 = (e >> 1) & 1, e2 = e >> 2;
        const int ex = lx - 1 + e0, ey = ly - 1 + e1, ez = lz - 1 + e2;
        const bool in = rv && ex >= 0 && ex < BE && ey >= 0 && ey < BE && ez >= 0 && ez < BE;
        if (in) {
          const int le = ex + BE * (ey + BE * ez);
          const int sc = corner(1 - e0, 1 - e1, 1 - e2);  // row of the element matrix
          const unsigned char *row = est + (sc >> 2) * ETILE + le * 128;
          const int c0 = 2 * (sc & 3);  // its two 16-byte chunks
          const float4 va = *reinterpret_cast<const float4 *>(row + (((c0 ^ le) & 7) << 4));
          const float4 vb = *reinterpret_cast<const float4 *>(row + ((((c0 + 1) ^ le) & 7) << 4));
          const float v8[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const int o = (e0 + cx(j)) + 3 * (e1 + cy(j)) + 9 * (e2 + cz(j));
            sten[o] += v8[j];
          }
        }
      }
      // the stage is read: the next box's copies may overwrite it
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(bar(B_EEMPTY));
      if (warp == W_ASM && b + (int)gridDim.x < a.nbox) {
        const bool read = tc::mbar_wait_sleep(bar(B_EEMPTY), (uint32_t)it & 1u, WAIT_LIMIT);
        if (!__all_sync(0xffffffffu, read)) {
          ok = false;
          break;
        }
        if (eissuer) load_elements(b + gridDim.x);
        issued++;
      }
      // into this node's staging row (fixed positions: the rest stays zero)
#pragma unroll
      for (int o = 0; o < 27; o++)
        if ((inb >> o) & 1u)
          srow[r + (o % 3 - 1) + BN * ((o / 3) % 3 - 1) + BN * BN * (o / 9 - 1)] = sten[o];
      // head and tail into TMEM, K half by K half as the previous box's
      // MMAs release them
#pragma unroll 1
      for (int hf = 0; hf < 2; hf++) {
        const bool freed =
            tc::mbar_wait_sleep(bar(B_AFREE + hf), ((uint32_t)it & 1u) ^ 1u, WAIT_LIMIT);
        if (!__all_sync(0xffffffffu, freed)) {
          ok = false;
          break;
        }
        tc::fence_after();
        const int c0 = c_lo > 4 * hf ? c_lo : 4 * hf;
        const int c1 = c_hi < 4 * hf + 4 ? c_hi : 4 * hf + 4;
#pragma unroll 1
        for (int c = c0; c < c1; c++) {
          const float4 *src = reinterpret_cast<const float4 *>(srow + 16 * c);
          uint32_t hi[16], lo[16];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const float4 v = src[u];
            const float f[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
              hi[4 * u + k] = tf32_head(f[k]);
              lo[4 * u + k] = SPLIT ? tf32_tail(f[k], hi[4 * u + k]) : 0u;
            }
          }
          tmem_st16(lane_base + A_HI + 16u * (uint32_t)c, hi);
          if (SPLIT) tmem_st16(lane_base + A_LO + 16u * (uint32_t)c, lo);
        }
        tmem_wait_st();
        tc::fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(bar(B_AFULL + hf));
      }
      if (!ok) break;
    }
    // drain: an element copy issued for a box never reached has landed
    if (eissuer && issued > it)
      tc::mbar_wait_sleep(bar(B_EFULL), (uint32_t)(issued - 1) & 1u, WAIT_LIMIT);
    if (!ok && lane == 0) atomicOr(a.err, 1);
  } else if (warp < W_SPL + 8) {
    // ------------------------------------------------ X split
    // warp g: box nodes 32 (g / 2) .. + 31 (K atom g / 2, in half g / 4 of
    // K), columns 32 (g % 2) .. + 31 (one region of the TMA stage); this
    // thread's node row, 8 chunks of 4 columns, to K position r of B rows n
    // (head) and 64 + n (tail); Dirichlet rows zero when masked
    const int g = warp - W_SPL, q = g >> 1, hf = g >> 2, ch = g & 1;
    const int r = 32 * q + lane;
    const bool rv = r < ROWS;
    const int lx = r % BN, ly = (r / BN) % BN, lz = r / (BN * BN);
    // byte offset of this lane's word in a B row n, by n % 8 (the swizzle)
    uint32_t woff[8];
#pragma unroll
    for (int k = 0; k < 8; k++) woff[k] = (((uint32_t)(lane >> 2) ^ (uint32_t)k) << 4) + (lane & 3) * 4;
    unsigned char *bq = bst + q * KATOM + ch * 32 * 128;  // rows n from 32 ch
    bool ok = true;
    int it = 0;
    for (int b = blockIdx.x; b < a.nbox; b += gridDim.x, it++) {
      const int s = it & 1;
      bool zero = !rv;
      if (a.mask && rv) {
        const int bx = b % a.nbx, by = (b / a.nbx) % a.nby, bz = b / (a.nbx * a.nby);
        const int gx = BE * bx + lx, gy = BE * by + ly, gz = BE * bz + lz;
        zero = gx < a.nax && gy < a.nay && gz < a.naz &&
               __ldg(a.mask + (size_t)gx + (size_t)a.nax * ((size_t)gy + (size_t)a.nay * gz));
      }
      const bool landed =
          tc::mbar_wait_sleep(bar(B_XFULL + s), (uint32_t)(it >> 1) & 1u, WAIT_LIMIT);
      const bool bfree = tc::mbar_wait_sleep(bar(B_AFREE + hf), ((uint32_t)it & 1u) ^ 1u, WAIT_LIMIT);
      if (!__all_sync(0xffffffffu, landed && bfree)) {
        ok = false;
        break;
      }
      const unsigned char *xr = xst + s * XSTAGE + ch * XREG + r * 128;
      if (rv) {
#pragma unroll
        for (int c = 0; c < 8; c++) {
          float4 v = *reinterpret_cast<const float4 *>(xr + ((c ^ (r & 7)) << 4));
          if (zero) v = make_float4(0.f, 0.f, 0.f, 0.f);
          const float f[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int n = 4 * c + i;  // column 32 ch + n
            const uint32_t h = tf32_head(f[i]);
            *reinterpret_cast<uint32_t *>(bq + n * 128 + woff[n & 7]) = h;
            if (SPLIT)
              *reinterpret_cast<uint32_t *>(bq + (64 + n) * 128 + woff[n & 7]) =
                  tf32_tail(f[i], h);
          }
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(bar(B_XEMPTY + s));
        tc::mbar_arrive(bar(B_AFULL + hf));
      }
    }
    if (!ok && lane == 0) atomicOr(a.err, 1);
  } else {
    // ------------------------------------------------ epilogue
    // D (head + tail halves) of box node r into its row of the shared Y
    // tile, laid out as the TMA box (128-byte swizzle), then one thread
    // adds the tile to Y with two tensor reduces; Dirichlet rows under a
    // mask send zeros, rows outside the mesh are skipped by the TMA unit
    const int q = warp & 3;
    const int r = 32 * q + lane;
    const bool rv = r < ROWS;
    const int lx = r % BN, ly = (r / BN) % BN, lz = r / (BN * BN);
    const bool issuer = warp == W_EPI && lane == 0;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    if (issuer) tc::prefetch_tensormap(&ymap);
    bool ok = true;
    int it = 0;
    for (int b = blockIdx.x; b < a.nbox; b += gridDim.x, it++) {
      const int d = it & 1;
      const int bx = b % a.nbx, by = (b / a.nbx) % a.nby, bz = b / (a.nbx * a.nby);
      bool zero = false;
      if (a.mask && rv) {
        const int gx = BE * bx + lx, gy = BE * by + ly, gz = BE * bz + lz;
        zero = gx < a.nax && gy < a.nay && gz < a.naz &&
               __ldg(a.mask + (size_t)gx + (size_t)a.nax * ((size_t)gy + (size_t)a.nay * gz));
      }
      const bool got = tc::mbar_wait_sleep(bar(B_DFULL + d), (uint32_t)(it >> 1) & 1u, WAIT_LIMIT);
      // the previous box's reduces have read the tile; every epilogue
      // thread got this box's D, or all four warps stop here
      if (issuer) bulk_wait_read0();
      if (epi_sync_or(!got)) {
        ok = false;
        break;
      }
      tc::fence_after();
      // four passes of 16 columns: TMEM -> registers -> the tile
      unsigned char *yr = yst + r * 128;
#pragma unroll
      for (int c0 = 0; c0 < 64; c0 += 16) {
        uint32_t r1[16], r2[16];
        tc::tmem_ld16(lane_base + D_BASE + 128u * (uint32_t)d + (uint32_t)c0, r1);
        if (SPLIT) tc::tmem_ld16(lane_base + D_BASE + 128u * (uint32_t)d + 64u + (uint32_t)c0, r2);
        tc::tmem_wait_ld();
        if (rv) {
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const int c = c0 / 4 + u;  // 16-byte chunk of the row
            float v[4];
#pragma unroll
            for (int k = 0; k < 4; k++)
              v[k] = zero ? 0.f
                          : __uint_as_float(r1[4 * u + k]) +
                                (SPLIT ? __uint_as_float(r2[4 * u + k]) : 0.f);
            *reinterpret_cast<float4 *>(yr + (c >> 3) * XREG + (((c & 7) ^ (r & 7)) << 4)) =
                make_float4(v[0], v[1], v[2], v[3]);
          }
        }
      }
      tc::fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(bar(B_DEMPTY + d));
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      epi_sync();
      if (issuer) {
        const uint32_t src = tc::smem_u32(yst);
        tma_reduce_add_4d(&ymap, src, 0, BE * bx, BE * by, BE * bz);
        tma_reduce_add_4d(&ymap, src + XREG, 32, BE * bx, BE * by, BE * bz);
        bulk_commit();
      }
    }
    if (issuer) bulk_wait_read0();
    if (!ok && lane == 0) atomicOr(a.err, 1);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, TMEM_COLS);
  }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion,
                                   CUtensorMapFloatOOBfill);
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

// The map of a node-major [N][64] FP32 block vector on the structured node
// grid: dimensions (64, nax, nay, naz), box (32 columns, 5 x 5 x 5 nodes),
// 128-byte swizzle; loads read nodes outside the grid as zero, reduces skip
// them.
bool make_xmap(CUtensorMap *m, const float *X, int nax, int nay, int naz) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !X || (reinterpret_cast<uintptr_t>(X) & 15)) return false;
  const cuuint64_t dims[4] = {64, (cuuint64_t)nax, (cuuint64_t)nay, (cuuint64_t)naz};
  const cuuint64_t strides[3] = {256, 256 * (cuuint64_t)nax,
                                 256 * (cuuint64_t)nax * (cuuint64_t)nay};
  const cuuint32_t box[4] = {32, BN, BN, BN};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float *>(X), dims, strides, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

// The map of the element-major FP32 operator copy [E][64] on the structured
// element grid: dimensions (64, nex, ney, nez), box (32 floats = 4 rows of
// an element matrix, 4 x 4 x 4 elements), 128-byte swizzle, elements outside
// the grid read as zero.
bool make_amap(CUtensorMap *m, const float *A, int nex, int ney, int nez) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !A || (reinterpret_cast<uintptr_t>(A) & 15)) return false;
  const cuuint64_t dims[4] = {64, (cuuint64_t)nex, (cuuint64_t)ney, (cuuint64_t)nez};
  const cuuint64_t strides[3] = {256, 256 * (cuuint64_t)nex,
                                 256 * (cuuint64_t)nex * (cuuint64_t)ney};
  const cuuint32_t box[4] = {32, BE, BE, BE};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float *>(A), dims, strides, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

}  // namespace blocktc

bool block_tc_supported(const Handle &h) {
  return h.nax > 1 && h.nay > 1 && h.naz > 1 && !h.perm_d && h.block_err &&
         blocktc::encode_tiled() != nullptr;
}

int launch_block_tc(const Handle &h, bool split, const float *A, const float *X, float *Y,
                    const int *skip, const unsigned char *mask, cudaStream_t s) {
  using namespace blocktc;
  if (!block_tc_supported(h) || (reinterpret_cast<uintptr_t>(Y) & 15)) {
    set_error("tcgen05 block apply: needs the structured numbering and 16-byte aligned vectors");
    return VDR_BAD_ARGUMENT;
  }
  CUtensorMap xmap, ymap, amap;
  if (!make_xmap(&xmap, X, h.nax, h.nay, h.naz) || !make_xmap(&ymap, Y, h.nax, h.nay, h.naz) ||
      !make_amap(&amap, A, h.nax - 1, h.nay - 1, h.naz - 1)) {
    set_error("tcgen05 block apply: tensor maps of X, Y and the operator could not be made");
    return VDR_CUDA_ERROR;
  }
  static std::atomic<unsigned> opted{0u};
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned bit = 1u << (dev & 31);
  if (!(opted.load(std::memory_order_relaxed) & bit)) {
    cudaError_t e1 = cudaFuncSetAttribute(block_apply_tc_kernel<true>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    cudaError_t e2 = cudaFuncSetAttribute(block_apply_tc_kernel<false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e1 || e2) return cuda_fail(e1 ? e1 : e2, "tcgen05 block apply");
    opted.fetch_or(bit, std::memory_order_relaxed);
  }
  Args a;
  a.A = A;
  a.Y = Y;
  a.mask = mask;
  a.nax = h.nax;
  a.nay = h.nay;
  a.naz = h.naz;
  a.nbx = (h.nax - 2) / BE + 1;
  a.nby = (h.nay - 2) / BE + 1;
  const int nbz = (h.naz - 2) / BE + 1;
  a.nbox = a.nbx * a.nby * nbz;
  a.skip = skip;
  a.err = h.block_err;
  const int grid = a.nbox < device_sm_count() ? a.nbox : device_sm_count();
  if (split)
    block_apply_tc_kernel<true><<<grid, THREADS, SMEM, s>>>(xmap, ymap, amap, a);
  else
    block_apply_tc_kernel<false><<<grid, THREADS, SMEM, s>>>(xmap, ymap, amap, a);
  count_launches(1);
  const cudaError_t e = cudaGetLastError();
  return e ? cuda_fail(e, "tcgen05 block apply") : VDR_OK;
}

}  // namespace vdr
