// block.cu -- many right-hand sides with one operator (K <= 64 columns).
//
// Block vectors are node-major, X[n*K + k], so the K values a node carries
// are contiguous.  The tensor-core applies compute Y^T (K x 8) += X_e^T
// (K x 8) . A_e^T (8 x 8) per element with mma.sync m16n8k8 TF32 (one MMA
// per 16 columns, three for split TF32) on FP32 vectors, A_e read from an
// element-major FP32 copy (256 contiguous bytes per element), so the
// element matrices stream once for all K columns:
//
//   block_apply_tile  (default on the structured numbering) boxes of
//                     8 x 2 x 2 elements, node rows staged once in shared
//                     memory, results added there and sent once per node
//   block_apply_tf32  one warp per element: row gathers and float4 atomics
//   block_apply_tma   the same with bulk copies and bulk reductions
//   block_apply_df    the FP64-accurate apply for the refinement residual:
//                     lane = column, double-float contraction of the pair
//                     store (FP32 pipe), FP64 vectors.
//
// The inner solver is K independent Jacobi-BiCGStab iterations sharing every
// launch: per-column scalars (rho, alpha, omega, norms) in FP64, per-column
// deterministic reductions, and a per-column "active" flag that freezes a
// column once it meets its tolerance.  The outer loop refines each column
// in FP64 (residual and update), as the single-RHS mixed solver does.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "dfloat.cuh"
#include "vdr_internal.h"

namespace vdr {
namespace {

constexpr int BT = 512;  // threads per block of the block-vector kernels
constexpr unsigned FULL = 0xffffffffu;

// --------------------------------------------------------------- applies
__device__ __forceinline__ unsigned to_tf32(float f) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(f));
  return r;
}

// Element-major FP32 copy of the operator for the tensor-core applies,
// Aaos[p*64 + 8i + j] = A_e(i, j) * s(node j), with the rows and columns of
// Dirichlet nodes zero; s is the FP32 inverse diagonal (the Jacobi
// preconditioner of the block solve folded in) or 1.  From the hi parts of
// the double-float store, or from the FP64 store.
template <bool F64>
__global__ void aos_build(const float4 *__restrict__ Ahi,
                          const double2 *__restrict__ A64,
                          const int *__restrict__ conn, int E,
                          const float *__restrict__ colscale,
                          float4 *__restrict__ Aaos) {
  const long total = (long)E * 16;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long p = t >> 4;
    const int chunk = (int)(t & 15);  // = 2i + h: row i, columns 4h..4h+3
    float4 v;
    if (F64) {
      const double2 a = A64[(size_t)(2 * chunk) * E + p];
      const double2 b = A64[(size_t)(2 * chunk + 1) * E + p];
      v = make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y);
    } else {
      v = Ahi[(size_t)chunk * E + p];
    }
    float sc[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int cj = __ldg(conn + (size_t)(4 * (chunk & 1) + q) * E + p);
      sc[q] = cj < 0 ? 0.f : (colscale ? __ldg(colscale + (cj & NODE_BITS)) : 1.f);
    }
    if (__ldg(conn + (size_t)(chunk >> 1) * E + p) < 0) sc[0] = sc[1] = sc[2] = sc[3] = 0.f;
    Aaos[t] = make_float4(v.x * sc[0], v.y * sc[1], v.z * sc[2], v.w * sc[3]);
  }
}

// K = 16 * tiles columns.  Warp per element.  The MMA's M dimension is the
// column k (16 per tile), N the element's output node i, K its input node
// j: D[k][i] = sum_j X[node j][k] * A[i][j].  Per tile, lane (c = lane/4,
// q = lane%4) loads the 16 bytes X[node c][16m + 4q .. +3] (times the
// optional per-node scale: the Jacobi preconditioner folded into the
// gather), the warp re-reads them from shared memory in the m16n8k8 TF32
// A-fragment layout (g = lane/4, t = lane%4), and the D fragment goes back
// through shared memory so that lane (c, q) adds 4 contiguous columns of
// node c with one float4 atomic.  Dirichlet nodes (negative conn) read as
// zero and receive nothing.  SPLIT: each operand is split into a TF32 head
// and tail and three MMAs (hi.hi + hi.lo + lo.hi) give FP32-level
// products; the apply is bound by memory traffic, so the extra MMAs cost
// little.
constexpr int XS = 24;  // row stride (floats) of the X stage: no conflicts
constexpr int DS = 20;  // row stride of the D stage
// The next element's connectivity and operator fragment are loaded while
// the current one is processed, and all TILES column tiles of X are
// gathered at once, so each warp keeps several loads in flight.
template <bool SPLIT, int TILES>
__global__ void __launch_bounds__(256) block_apply_tf32(
    const float *__restrict__ Aaos, const int *__restrict__ conn, int E,
    const float *__restrict__ X, const float *__restrict__ dscale,
    float *__restrict__ Y, const int *skip) {
  constexpr int K = 16 * TILES;
  if (skip && *(volatile const int *)skip) return;
  __shared__ __align__(16) float xs_all[8][8 * XS];
  __shared__ __align__(16) float ds_all[8][8 * DS];
  float *xs = xs_all[threadIdx.x >> 5];
  float *ds = ds_all[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;  // fragment coordinates
  const int c = lane >> 2, q = lane & 3;  // staging coordinates
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  long p = warp;
  int cl = 0;
  float f0 = 0.f, f1 = 0.f;
  if (p < E) {
    if (lane < 8) cl = __ldg(conn + (size_t)lane * E + p);
    f0 = __ldg(Aaos + (size_t)p * 64 + 8 * g + t);
    f1 = __ldg(Aaos + (size_t)p * 64 + 8 * g + t + 4);
  }
  for (; p < E; p += nwarps) {
    const long pn = p + nwarps;
    int cln = 0;
    float f0n = 0.f, f1n = 0.f;
    if (pn < E) {
      if (lane < 8) cln = __ldg(conn + (size_t)lane * E + pn);
      f0n = __ldg(Aaos + (size_t)pn * 64 + 8 * g + t);
      f1n = __ldg(Aaos + (size_t)pn * 64 + 8 * g + t + 4);
    }
    const int nc = __shfl_sync(FULL, cl, c);
    float4 xv[TILES];
#pragma unroll
    for (int m = 0; m < TILES; m++)
      xv[m] = nc >= 0
          ? __ldg(reinterpret_cast<const float4 *>(X + (size_t)nc * K + 16 * m) + q)
          : make_float4(0.f, 0.f, 0.f, 0.f);
    const float sc = (nc >= 0 && dscale) ? __ldg(dscale + nc) : 1.f;
    const unsigned b0 = to_tf32(f0), b1 = to_tf32(f1);
    unsigned c0 = 0u, c1 = 0u;
    if (SPLIT) {
      c0 = to_tf32(f0 - __uint_as_float(b0));
      c1 = to_tf32(f1 - __uint_as_float(b1));
    }
#pragma unroll
    for (int m = 0; m < TILES; m++) {
      float4 x4 = xv[m];
      x4.x *= sc; x4.y *= sc; x4.z *= sc; x4.w *= sc;
      *reinterpret_cast<float4 *>(xs + c * XS + 4 * q) = x4;
      __syncwarp();
      float xa[4];
      xa[0] = xs[t * XS + g];
      xa[1] = xs[t * XS + g + 8];
      xa[2] = xs[(t + 4) * XS + g];
      xa[3] = xs[(t + 4) * XS + g + 8];
      unsigned ah[4], al[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        ah[u] = to_tf32(xa[u]);
        al[u] = SPLIT ? to_tf32(xa[u] - __uint_as_float(ah[u])) : 0u;
      }
      float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
      if (SPLIT) {
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
            : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
            : "r"(al[0]), "r"(al[1]), "r"(al[2]), "r"(al[3]), "r"(b0), "r"(b1));
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
            : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
            : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(c0), "r"(c1));
      }
      asm volatile(
          "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
          "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
          : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
          : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(b0), "r"(b1));
      // D[k][i]: d0 (g, 2t), d1 (g, 2t+1), d2 (g+8, 2t), d3 (g+8, 2t+1)
      ds[(2 * t) * DS + g] = d0;
      ds[(2 * t + 1) * DS + g] = d1;
      ds[(2 * t) * DS + g + 8] = d2;
      ds[(2 * t + 1) * DS + g + 8] = d3;
      __syncwarp();
      if (nc >= 0)
        atomicAdd(reinterpret_cast<float4 *>(Y + (size_t)nc * K + 16 * m) + q,
                  *reinterpret_cast<const float4 *>(ds + c * DS + 4 * q));
      __syncwarp();
    }
    cl = cln;
    f0 = f0n;
    f1 = f1n;
  }
}

// ------------------------------------------- node-tile variant (default)
// On the canonical structured numbering (element (i, j, k), i fastest, has
// nodes i + a j + a b k + {0, 1, 1 + a, a} and the same plus a b, on an
// a x b x c node grid) a block takes a box of TILE_X x TY x TILE_Z
// elements.  The (TILE_X + 1)(TY + 1)(TILE_Z + 1) node rows the box touches
// (K contiguous floats per node) arrive once in shared memory by 16-byte
// asynchronous copies, coalesced along x and zero-filled outside the mesh;
// the elements' mma.sync contractions read their operands there and add
// their results into a second shared tile (its rows enter the MMAs as the
// accumulator), which then goes to Y with one float4 atomic per 4 columns
// of each node.  Per element this reads and
// adds about 2.5 node rows instead of 8 and 8.  The operator copy carries
// the Dirichlet mask (zero rows and columns) and, in the block solve, the
// Jacobi scale (see aos_build); the kernel reads one mask byte per node row
// so that Dirichlet rows of X read as zero and of Y receive nothing.  The
// elements of a box are taken in the 8 parity classes of (i, j, k) (no two
// elements of one class share a node), one element per warp per class with
// a block barrier between classes, so the shared result tile needs no
// atomics.  Shared rows are K + 8 floats apart (K + 24 for K = 16; 8 banks
// mod 32) and x lines TILE_WP = 10 rows apart, which leaves every fragment
// read and result update of a warp free of bank conflicts for TY + 1 odd.
constexpr int TILE_X = 8, TILE_Y = 2, TILE_Z = 2, TILE_WP = 10;

template <int K>
__host__ __device__ constexpr int tile_row_stride() {
  return K % 32 == 0 ? K + 8 : K + 24;
}

template <int TY, int KC>
constexpr int tile_smem_bytes() {
  return 2 * TILE_WP * (TY + 1) * (TILE_Z + 1) * tile_row_stride<KC>() * 4;
}

// Shared row offset of local node s (w_el order) of an element.
template <int TY>
__device__ __forceinline__ int tile_node_off(int s) {
  const int s2 = s & 3;
  const int dx = (s2 == 1 || s2 == 2) ? 1 : 0, dy = s2 >> 1, dz = s >> 2;
  return dx + TILE_WP * (dy + (TY + 1) * dz);
}

// 16-byte global -> shared copy; bytes beyond src_bytes are zero-filled.
__device__ __forceinline__ void cp_async16(void *dst, const void *src,
                                           unsigned src_bytes) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;"
               :: "r"(d), "l"(src), "r"(src_bytes) : "memory");
}

template <bool SPLIT, int TILES, int TY, int HALVES>
__global__ void __launch_bounds__(64 * TY, 8 / TY) block_apply_tile(
    const float *__restrict__ Aaos, int nax, int nay, int naz,
    const unsigned char *__restrict__ mask, const float *__restrict__ X,
    float *__restrict__ Y, const int *skip) {
  // KC columns per block (of the KR = HALVES * KC of a block-vector row)
  constexpr int KC = 16 * TILES, KR = KC * HALVES;
  constexpr int S = tile_row_stride<KC>(), C4 = KC / 4;
  constexpr int LX = TILE_X + 1, HP = TY + 1, LZ = TILE_Z + 1;
  constexpr int ROWS = TILE_WP * HP * LZ;
  constexpr int NT = 64 * TY;            // threads: one warp per element of a class
  constexpr int NV = LX * HP * LZ * C4;  // float4 slots of the node box
  constexpr int PER = (NV + NT - 1) / NT;
  static_assert(NT % C4 == 0, "a thread keeps its column chunk");
  static_assert(PER <= 32, "one bit per slot");
  constexpr int RSTEP = NT / C4;         // box rows between a thread's slots
  if (skip && *(volatile const int *)skip) return;
  extern __shared__ __align__(16) float tile_sm[];
  float *xs = tile_sm, *ys = tile_sm + ROWS * S;
  const int nex = nax - 1, ney = nay - 1, nez = naz - 1;
  const int ntx = (nex + TILE_X - 1) / TILE_X, nty = (ney + TY - 1) / TY;
  const int bid = blockIdx.x / HALVES;
  const int col0 = (blockIdx.x % HALVES) * KC;
  X += col0;
  Y += col0;
  const int gx0 = (bid % ntx) * TILE_X, gy0 = ((bid / ntx) % nty) * TY,
            gz0 = (bid / (ntx * nty)) * TILE_Z;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int c = threadIdx.x % C4, r0 = threadIdx.x / C4;

  // Node rows of the box into shared memory; the result tile zeroed; the
  // slots' mask bytes loaded (all in flight before any is used).
  unsigned inmesh = 0u;  // bit u: slot u's node is in the mesh
  unsigned char mk[PER];
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int r = r0 + u * RSTEP;
    mk[u] = 0;
    if (r < LX * HP * LZ) {
      const int li = r % LX, lj = (r / LX) % HP, lk = r / (LX * HP);
      const int gx = gx0 + li, gy = gy0 + lj, gz = gz0 + lk;
      const bool in = gx < nax && gy < nay && gz < naz;
      const size_t n = in ? gx + (size_t)nax * (gy + (size_t)nay * gz) : 0;
      const int row = li + TILE_WP * (lj + HP * lk);
      cp_async16(xs + row * S + 4 * c, X + n * KR + 4 * c, in ? 16u : 0u);
      *reinterpret_cast<float4 *>(ys + row * S + 4 * c) =
          make_float4(0.f, 0.f, 0.f, 0.f);
      if (in) {
        inmesh |= 1u << u;
        if (mask) mk[u] = __ldg(mask + n);
      }
    }
  }
  asm volatile("cp.async.commit_group;" ::: "memory");

  // This warp's element of each parity class and its operator fragment
  // (B[j][i] = A_e[i][j]: lane (g, t) holds A_e[g][t] and A_e[g][t + 4]).
  float fa[8][2];
#pragma unroll
  for (int ph = 0; ph < 8; ph++) {
    const int gi = gx0 + (ph & 1) + 2 * (w & 3);
    const int gj = gy0 + ((ph >> 1) & 1) + 2 * (w >> 2);
    const int gk = gz0 + (ph >> 2);
    fa[ph][0] = fa[ph][1] = 0.f;
    if (gi < nex && gj < ney && gk < nez) {
      const float *a =
          Aaos + ((size_t)gi + (size_t)nex * (gj + (size_t)ney * gk)) * 64 + 8 * g + t;
      fa[ph][0] = __ldg(a);
      fa[ph][1] = __ldg(a + 4);
    }
  }
  unsigned live = inmesh;  // bit u: in the mesh and not Dirichlet
#pragma unroll
  for (int u = 0; u < PER; u++)
    if (mk[u]) live &= ~(1u << u);
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  // Dirichlet rows read as zero whatever X holds there (each thread clears
  // the chunks it copied itself, so the barrier below publishes them); the
  // block solve passes no mask: its X is zero on those rows already.
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int r = r0 + u * RSTEP;
    if (mask && r < LX * HP * LZ && !((live >> u) & 1u)) {
      const int li = r % LX, lj = (r / LX) % HP, lk = r / (LX * HP);
      *reinterpret_cast<float4 *>(xs + (li + TILE_WP * (lj + HP * lk)) * S + 4 * c) =
          make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  __syncthreads();

  // The contractions, one parity class at a time.
#pragma unroll
  for (int ph = 0; ph < 8; ph++) {
    const int ei = (ph & 1) + 2 * (w & 3), ej = ((ph >> 1) & 1) + 2 * (w >> 2),
              ek = ph >> 2;
    if (gx0 + ei < nex && gy0 + ej < ney && gz0 + ek < nez) {
      const int rb = ei + TILE_WP * (ej + HP * ek);
      const float *xl = xs + (rb + tile_node_off<TY>(t)) * S + g;
      const float *xh = xs + (rb + tile_node_off<TY>(t + 4)) * S + g;
      float *y0 = ys + (rb + tile_node_off<TY>(2 * t)) * S + g;
      float *y1 = ys + (rb + tile_node_off<TY>(2 * t + 1)) * S + g;
      const unsigned b0 = to_tf32(fa[ph][0]), b1 = to_tf32(fa[ph][1]);
      unsigned c0 = 0u, c1 = 0u;
      if (SPLIT) {
        c0 = to_tf32(fa[ph][0] - __uint_as_float(b0));
        c1 = to_tf32(fa[ph][1] - __uint_as_float(b1));
      }
#pragma unroll
      for (int m = 0; m < TILES; m++) {
        const float xa[4] = {xl[16 * m], xl[16 * m + 8], xh[16 * m], xh[16 * m + 8]};
        unsigned ah[4], al[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          ah[u] = to_tf32(xa[u]);
          al[u] = SPLIT ? to_tf32(xa[u] - __uint_as_float(ah[u])) : 0u;
        }
        // the result rows enter as the accumulator: D = X_e^T A_e^T + Y
        float d0 = y0[16 * m], d1 = y1[16 * m], d2 = y0[16 * m + 8],
              d3 = y1[16 * m + 8];
        if (SPLIT) {
          asm volatile(
              "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
              "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
              : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
              : "r"(al[0]), "r"(al[1]), "r"(al[2]), "r"(al[3]), "r"(b0), "r"(b1));
          asm volatile(
              "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
              "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
              : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
              : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(c0), "r"(c1));
        }
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
            : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
            : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(b0), "r"(b1));
        // D[k][i]: d0 (g, 2t), d1 (g, 2t+1), d2 (g+8, 2t), d3 (g+8, 2t+1)
        y0[16 * m] = d0;
        y1[16 * m] = d1;
        y0[16 * m + 8] = d2;
        y1[16 * m + 8] = d3;
      }
    }
    __syncthreads();
  }

  // The result tile into Y (Dirichlet nodes receive nothing).
#pragma unroll
  for (int u = 0; u < PER; u++) {
    const int r = r0 + u * RSTEP;
    if (r < LX * HP * LZ && ((live >> u) & 1u)) {
      const int li = r % LX, lj = (r / LX) % HP, lk = r / (LX * HP);
      const int gx = gx0 + li, gy = gy0 + lj, gz = gz0 + lk;
      const int row = li + TILE_WP * (lj + HP * lk);
      const size_t n = gx + (size_t)nax * (gy + (size_t)nay * gz);
      atomicAdd(reinterpret_cast<float4 *>(Y + n * KR) + c,
                *reinterpret_cast<const float4 *>(ys + row * S + 4 * c));
    }
  }
}

// ---------------------------------------------- bulk-copy (TMA) variant
// The same contraction with the data movement taken off the LSU pipe: the
// eight X rows of an element (K floats each, contiguous in the node-major
// block vector) arrive in shared memory by cp.async.bulk (one per node,
// completion on an mbarrier), three elements ahead per warp, and the 8 x K
// result rows leave by cp.reduce.async.bulk .add.f32 straight from shared
// memory.  Every mbarrier wait is bounded by a clock budget; a wait that
// runs out sets *err, drains this warp's copies (again bounded) and
// returns, so the host can report VDR_TIMEOUT.
constexpr int TMA_WARPS = 4, TMA_S = 3;
constexpr long long TMA_WAIT_CYCLES = 4000000000LL;  // about 2 s

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned a) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned a, unsigned bytes) {
  unsigned long long st;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
               : "=l"(st)
               : "r"(a), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned a, unsigned parity) {
  unsigned d;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
      "selp.u32 %0, 1, 0, p; }"
      : "=r"(d)
      : "r"(a), "r"(parity)
      : "memory");
  return d != 0u;
}
// Warp-uniform bounded wait; false when the budget (clock cycles) ran out.
__device__ __forceinline__ bool mbar_wait(unsigned a, unsigned parity,
                                          long long budget = TMA_WAIT_CYCLES) {
  const long long t0 = clock64();
  while (!__all_sync(FULL, mbar_try(a, parity))) {
    if (__any_sync(FULL, clock64() - t0 > budget)) return false;
  }
  return true;
}

// The bounded wait's failure path on its own: one warp waits, with a short
// budget, on an mbarrier that nothing arrives at (no copy is issued, so
// nothing is in flight), sets *err when the budget runs out and returns.
__global__ void __launch_bounds__(32) wait_timeout_kernel(int *err, long long budget) {
  __shared__ __align__(8) unsigned long long bar;
  const unsigned a = smem_u32(&bar);
  if (threadIdx.x == 0) mbar_init(a);
  __syncthreads();
  if (!mbar_wait(a, 0u, budget) && threadIdx.x == 0) atomicOr(err, 1);
}
__device__ __forceinline__ void bulk_load(unsigned dst, const void *src, unsigned bytes,
                                          unsigned bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void bulk_reduce_add(float *dst, unsigned src, unsigned bytes) {
  asm volatile(
      "cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f32 [%0], [%1], %2;" ::"l"(dst),
      "r"(src), "r"(bytes)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read1() {
  asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <int K>
__device__ __forceinline__ void tma_issue(unsigned xs_a, unsigned bar, int b, int lane,
                                          int cl, const float *X) {
  constexpr int XR = K + 8, XBUF = 8 * XR;
  if (lane == 0) mbar_expect(bar, 8u * K * 4u);
  __syncwarp();
  if (lane < 8)
    bulk_load(xs_a + (unsigned)(b * XBUF + lane * XR) * 4u,
              X + (size_t)(cl & NODE_BITS) * K, K * 4u, bar);
}

template <bool SPLIT, int TILES>
__global__ void __launch_bounds__(TMA_WARPS * 32) block_apply_tma(
    const float *__restrict__ Aaos, const int *__restrict__ conn, int E,
    const float *__restrict__ X, const float *__restrict__ dscale,
    float *__restrict__ Y, const int *skip, int *err) {
  constexpr int K = 16 * TILES, XR = K + 8, DR = K + 4;
  constexpr int XBUF = 8 * XR, DBUF = 8 * DR;
  if (skip && *(volatile const int *)skip) return;
  extern __shared__ __align__(128) float tma_smem[];
  __shared__ __align__(8) unsigned long long bars[TMA_WARPS][TMA_S];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  float *xs = tma_smem + w * (TMA_S * XBUF + 2 * DBUF);
  float *ds = xs + TMA_S * XBUF;
  const unsigned xs_a = smem_u32(xs), ds_a = smem_u32(ds);
  unsigned bar_a[TMA_S];
#pragma unroll
  for (int s = 0; s < TMA_S; s++) bar_a[s] = smem_u32(&bars[w][s]);
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < TMA_S; s++) mbar_init(bar_a[s]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  const long gw = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nw = ((long)gridDim.x * blockDim.x) >> 5;
  int cn[TMA_S];
  long issued = 0;  // elements whose rows were requested
#pragma unroll
  for (int s = 0; s < TMA_S; s++) {
    const long pe = gw + s * nw;
    cn[s] = (pe < E && lane < 8) ? __ldg(conn + (size_t)lane * E + pe) : 0;
    if (pe < E) {
      tma_issue<K>(xs_a, bar_a[s], s, lane, cn[s], X);
      issued++;
    }
  }
  float f0 = 0.f, f1 = 0.f;
  if (gw < E) {
    f0 = __ldg(Aaos + (size_t)gw * 64 + 8 * g + t);
    f1 = __ldg(Aaos + (size_t)gw * 64 + 8 * g + t + 4);
  }
  long it = 0;
  bool failed = false;
  for (long p = gw; p < E; p += nw, it++) {
    const int b = (int)(it % TMA_S);
    if (!mbar_wait(bar_a[b], (unsigned)((it / TMA_S) & 1))) {
      failed = true;
      break;
    }
    const long pn = p + nw;
    float f0n = 0.f, f1n = 0.f;
    if (pn < E) {
      f0n = __ldg(Aaos + (size_t)pn * 64 + 8 * g + t);
      f1n = __ldg(Aaos + (size_t)pn * 64 + 8 * g + t + 4);
    }
    const int cl = cn[0];
    const int na = __shfl_sync(FULL, cl, t), nb = __shfl_sync(FULL, cl, t + 4);
    const float sa = (na >= 0 && dscale) ? __ldg(dscale + na) : 1.f;
    const float sb = (nb >= 0 && dscale) ? __ldg(dscale + nb) : 1.f;
    const unsigned b0 = to_tf32(f0), b1 = to_tf32(f1);
    unsigned c0 = 0u, c1 = 0u;
    if (SPLIT) {
      c0 = to_tf32(f0 - __uint_as_float(b0));
      c1 = to_tf32(f1 - __uint_as_float(b1));
    }
    const int db = (int)(it & 1);
    if (lane < 8) bulk_wait_read1();  // the reduce that last read this D buffer
    __syncwarp();
    const float *xb = xs + b * XBUF;
    float *dbp = ds + db * DBUF;
#pragma unroll
    for (int m = 0; m < TILES; m++) {
      float xa[4];
      xa[0] = na < 0 ? 0.f : xb[t * XR + 16 * m + g] * sa;
      xa[1] = na < 0 ? 0.f : xb[t * XR + 16 * m + g + 8] * sa;
      xa[2] = nb < 0 ? 0.f : xb[(t + 4) * XR + 16 * m + g] * sb;
      xa[3] = nb < 0 ? 0.f : xb[(t + 4) * XR + 16 * m + g + 8] * sb;
      unsigned ah[4], al[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        ah[u] = to_tf32(xa[u]);
        al[u] = SPLIT ? to_tf32(xa[u] - __uint_as_float(ah[u])) : 0u;
      }
      float d0 = 0.f, d1 = 0.f, d2 = 0.f, d3 = 0.f;
      if (SPLIT) {
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
            : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
            : "r"(al[0]), "r"(al[1]), "r"(al[2]), "r"(al[3]), "r"(b0), "r"(b1));
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
            : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
            : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(c0), "r"(c1));
      }
      asm volatile(
          "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
          "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
          : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
          : "r"(ah[0]), "r"(ah[1]), "r"(ah[2]), "r"(ah[3]), "r"(b0), "r"(b1));
      // D[k][i] -> row i of the output stage: d0 (k=g, i=2t), d1 (g, 2t+1),
      // d2 (g+8, 2t), d3 (g+8, 2t+1)
      dbp[(2 * t) * DR + 16 * m + g] = d0;
      dbp[(2 * t + 1) * DR + 16 * m + g] = d1;
      dbp[(2 * t) * DR + 16 * m + g + 8] = d2;
      dbp[(2 * t + 1) * DR + 16 * m + g + 8] = d3;
    }
    fence_proxy_async();
    __syncwarp();
    if (lane < 8) {
      if (cl >= 0)
        bulk_reduce_add(Y + (size_t)cl * K, ds_a + (unsigned)(db * DBUF + lane * DR) * 4u,
                        K * 4u);
      bulk_commit();
    }
    // refill this stage with the element TMA_S ahead (every lane has read it)
    const long p2 = p + TMA_S * nw;
#pragma unroll
    for (int s = 0; s + 1 < TMA_S; s++) cn[s] = cn[s + 1];
    cn[TMA_S - 1] = (p2 < E && lane < 8) ? __ldg(conn + (size_t)lane * E + p2) : 0;
    if (p2 < E) {
      fence_proxy_async();
      tma_issue<K>(xs_a, bar_a[b], b, lane, cn[TMA_S - 1], X);
      issued++;
    }
    f0 = f0n;
    f1 = f1n;
  }
  if (lane < 8) bulk_wait_all();
  if (failed) {
    if (lane == 0) atomicOr(err, 1);
    // drain the loads this warp still has in flight (bounded)
    for (long j = it; j < issued; j++)
      if (!mbar_wait(bar_a[(int)(j % TMA_S)], (unsigned)((j / TMA_S) & 1))) break;
  }
}

// FP64-accurate block apply over the pair store: warp per element, lane =
// columns lane, lane+32.  The element's 64 pairs are staged in shared memory.
__global__ void __launch_bounds__(256) block_apply_df(
    const float4 *__restrict__ Ahi, const float4 *__restrict__ Alo,
    const int *__restrict__ conn, int E, int K, const double *__restrict__ X,
    double *__restrict__ Y) {
  __shared__ float2 sa[8][64];  // per warp: (hi, lo) of entry 8i + j
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long p = warp; p < E; p += nwarps) {
    __syncwarp();
    if (lane < 16) {
      const float4 h = Ahi[(size_t)lane * E + p];
      const float4 l = Alo[(size_t)lane * E + p];
      sa[w][4 * lane + 0] = make_float2(h.x, l.x);
      sa[w][4 * lane + 1] = make_float2(h.y, l.y);
      sa[w][4 * lane + 2] = make_float2(h.z, l.z);
      sa[w][4 * lane + 3] = make_float2(h.w, l.w);
    }
    const int cl = lane < 8 ? __ldg(conn + (size_t)lane * E + p) : 0;
    int c[8];
#pragma unroll
    for (int s = 0; s < 8; s++) c[s] = __shfl_sync(FULL, cl, s);
    __syncwarp();
    for (int k = lane; k < K; k += 32) {
      double xv[8];
      int emax = 0;
#pragma unroll
      for (int s = 0; s < 8; s++) {
        xv[s] = c[s] < 0 ? 0.0 : X[(size_t)c[s] * K + k];
        emax = max(emax, df_exp(xv[s]));
      }
      const int shift = emax - 1023;
      float xh[8], xl[8];
      bool bad = false;
#pragma unroll
      for (int s = 0; s < 8; s++) df_split(xv[s], xh[s], xl[s], bad, shift);
      double out[8];
      if (bad) {  // inf/NaN input: plain FP64 from the merged pairs
#pragma unroll
        for (int i = 0; i < 8; i++) {
          double acc = 0.0;
#pragma unroll
          for (int j = 0; j < 8; j++)
            acc += df_to_double(sa[w][8 * i + j].x, sa[w][8 * i + j].y) * xv[j];
          out[i] = acc;
        }
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++) {
          DfAcc acc{0.f, 0.f};
#pragma unroll
          for (int j = 0; j < 8; j++)
            df_fma_acc(acc, sa[w][8 * i + j].x, sa[w][8 * i + j].y, xh[j], xl[j]);
          out[i] = df_to_double(acc.s, acc.c);
          if (!df_scale(out[i], shift)) out[i] = ldexp(out[i], shift);
        }
      }
#pragma unroll
      for (int s = 0; s < 8; s++)
        if (c[s] >= 0) atomicAdd(Y + (size_t)c[s] * K + k, out[s]);
    }
  }
}

// FP64 block apply from the FP64 store (used when the handle holds FP64).
__global__ void __launch_bounds__(256) block_apply_f64(
    const double2 *__restrict__ A64, const int *__restrict__ conn, int E, int K,
    const double *__restrict__ X, double *__restrict__ Y) {
  __shared__ double sa[8][64];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long p = warp; p < E; p += nwarps) {
    __syncwarp();
    {
      const double2 v = A64[(size_t)lane * E + p];
      sa[w][2 * lane] = v.x;
      sa[w][2 * lane + 1] = v.y;
    }
    const int cl = lane < 8 ? __ldg(conn + (size_t)lane * E + p) : 0;
    int c[8];
#pragma unroll
    for (int s = 0; s < 8; s++) c[s] = __shfl_sync(FULL, cl, s);
    __syncwarp();
    for (int k = lane; k < K; k += 32) {
      double xv[8];
#pragma unroll
      for (int s = 0; s < 8; s++) xv[s] = c[s] < 0 ? 0.0 : X[(size_t)c[s] * K + k];
#pragma unroll
      for (int i = 0; i < 8; i++) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < 8; j++) acc += sa[w][8 * i + j] * xv[j];
        if (c[i] >= 0) atomicAdd(Y + (size_t)c[i] * K + k, acc);
      }
    }
  }
}

// ---------------------------------------------------- block right-hand side
// B[n*K + k] += cf * Q[k*E + e] * phi[i*E + e] for the element's nodes.
__global__ void block_rhs(const double *__restrict__ phi,
                          const int *__restrict__ conn, int E, int K,
                          const double *__restrict__ Q,
                          const int *__restrict__ perm, double cf,
                          double *__restrict__ B) {
  const long total = (long)E * K;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    const long e = t / K;
    const int k = (int)(t % K);
    const long ecaller = perm ? perm[e] : e;  // Q is in the caller's order
    const double qe = Q[(size_t)k * E + ecaller];
    if (qe == 0.0) continue;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int c = conn[(size_t)i * E + e];
      if (c >= 0) atomicAdd(B + (size_t)c * K + k, cf * qe * phi[(size_t)i * E + e]);
    }
  }
}

// ------------------------------------------------------ block Krylov state
struct BState {
  unsigned ticket;
  int done, iter, itmax;
  double tol;
};
// per-column arrays, each of length K (kept in one device buffer)
struct BCols {
  double *bnrm2, *err, *rho, *rho_old, *alpha, *omega, *snrm;
  double *tol;  // the column's inner tolerance
  int *active, *sconv, *status;
};

struct BVec {
  long n;  // N*K
  int K;
  BState *st;
  BCols c;
  double *partials;  // [q][k][block]
  const float *b, *dinv;  // dinv per node
  const unsigned char *m; // per node
  float *x, *r, *rh, *p, *v, *s, *t;
  int kshift;               // K = 1 << kshift
  const double *outer_err;  // per column FP64 residual of the refinement
  double outer_tol;         // columns already at outer_tol stay inactive
};

// Per-column grid reduction: thread tid owns column tid % K (blockDim is a
// multiple of K and the grid stride keeps the column).  Each block writes
// its per-column sums of NQ quantities to partials[q][k][block]; the last
// block to finish (ticket) combines them: BT/K threads per column each
// take a strided slice of the blocks (four loads in flight), then one
// thread per column adds the slices in fixed order -- deterministic for a
// given grid.  Returns true in threads tid < K of the last block, with
// out[q*K + k] the column totals.  MAX: maxima of non-negative values.
template <int NQ, bool MAX = false>
__device__ __forceinline__ bool col_grid_sum(double (&v)[NQ], const BVec &a,
                                             double *out /* [NQ][K] */) {
  __shared__ double sm[NQ][BT];
  __shared__ bool last;
  const int K = a.K;
  const int tid = threadIdx.x;
#pragma unroll
  for (int q = 0; q < NQ; q++) sm[q][tid] = v[q];
  __syncthreads();
  if (tid < K) {
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      double s = 0.0;
      for (int r = tid; r < BT; r += K) s = MAX ? fmax(s, sm[q][r]) : s + sm[q][r];
      a.partials[((size_t)q * K + tid) * gridDim.x + blockIdx.x] = s;
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = atomicAdd(&a.st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  const int T = BT >> a.kshift;  // threads per column
  const int k = tid & (K - 1), sub = tid >> a.kshift;
  const int G = (int)gridDim.x;
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const double *pp = a.partials + ((size_t)q * K + k) * G;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int b = sub;
    for (; b + 3 * T < G; b += 4 * T) {
      const double v0 = __ldcg(pp + b), v1 = __ldcg(pp + b + T);
      const double v2 = __ldcg(pp + b + 2 * T), v3 = __ldcg(pp + b + 3 * T);
      s0 = MAX ? fmax(s0, v0) : s0 + v0;
      s1 = MAX ? fmax(s1, v1) : s1 + v1;
      s2 = MAX ? fmax(s2, v2) : s2 + v2;
      s3 = MAX ? fmax(s3, v3) : s3 + v3;
    }
    for (; b < G; b += T) {
      const double v0 = __ldcg(pp + b);
      s0 = MAX ? fmax(s0, v0) : s0 + v0;
    }
    sm[q][tid] = MAX ? fmax(fmax(s0, s1), fmax(s2, s3)) : (s0 + s1) + (s2 + s3);
  }
  __syncthreads();
  if (tid < K) {
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      double s = 0.0;
      for (int u = 0; u < T; u++)
        s = MAX ? fmax(s, sm[q][u * K + tid]) : s + sm[q][u * K + tid];
      out[q * K + tid] = s;
    }
  }
  __syncthreads();
  if (tid == 0) a.st->ticket = 0u;
  return tid < K;
}

// Per-thread inner-product accumulation in double-float: exact FP32
// products (two-product) summed with TwoSum, i.e. FP64-accurate inner
// products without the FP64 pipe.
__device__ __forceinline__ void dot_acc(DfAcc &acc, float a, float b) {
  df_fma_acc(acc, a, 0.0f, b, 0.0f);
}
__device__ __forceinline__ double dot_val(const DfAcc &acc) {
  return df_to_double(acc.s, acc.c);
}

// Grid-stride loops.  BLOOP: over the N*K block entries, one per thread per
// trip (the FP64 glue kernels below).  ULOOP: over units of four
// consecutive columns 4g .. 4g+3 of one node row (unit j = node * K/4 + g,
// float4 loads and stores); the stride is a multiple of K/4, so a thread's
// column group g = threadIdx.x % (K/4) never changes.
#define BSTRIDE ((long)gridDim.x * blockDim.x)
#define BLOOP(i)                                                      \
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; \
       i += BSTRIDE)
#define ULOOP(j)                                                           \
  for (long j = (long)blockIdx.x * blockDim.x + threadIdx.x; j < (a.n >> 2); \
       j += BSTRIDE)

__device__ __forceinline__ float4 ld4(const float *p, long j) {
  return reinterpret_cast<const float4 *>(p)[j];
}
__device__ __forceinline__ void st4(float *p, long j, float4 v) {
  reinterpret_cast<float4 *>(p)[j] = v;
}
__device__ __forceinline__ float f4(const float4 &v, int c) {
  return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
}

// col_grid_sum for threads that own four columns: each block first adds,
// per column 4g + c, the values of its threads with column group g, then
// the last block combines the blocks as col_grid_sum does.
template <int NQ>
__device__ __forceinline__ bool col_grid_sum4(double (&v)[NQ][4], const BVec &a,
                                              double *out /* [NQ][K] */) {
  __shared__ double sm4[NQ][4][BT];
  const int K = a.K, Q = K >> 2;
  const int tid = threadIdx.x;
#pragma unroll
  for (int q = 0; q < NQ; q++)
#pragma unroll
    for (int c = 0; c < 4; c++) sm4[q][c][tid] = v[q][c];
  __syncthreads();
  double w[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) w[q] = 0.0;
  if (tid < K) {
    const int g = tid >> 2, c = tid & 3;
#pragma unroll
    for (int q = 0; q < NQ; q++)
      for (int t = g; t < BT; t += Q) w[q] += sm4[q][c][t];
  }
  // the block's per-column sums now sit in threads tid < K: hand them to the
  // one-column-per-thread reduction (threads tid >= K contribute zero)
  return col_grid_sum<NQ>(w, a, out);
}

// r = b - r (r holds A x); rh = r; per-column norms; columns with b = 0 are
// inactive from the start.
__global__ void __launch_bounds__(BT, 2) bb_start(BVec a) {
  DfAcc d0[4], d1[4];
#pragma unroll
  for (int c = 0; c < 4; c++) d0[c] = d1[c] = DfAcc{0.f, 0.f};
  ULOOP(j) {
    const float4 bv = ld4(a.b, j), rv = ld4(a.r, j);
    const float4 ri = make_float4(bv.x - rv.x, bv.y - rv.y, bv.z - rv.z, bv.w - rv.w);
    st4(a.r, j, ri);
    st4(a.rh, j, ri);
#pragma unroll
    for (int c = 0; c < 4; c++) {
      dot_acc(d0[c], f4(bv, c), f4(bv, c));
      dot_acc(d1[c], f4(ri, c), f4(ri, c));
    }
  }
  double v[2][4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    v[0][c] = dot_val(d0[c]);
    v[1][c] = dot_val(d1[c]);
  }
  __shared__ double out[2 * 64];
  if (col_grid_sum4<2>(v, a, out)) {
    const int k = threadIdx.x;
    const double bb = out[k], rr = out[a.K + k];
    a.c.bnrm2[k] = bb;
    a.c.rho[k] = rr;
    a.c.rho_old[k] = 1.0;
    a.c.alpha[k] = 1.0;
    a.c.omega[k] = 1.0;
    a.c.sconv[k] = 0;
    const double err = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    a.c.err[k] = err;
    a.c.active[k] = (bb > 0.0 && err > a.c.tol[k] &&
                     !(a.outer_err && a.outer_err[k] <= a.outer_tol)) ? 1 : 0;
    a.c.status[k] = a.c.active[k] ? VDR_NOT_CONVERGED : VDR_OK;
  }
}

__global__ void bb_finish_start(BVec a) {  // one block: any column active?
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  if (threadIdx.x < a.K && a.c.active[threadIdx.x]) any = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    a.st->iter = 0;
    a.st->done = any ? 0 : 1;
  }
}

// p = r + beta (p - omega v) (p = r on the first iteration); v = 0;
// inactive columns get p = 0.
__global__ void __launch_bounds__(BT, 2) bb_p(BVec a) {
  if (a.st->done) return;
  const int k0 = 4 * (threadIdx.x & ((a.K >> 2) - 1));
  const bool first = a.st->iter == 0;
  float beta[4], om[4];
  bool on[4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const int k = k0 + c;
    on[c] = a.c.active[k] != 0;
    beta[c] = first ? 0.f
        : (float)((a.c.rho[k] / a.c.rho_old[k]) * (a.c.alpha[k] / a.c.omega[k]));
    om[c] = (float)a.c.omega[k];
  }
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  ULOOP(j) {
    const float4 rv = ld4(a.r, j);
    const float4 pv = first ? z4 : ld4(a.p, j);
    const float4 vv = first ? z4 : ld4(a.v, j);
    float o[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const float r = f4(rv, c), p = f4(pv, c), v = f4(vv, c);
      o[c] = on[c] ? (first ? r : r + beta[c] * (p - om[c] * v)) : 0.f;
    }
    st4(a.p, j, make_float4(o[0], o[1], o[2], o[3]));
    st4(a.v, j, z4);
  }
}

__global__ void __launch_bounds__(BT, 2) bb_alpha(BVec a) {
  if (a.st->done) return;
  DfAcc d0[4];
#pragma unroll
  for (int c = 0; c < 4; c++) d0[c] = DfAcc{0.f, 0.f};
  ULOOP(j) {
    const float4 hv = ld4(a.rh, j), vv = ld4(a.v, j);
#pragma unroll
    for (int c = 0; c < 4; c++) dot_acc(d0[c], f4(hv, c), f4(vv, c));
  }
  double v[1][4];
#pragma unroll
  for (int c = 0; c < 4; c++) v[0][c] = dot_val(d0[c]);
  __shared__ double out[64];
  if (col_grid_sum4<1>(v, a, out)) {
    const int k = threadIdx.x;
    if (a.c.active[k]) {
      const double rv = out[k];
      if (rv == 0.0 || !isfinite(rv)) {
        a.c.active[k] = 0;
        a.c.status[k] = VDR_BREAKDOWN;
        a.c.alpha[k] = 0.0;
      } else {
        a.c.alpha[k] = a.c.rho[k] / rv;
      }
    }
  }
}

// s = r - alpha v; t = 0; ||s|| per column.
__global__ void __launch_bounds__(BT, 2) bb_s(BVec a) {
  if (a.st->done) return;
  const int k0 = 4 * (threadIdx.x & ((a.K >> 2) - 1));
  float al[4];
#pragma unroll
  for (int c = 0; c < 4; c++)
    al[c] = a.c.active[k0 + c] ? (float)a.c.alpha[k0 + c] : 0.f;
  DfAcc d0[4];
#pragma unroll
  for (int c = 0; c < 4; c++) d0[c] = DfAcc{0.f, 0.f};
  ULOOP(j) {
    const float4 rv = ld4(a.r, j), vv = ld4(a.v, j);
    float sv[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      sv[c] = f4(rv, c) - al[c] * f4(vv, c);
      dot_acc(d0[c], sv[c], sv[c]);
    }
    st4(a.s, j, make_float4(sv[0], sv[1], sv[2], sv[3]));
    st4(a.t, j, make_float4(0.f, 0.f, 0.f, 0.f));
  }
  double v[1][4];
#pragma unroll
  for (int c = 0; c < 4; c++) v[0][c] = dot_val(d0[c]);
  __shared__ double out[64];
  if (col_grid_sum4<1>(v, a, out)) {
    const int k = threadIdx.x;
    const double sn = a.c.bnrm2[k] > 0.0 ? sqrt(out[k] / a.c.bnrm2[k]) : 0.0;
    a.c.snrm[k] = sn;
    a.c.sconv[k] = (a.c.active[k] && sn <= a.c.tol[k]) ? 1 : 0;
  }
}

__global__ void __launch_bounds__(BT, 2) bb_omega(BVec a) {
  if (a.st->done) return;
  DfAcc d0[4], d1[4];
#pragma unroll
  for (int c = 0; c < 4; c++) d0[c] = d1[c] = DfAcc{0.f, 0.f};
  ULOOP(j) {
    const float4 tv = ld4(a.t, j), sv = ld4(a.s, j);
#pragma unroll
    for (int c = 0; c < 4; c++) {
      dot_acc(d0[c], f4(tv, c), f4(sv, c));
      dot_acc(d1[c], f4(tv, c), f4(tv, c));
    }
  }
  double v[2][4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    v[0][c] = dot_val(d0[c]);
    v[1][c] = dot_val(d1[c]);
  }
  __shared__ double out[2 * 64];
  if (col_grid_sum4<2>(v, a, out)) {
    const int k = threadIdx.x;
    if (a.c.active[k] && !a.c.sconv[k]) {
      const double ts = out[k], tt = out[a.K + k];
      if (tt == 0.0 || !isfinite(tt) || !isfinite(ts)) {
        a.c.omega[k] = 0.0;
      } else {
        a.c.omega[k] = ts / tt;
      }
    }
  }
}

// x += D^-1 (alpha p + omega s) (Dirichlet entries stay); r = s - omega t
// (r = s when s already met the tolerance); norms for the next iteration.
// Inactive columns keep x and r.
__global__ void __launch_bounds__(BT, 2) bb_xr(BVec a) {
  if (a.st->done) return;
  const int k0 = 4 * (threadIdx.x & ((a.K >> 2) - 1));
  const int qshift = a.kshift - 2;  // units per node row = 1 << qshift
  bool act[4];
  float al[4], om[4];
  bool any_act = false;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const int k = k0 + c;
    act[c] = a.c.active[k] != 0;
    const bool sc = a.c.sconv[k] != 0;
    al[c] = act[c] ? (float)a.c.alpha[k] : 0.f;
    om[c] = (act[c] && !sc) ? (float)a.c.omega[k] : 0.f;
    any_act |= act[c];
  }
  DfAcc d0[4], d1[4];
#pragma unroll
  for (int c = 0; c < 4; c++) d0[c] = d1[c] = DfAcc{0.f, 0.f};
  ULOOP(j) {
    const long node = j >> qshift;
    const float4 hv = ld4(a.rh, j), rv = ld4(a.r, j);
    float4 xv = make_float4(0.f, 0.f, 0.f, 0.f), pv = xv, sv = xv, tv = xv;
    float dn = 0.f;
    if (any_act) {
      xv = ld4(a.x, j);
      pv = ld4(a.p, j);
      sv = ld4(a.s, j);
      tv = ld4(a.t, j);
      dn = a.m[node] ? 0.f : a.dinv[node];
    }
    float xo[4], ro[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float ri = f4(rv, c), xi = f4(xv, c);
      if (act[c]) {
        ri = f4(sv, c) - om[c] * f4(tv, c);
        xi = xi + dn * (al[c] * f4(pv, c) + om[c] * f4(sv, c));
      }
      xo[c] = xi;
      ro[c] = ri;
      dot_acc(d0[c], ri, ri);
      dot_acc(d1[c], f4(hv, c), ri);
    }
    if (any_act) {
      st4(a.x, j, make_float4(xo[0], xo[1], xo[2], xo[3]));
      st4(a.r, j, make_float4(ro[0], ro[1], ro[2], ro[3]));
    }
  }
  double v[2][4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    v[0][c] = dot_val(d0[c]);
    v[1][c] = dot_val(d1[c]);
  }
  __shared__ double out[2 * 64];
  if (col_grid_sum4<2>(v, a, out)) {
    const int k = threadIdx.x;
    if (a.c.active[k]) {
      const bool sc = a.c.sconv[k] != 0;
      const double omk = a.c.omega[k];
      a.c.rho_old[k] = a.c.rho[k];
      a.c.rho[k] = out[a.K + k];
      const double err = sqrt(out[k] / a.c.bnrm2[k]);
      a.c.err[k] = err;
      if (!(err == err)) {
        a.c.active[k] = 0;
        a.c.status[k] = VDR_BREAKDOWN;
      } else if (err <= a.c.tol[k] || sc) {
        a.c.active[k] = 0;
        a.c.status[k] = VDR_OK;
      } else if (out[a.K + k] == 0.0 || (float)omk == 0.f) {
        a.c.active[k] = 0;
        a.c.status[k] = VDR_BREAKDOWN;
      }
    }
  }
}

// After an iteration: iteration count, and done when no column is active
// or itmax is reached.
__global__ void bb_tail(BVec a) {
  if (a.st->done) return;
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  if (threadIdx.x < a.K && a.c.active[threadIdx.x]) any = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    a.st->iter += 1;
    if (!any || a.st->iter >= a.st->itmax) a.st->done = 1;
  }
}

// ------------------------------------------------ FP64 <-> FP32 block glue
// R = B - R (R holds A X) in FP64; per-column max |R| and max |B|.
__global__ void __launch_bounds__(BT, 2) bo_residual(BVec a, const double *B,
                                                  double *R, double *mx) {
  const int k = threadIdx.x & (a.K - 1);
  double v[2] = {0.0, 0.0};
  BLOOP(i) {
    const double bi = B[i];
    const double ri = bi - R[i];
    R[i] = ri;
    v[0] = fmax(v[0], fabs(ri));
    v[1] = fmax(v[1], fabs(bi));
  }
  __shared__ double out[2 * 64];
  if (col_grid_sum<2, true>(v, a, out)) {
    mx[k] = out[k];
    mx[a.K + k] = out[a.K + k];
  }
}

// Per-column scale 2^e >= max |R_k| (a power of two, so scaling is exact);
// Rf = R / scale in FP32 (values in [-1, 1]); err_k = ||R_k|| / ||B_k||
// from the norms of the max-scaled columns (no overflow or underflow).
__global__ void __launch_bounds__(BT, 2) bo_scale(BVec a, const double *B,
                                               const double *R, float *Rf,
                                               const double *mx, double *scale,
                                               double *err_out) {
  const int k = threadIdx.x & (a.K - 1);
  const double rm = mx[k], bm = mx[a.K + k];
  int er = 0;
  if (rm > 0.0 && isfinite(rm)) frexp(rm, &er);
  const double inv_r = ldexp(1.0, -er);
  const double inv_b = (bm > 0.0 && isfinite(bm)) ? 1.0 / bm : 1.0;
  double v[2] = {0.0, 0.0};
  BLOOP(i) {
    const double rs = R[i] * inv_r;
    Rf[i] = (float)rs;
    v[0] += rs * rs;
    const double bs = B[i] * inv_b;
    v[1] += bs * bs;
  }
  __shared__ double out[2 * 64];
  if (col_grid_sum<2>(v, a, out)) {
    scale[k] = ldexp(1.0, er);
    double err;
    if (!(rm == rm) || isinf(rm)) err = rm + rm;   // NaN / inf propagate
    else if (rm == 0.0) err = 0.0;
    else if (!(bm > 0.0)) err = INFINITY;          // zero column, nonzero R
    else err = (ldexp(1.0, er) * sqrt(out[k])) / (bm * sqrt(out[a.K + k]));
    err_out[k] = err;
  }
}

__global__ void bo_update(long n, int K, double *X, const float *D,
                          const double *scale) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    X[i] += (double)D[i] * scale[i & (K - 1)];
}

// X = 0 on Dirichlet rows; *nonzero set when any entry is left nonzero.
__global__ void bo_mask(long n, int kshift, double *X, const unsigned char *m, int *nonzero) {
  bool nz = false;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    if (m[i >> kshift]) X[i] = 0.0;
    else if (X[i] != 0.0) nz = true;
  }
  if (__any_sync(FULL, nz) && (threadIdx.x & 31) == 0) atomicOr(nonzero, 1);
}

__global__ void dinv_to_f32(const double *__restrict__ d, float *__restrict__ f,
                            int N) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (long)gridDim.x * blockDim.x)
    f[i] = (float)d[i];
}

// Resident blocks per SM of `kern`, queried once per instantiation.
template <typename Kern>
int cached_per_sm(std::atomic<int> &slot, Kern kern, int threads, int smem) {
  int n = slot.load(std::memory_order_relaxed);
  if (n > 0) return n;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem);
  if (n < 1) n = 1;
  slot.store(n, std::memory_order_relaxed);
  return n;
}

int grid_n(long n, int threads, int per_sm) {
  const long need = (n + threads - 1) / threads;
  return (int)std::max<long>(1, std::min<long>(need, (long)device_sm_count() * per_sm));
}

// One block per TILE_X x TY x TILE_Z box of elements and column half; the
// dynamic shared memory above 48 KB is opted into once per device.
template <bool SPLIT, int TILES, int TY, int HALVES>
void launch_tile(const Handle &h, const float *A, const float *X, float *Y,
                 const int *skip, const unsigned char *mask, cudaStream_t s) {
  constexpr int smem = tile_smem_bytes<TY, 16 * TILES>();
  static std::atomic<unsigned> opted{0u};
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned bit = 1u << (dev & 31);
  if (!(opted.load(std::memory_order_relaxed) & bit)) {
    cudaFuncSetAttribute(block_apply_tile<SPLIT, TILES, TY, HALVES>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    opted.fetch_or(bit, std::memory_order_relaxed);
  }
  const long tiles = (long)((h.nax - 2) / TILE_X + 1) * ((h.nay - 2) / TY + 1) *
                     ((h.naz - 2) / TILE_Z + 1);
  block_apply_tile<SPLIT, TILES, TY, HALVES>
      <<<(unsigned)(tiles * HALVES), 64 * TY, smem, s>>>(A, h.nax, h.nay, h.naz,
                                                         mask, X, Y, skip);
}

// K = 64: the box height (TILE_Y = 2 or 4 element rows) and whether the 64
// columns run as two blocks of 32 or one block of 64 are chosen by
// measurement (tune_block_apply; two halves of 32 at TILE_Y = 2 measured
// 0.43 vs 0.51 ms per apply at 1M elements when this was fixed by hand).
template <bool SPLIT>
void launch_tile_64(const Handle &h, const float *A, const float *X, float *Y,
                    const int *skip, const unsigned char *mask, cudaStream_t s) {
  if (h.blk_ty == 4) launch_tile<SPLIT, 2, 4, 2>(h, A, X, Y, skip, mask, s);
  else if (h.blk_halves == 1) launch_tile<SPLIT, 4, TILE_Y, 1>(h, A, X, Y, skip, mask, s);
  else launch_tile<SPLIT, 2, TILE_Y, 2>(h, A, X, Y, skip, mask, s);
}

void launch_tile_k(const Handle &h, int K, bool split, const float *A,
                   const float *X, float *Y, const int *skip,
                   const unsigned char *mask, cudaStream_t s) {
  if (split) {
    if (K == 16) launch_tile<true, 1, TILE_Y, 1>(h, A, X, Y, skip, mask, s);
    else if (K == 32) launch_tile<true, 2, TILE_Y, 1>(h, A, X, Y, skip, mask, s);
    else launch_tile_64<true>(h, A, X, Y, skip, mask, s);
  } else {
    if (K == 16) launch_tile<false, 1, TILE_Y, 1>(h, A, X, Y, skip, mask, s);
    else if (K == 32) launch_tile<false, 2, TILE_Y, 1>(h, A, X, Y, skip, mask, s);
    else launch_tile_64<false>(h, A, X, Y, skip, mask, s);
  }
}

}  // namespace

// ------------------------------------------------------------ host side
int block_apply_launches_tf32(const Handle &h, int K, bool split,
                              const float *X, const float *dscale, float *Y,
                              const float4 *Aaos, const int *skip,
                              cudaStream_t s, bool x_clean) {
  const float *A = reinterpret_cast<const float *>(Aaos);
  // The node-tile apply needs the canonical structured numbering in storage
  // order (not the colour permutation), and any scale folded into the
  // operator copy.
  if (!h.block_tma && h.block_tile && h.nax > 1 && h.nay > 1 && h.naz > 1 &&
      !h.perm_d && !dscale && !(reinterpret_cast<uintptr_t>(X) & 15) &&
      !(reinterpret_cast<uintptr_t>(Y) & 15)) {
    // K = 64: the tcgen05 box apply when requested or measured fastest
    if (K == 64 && (h.blk_tc_mode == 1 || (h.blk_tc_mode < 0 && h.blk_use_tc)) &&
        block_tc_supported(h))
      return launch_block_tc(h, split, A, X, Y, skip, x_clean ? nullptr : h.mask, s);
    launch_tile_k(h, K, split, A, X, Y, skip, x_clean ? nullptr : h.mask, s);
    count_launches(1);
    return cudaGetLastError() == cudaSuccess ? VDR_OK : VDR_CUDA_ERROR;
  }
  // Bulk copies need 16-byte aligned rows (K * 4 bytes is a multiple of 16).
  const bool tma = h.block_tma && h.block_err &&
                   !(reinterpret_cast<uintptr_t>(X) & 15) &&
                   !(reinterpret_cast<uintptr_t>(Y) & 15);
  if (tma) {
#define VDR_BLOCK_TMA(SPLIT, TILES)                                               \
  do {                                                                            \
    constexpr int KK = 16 * TILES;                                                \
    const int smem = TMA_WARPS * (TMA_S * 8 * (KK + 8) + 2 * 8 * (KK + 4)) * 4;   \
    static std::atomic<int> slot{0};                                              \
    const int per_sm = cached_per_sm(slot, block_apply_tma<SPLIT, TILES>,         \
                                     TMA_WARPS * 32, smem);                       \
    block_apply_tma<SPLIT, TILES><<<grid_n((long)h.E * 32, TMA_WARPS * 32,        \
                                           per_sm),                               \
                                    TMA_WARPS * 32, smem, s>>>(                   \
        A, h.conn, h.E, X, dscale, Y, skip, h.block_err);                         \
  } while (0)
    if (split) {
      if (K == 16) VDR_BLOCK_TMA(true, 1);
      else if (K == 32) VDR_BLOCK_TMA(true, 2);
      else VDR_BLOCK_TMA(true, 4);
    } else {
      if (K == 16) VDR_BLOCK_TMA(false, 1);
      else if (K == 32) VDR_BLOCK_TMA(false, 2);
      else VDR_BLOCK_TMA(false, 4);
    }
#undef VDR_BLOCK_TMA
    count_launches(1);
    return cudaGetLastError() == cudaSuccess ? VDR_OK : VDR_CUDA_ERROR;
  }
#define VDR_BLOCK_APPLY(SPLIT, TILES)                                        \
  do {                                                                       \
    static std::atomic<int> slot{0};                                         \
    const int per_sm =                                                       \
        cached_per_sm(slot, block_apply_tf32<SPLIT, TILES>, 256, 0);         \
    block_apply_tf32<SPLIT, TILES><<<grid_n((long)h.E * 32, 256, per_sm),    \
                                     256, 0, s>>>(A, h.conn, h.E, X, dscale, \
                                                  Y, skip);                  \
  } while (0)
  if (split) {
    if (K == 16) VDR_BLOCK_APPLY(true, 1);
    else if (K == 32) VDR_BLOCK_APPLY(true, 2);
    else VDR_BLOCK_APPLY(true, 4);
  } else {
    if (K == 16) VDR_BLOCK_APPLY(false, 1);
    else if (K == 32) VDR_BLOCK_APPLY(false, 2);
    else VDR_BLOCK_APPLY(false, 4);
  }
#undef VDR_BLOCK_APPLY
  count_launches(1);
  return cudaGetLastError() == cudaSuccess ? VDR_OK : VDR_CUDA_ERROR;
}

cudaError_t launch_block_apply64(const Handle &h, int K, const double *X,
                                 double *Y, cudaStream_t s) {
  const int grid = grid_n((long)h.E * 32, 256, 8);
  if (h.storage == VDR_STORE_DF && h.Ahi)
    block_apply_df<<<grid, 256, 0, s>>>(h.Ahi, h.Alo, h.conn, h.E, K, X, Y);
  else
    block_apply_f64<<<grid, 256, 0, s>>>(h.A64, h.conn, h.E, K, X, Y);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_block_rhs(const Handle &h, const double *phi, int K,
                             const double *Q, double cf, double *B,
                             cudaStream_t s) {
  block_rhs<<<grid_n((long)h.E * K, 256, 8), 256, 0, s>>>(phi, h.conn, h.E, K,
                                                          Q, h.perm_d, cf, B);
  count_launches(1);
  return cudaGetLastError();
}

// The K = 64 block apply's form by measurement, once per handle and
// before any capture: the node tile at (box height, column halves) (2, 2),
// (2, 1), (4, 2) and the tcgen05 box apply, each timed over 3 applies of X
// into the scratch Y after one warm-up; the fastest is kept.
int tune_block_apply(Handle &h, const float *X, float *Y, const float4 *Aaos) {
  if (h.blk_tuned) return VDR_OK;
  h.blk_tuned = true;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h.stream, &cs) != cudaSuccess ||
      cs != cudaStreamCaptureStatusNone || h.E < 65536 || !h.block_tile ||
      h.block_tma || !(h.nax > 1 && h.nay > 1 && h.naz > 1) || h.perm_d)
    return VDR_OK;
  // candidates 0-2: node-tile shapes; 3: the tcgen05 box apply
  const int ty[TUNE_TILES] = {2, 2, 4, 2}, halves[TUNE_TILES] = {2, 1, 2, 2};
  const int ncand = (block_tc_supported(h) && h.blk_tc_mode != 0) ? TUNE_TILES : TUNE_TILES - 1;
  cudaEvent_t e0, e1;
  cudaError_t e;
  if ((e = cudaEventCreate(&e0))) return cuda_fail(e, "tune events");
  if ((e = cudaEventCreate(&e1))) {
    cudaEventDestroy(e0);
    return cuda_fail(e, "tune events");
  }
  float best = 1e30f;
  int bi = 0;
  const float *A = reinterpret_cast<const float *>(Aaos);
  int st = VDR_OK;
  for (int c = 0; c < ncand && !e && !st; c++) {
    h.blk_ty = ty[c];
    h.blk_halves = halves[c];
    auto launch = [&]() {
      if (c == TUNE_TILES - 1)
        return launch_block_tc(h, true, A, X, Y, nullptr, nullptr, h.stream);
      launch_tile_k(h, 64, true, A, X, Y, nullptr, nullptr, h.stream);
      count_launches(1);
      return VDR_OK;
    };
    if ((st = launch())) break;  // warm
    cudaEventRecord(e0, h.stream);
    for (int rep = 0; rep < 3 && !st; rep++) st = launch();
    cudaEventRecord(e1, h.stream);
    if (st || (e = cudaEventSynchronize(e1))) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    h.blk_tune_ms[c] = ms / 3.f;
    if (ms < best) {
      best = ms;
      bi = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if (e) return cuda_fail(e, "block apply tuning");
  h.blk_use_tc = bi == TUNE_TILES - 1;
  h.blk_ty = ty[bi];
  h.blk_halves = halves[bi];
  return VDR_OK;
}

// Element-major FP32 copy of the operator for the tensor-core applies (and
// the error flag of their bounded waits); `scaled`: the Jacobi
// preconditioner h.dinv32 folded into the columns (the block solve), else
// the plain operator (the block apply of the C ABI).
cudaError_t ensure_aos(Handle &h, bool scaled, float4 **out) {
  cudaError_t e;
  if (!h.block_err) {
    if ((e = cudaMalloc(&h.block_err, sizeof(int)))) return e;
    if ((e = cudaMemset(h.block_err, 0, sizeof(int)))) return e;
  }
  if (!h.Aaos) {
    if ((e = cudaMalloc(&h.Aaos, sizeof(float4) * 16 * (size_t)h.E))) return e;
    h.aos_valid = false;
  }
  if (!h.aos_valid || h.aos_scaled != scaled) {
    const int grid = grid_n((long)h.E * 16, 256, 16);
    const float *cs = scaled ? h.dinv32 : nullptr;
    if (h.storage == VDR_STORE_DF && h.Ahi)
      aos_build<false><<<grid, 256, 0, h.stream>>>(h.Ahi, nullptr, h.conn, h.E, cs, h.Aaos);
    else
      aos_build<true><<<grid, 256, 0, h.stream>>>(nullptr, h.A64, h.conn, h.E, cs, h.Aaos);
    count_launches(1);
    if ((e = cudaGetLastError())) return e;
    h.aos_valid = true;
    h.aos_scaled = scaled;
  }
  *out = h.Aaos;
  return cudaSuccess;
}

namespace {
// device workspace of the block solve, carved from h.bk_f / h.bk_d
constexpr int BK_COLS = 16 * 64;            // per-column doubles and ints
constexpr int BK_PARTIALS = 2 * 64 * 2048;  // NQ x K x blocks
constexpr int BK_MAX_GRID = 2048;
}  // namespace

// The bulk-copy wait's timeout path, end to end: VDR_TIMEOUT when a wait
// that nothing completes ran out of its (about 1 ms) budget and the flag
// reached the host; the context stays usable.
int diag_wait_timeout(Handle &h) {
  cudaError_t e;
  if (!h.block_err && (e = cudaMalloc(&h.block_err, sizeof(int))))
    return cuda_fail(e, "diag: alloc");
  int flag = 0;
  if ((e = cudaMemsetAsync(h.block_err, 0, sizeof(int), h.stream))) return cuda_fail(e, "diag");
  wait_timeout_kernel<<<1, 32, 0, h.stream>>>(h.block_err, 2000000LL);
  count_launches(1);
  if ((e = cudaGetLastError()) ||
      (e = cudaMemcpyAsync(&flag, h.block_err, sizeof(int), cudaMemcpyDeviceToHost,
                           h.stream)) ||
      (e = cudaMemsetAsync(h.block_err, 0, sizeof(int), h.stream)) ||
      (e = cudaStreamSynchronize(h.stream)))
    return cuda_fail(e, "diag");
  if (!flag) {
    set_error("diag: the wait completed although nothing arrived");
    return VDR_CUDA_ERROR;
  }
  set_error("diag: the bounded wait ran out as designed");
  return VDR_TIMEOUT;
}

// Block solve: FP64 refinement around K-column FP32 BiCGStab with the TF32
// tensor-core apply.  B, X are N x K FP64 device arrays (node-major).
int solve_block_device(Handle &h, int K, int precision, const double *B,
                       double *X, double tol, double inner_tol, int max_outer,
                       int inner_itmax, int *outer_iters, int *inner_iters,
                       double *errs_host) {
  if (K != 16 && K != 32 && K != 64) {
    set_error("block solve: K must be 16, 32 or 64");
    return VDR_BAD_ARGUMENT;
  }
  if (precision != VDR_BLOCK_TF32 && precision != VDR_BLOCK_TF32X3) {
    set_error("block solve: precision must be VDR_BLOCK_TF32 or VDR_BLOCK_TF32X3");
    return VDR_BAD_ARGUMENT;
  }
  const bool split = precision == VDR_BLOCK_TF32X3;
  cudaError_t e;
  cudaStream_t s = h.stream;
  const long n = (long)h.N * K;
  if (h.bk_K != K || !h.bk_f) {
    if (h.bk_f) cudaFree(h.bk_f);
    if (h.bk_d) cudaFree(h.bk_d);
    h.bk_f = nullptr;
    h.bk_d = nullptr;
    h.bk_K = 0;
    if (h.bk_graph) cudaGraphExecDestroy(h.bk_graph);
    h.bk_graph = nullptr;
    if ((e = cudaMalloc(&h.bk_f, sizeof(float) * 8 * (size_t)n)) ||
        (e = cudaMalloc(&h.bk_d, sizeof(double) * ((size_t)n + BK_COLS +
                                                   BK_PARTIALS + 8))))
      return cuda_fail(e, "block workspace");
    h.bk_K = K;
  }
  if (!h.dinv32 && (e = cudaMalloc(&h.dinv32, sizeof(float) * (size_t)h.N)))
    return cuda_fail(e, "block workspace");
  float *fv = h.bk_f;
  double *R = h.bk_d;
  double *colsd = R + n;
  double *partials = colsd + BK_COLS;
  BState *st = reinterpret_cast<BState *>(partials + BK_PARTIALS);
  BVec a{};
  a.n = n;
  a.K = K;
  a.kshift = K == 16 ? 4 : (K == 32 ? 5 : 6);
  a.st = st;
  a.partials = partials;
  a.c.bnrm2 = colsd + 0 * 64;
  a.c.err = colsd + 1 * 64;
  a.c.rho = colsd + 2 * 64;
  a.c.rho_old = colsd + 3 * 64;
  a.c.alpha = colsd + 4 * 64;
  a.c.omega = colsd + 5 * 64;
  a.c.snrm = colsd + 6 * 64;
  double *outer_err = colsd + 7 * 64;
  double *mx = colsd + 8 * 64;      // 2 x 64
  double *scale = colsd + 10 * 64;
  int *colsi = reinterpret_cast<int *>(colsd + 11 * 64);  // 3 x 64 ints + a flag
  a.c.tol = colsd + 13 * 64;
  a.c.active = colsi;
  a.c.sconv = colsi + 64;
  a.c.status = colsi + 128;
  a.m = h.mask;
  a.dinv = h.dinv32;
  a.outer_err = outer_err;
  a.outer_tol = tol;
  float *bf = fv;  // inner right-hand side: scaled FP32 residual
  a.b = bf;
  a.x = fv + 1 * n;
  a.r = fv + 2 * n;
  a.rh = fv + 3 * n;
  a.p = fv + 4 * n;
  a.v = fv + 5 * n;
  a.s = fv + 6 * n;
  a.t = fv + 7 * n;

  dinv_to_f32<<<grid_n(h.N, 256, 8), 256, 0, s>>>(h.dinv, h.dinv32, h.N);
  count_launches(1);
  if ((e = cudaGetLastError())) return cuda_fail(e, "block setup");
  // The apply's operator copy carries the Jacobi scale (A D^-1).
  float4 *Aaos = nullptr;
  if ((e = ensure_aos(h, true, &Aaos))) return cuda_fail(e, "block operator copy");
  if (K == 64 && !h.blk_tuned) {  // launch shape by measurement, before capture
    if ((e = cudaMemsetAsync(a.p, 0, sizeof(float) * 2 * n, s)))
      return cuda_fail(e, "block tuning");
    const int tst = tune_block_apply(h, a.p, a.v, Aaos);
    if (tst) return tst;
    if (h.bk_graph) cudaGraphExecDestroy(h.bk_graph);
    h.bk_graph = nullptr;
  }
  const int gv = std::min(BK_MAX_GRID, grid_n(n, BT, 2));  // one wave
  const int gm = grid_n(n, 256, 8);
  // the initial guess masked; a zero one makes the first residual B itself
  int *x_nonzero = colsi + 3 * 64;
  int x_nz_host = 1;
  if ((e = cudaMemsetAsync(x_nonzero, 0, sizeof(int), s))) return cuda_fail(e, "block setup");
  bo_mask<<<gm, 256, 0, s>>>(n, a.kshift, X, h.mask, x_nonzero);
  count_launches(1);
  if ((e = cudaGetLastError()) ||
      (e = cudaMemcpyAsync(&x_nz_host, x_nonzero, sizeof(int), cudaMemcpyDeviceToHost, s)) ||
      (e = cudaStreamSynchronize(s)))
    return cuda_fail(e, "block setup");

  // KI inner iterations per graph launch (8 kernels each)
  constexpr int KI = 4;
  if (!h.bk_graph || h.bk_graph_split != split) {
    if (h.bk_graph) cudaGraphExecDestroy(h.bk_graph);
    h.bk_graph = nullptr;
    cudaGraph_t graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)))
      return cuda_fail(e, "capture");
    for (int it = 0; it < KI; it++) {
      bb_p<<<gv, BT, 0, s>>>(a);
      block_apply_launches_tf32(h, K, split, a.p, nullptr, a.v, Aaos,
                                &st->done, s, true);
      bb_alpha<<<gv, BT, 0, s>>>(a);
      bb_s<<<gv, BT, 0, s>>>(a);
      block_apply_launches_tf32(h, K, split, a.s, nullptr, a.t, Aaos,
                                &st->done, s, true);
      bb_omega<<<gv, BT, 0, s>>>(a);
      bb_xr<<<gv, BT, 0, s>>>(a);
      bb_tail<<<1, 64, 0, s>>>(a);
    }
    count_launches(-2L * KI);  // the captured applies count at replay
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e2) return cuda_fail(e2, "end capture");
    e = cudaGraphInstantiate(&h.bk_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e) return cuda_fail(e, "instantiate");
    h.bk_graph_split = split;
  }

  BState init{};
  init.tol = inner_tol;
  init.itmax = inner_itmax;
  int total_inner = 0, outer = 0;
  std::vector<double> herr(K, 0.0), htol(K, inner_tol);
  int status = VDR_NOT_CONVERGED;
  for (outer = 0;; outer++) {
    // FP64 residual of every column, its scale and relative norm
    if ((e = cudaMemsetAsync(R, 0, sizeof(double) * n, s)) ||
        ((outer > 0 || x_nz_host) && (e = launch_block_apply64(h, K, X, R, s))) ||
        (e = cudaMemsetAsync(st, 0, sizeof(BState), s)))
      return cuda_fail(e, "block residual");
    bo_residual<<<gv, BT, 0, s>>>(a, B, R, mx);
    bo_scale<<<gv, BT, 0, s>>>(a, B, R, bf, mx, scale, outer_err);
    count_launches(2);
    if ((e = cudaMemcpyAsync(herr.data(), outer_err, sizeof(double) * K,
                             cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
      return cuda_fail(e, "block residual");
    double worst = 0.0;
    bool nan = false;
    for (int k = 0; k < K; k++) {
      if (!(herr[k] == herr[k])) nan = true;
      worst = std::max(worst, herr[k]);
    }
    if (nan) {
      status = VDR_BREAKDOWN;
      break;
    }
    if (worst <= tol) {
      status = VDR_OK;
      break;
    }
    if (outer >= max_outer) break;
    // K simultaneous FP32 inner solves of A D = R / scale, D = 0; column k
    // is solved to max(inner_tol, 0.5 tol / err_k): no further than its
    // outer residual needs to reach tol
    for (int k = 0; k < K; k++)
      htol[k] = herr[k] > 0.0 ? std::max(inner_tol, 0.5 * tol / herr[k]) : inner_tol;
    if ((e = cudaMemcpyAsync(a.c.tol, htol.data(), sizeof(double) * K,
                             cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync(st, &init, sizeof(BState), cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemsetAsync(a.x, 0, sizeof(float) * n, s)) ||
        (e = cudaMemsetAsync(a.r, 0, sizeof(float) * n, s)))
      return cuda_fail(e, "inner reset");
    bb_start<<<gv, BT, 0, s>>>(a);
    bb_finish_start<<<1, 64, 0, s>>>(a);
    count_launches(2);
    BState hs{};
    for (int c = 0; c * KI < inner_itmax + KI; c++) {
      if ((e = cudaGraphLaunch(h.bk_graph, s))) return cuda_fail(e, "graph");
      count_launches(8L * KI);
      if ((e = cudaMemcpyAsync(&hs, st, sizeof(BState), cudaMemcpyDeviceToHost, s)) ||
          (e = cudaStreamSynchronize(s)))
        return cuda_fail(e, "inner state");
      if (hs.done) break;
    }
    total_inner += hs.iter;
    bo_update<<<gm, 256, 0, s>>>(n, K, X, a.x, scale);
    count_launches(1);
    if ((e = cudaGetLastError())) return cuda_fail(e, "update");
  }
  if ((e = cudaStreamSynchronize(s))) return cuda_fail(e, "block solve");
  int tma_err = 0;
  if ((e = cudaMemcpy(&tma_err, h.block_err, sizeof(int), cudaMemcpyDeviceToHost)))
    return cuda_fail(e, "block solve");
  if (tma_err) {
    cudaMemset(h.block_err, 0, sizeof(int));
    set_error("block solve: a bounded device wait of the block apply ran out of time");
    return VDR_TIMEOUT;
  }
  if (outer_iters) *outer_iters = outer;
  if (inner_iters) *inner_iters = total_inner;
  if (errs_host)
    for (int k = 0; k < K; k++) errs_host[k] = herr[k];
  return status;
}

}  // namespace vdr
