// vdr_internal.h -- host-side internals shared by the translation units of
// libvdr.so.  Not installed; the public surface is include/vdr.h.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "vdr.h"

namespace vdr {

// A Dirichlet node is stored in the connectivity with this bit set, so the
// operator applies mask their inputs and outputs without extra loads.
constexpr int MASK_BIT = (int)0x80000000u;
constexpr int NODE_BITS = 0x7fffffff;

// Reduction scratch: per-block partial sums of up to MAXQ quantities.
constexpr int MAXQ = 4;
constexpr int RED_THREADS = 256;
constexpr int GCR_MAX_RESTART = 32;

// Device-resident Krylov state.  Scalars live here so that a captured
// iteration never needs the host; `done` gates every kernel of the graph.
struct KState {
  double bnrm2, err, snrm;
  double rho, rho_old, alpha, omega;       // BiCGStab
  double bknum, bkden, ak;                 // BiCG
  double tol;
  double best_err;   // lowest residual so far (stall detection)
  int iter, itmax, done, sconv, status, reason;  // reason: see vdr_solve_stats
  int since_best, stall_window;  // iterations without a 1% gain; 0 = off
  int x_zero;  // the initial guess is zero (its apply is skipped)
  unsigned int ticket;
  unsigned int pad2;
  unsigned int bar_count, bar_gen;  // grid barrier of the fused inner kernels
};

// A right preconditioner for BiCGStab beyond Jacobi: `enqueue` adds
// (M(in) - D^-1 in) to `out`, which already holds D^-1 in (zero on
// Dirichlet nodes).  Every kernel it enqueues returns at entry while
// *skip or *skip2 is nonzero, so the iteration can be captured in a graph.
struct Precond {
  cudaError_t (*enqueue)(void *ctx, const double *in, double *out,
                         const int *skip, const int *skip2, cudaStream_t s);
  void *ctx;
  int launches;  // kernels per enqueue
};

struct DeviceOp;  // forward

// Optional gate of the stored-matrix applies: element p is skipped when
// active[eseg[p]] == 0 (segments that have converged).
struct ElemGate {
  const int *eseg = nullptr;
  const int *active = nullptr;
};

// Element connectivity as the stored applies read it: the table (8 ints per
// element, Dirichlet flag in bit 31) or, on the canonical structured
// numbering in natural storage order, node numbers computed from the
// element number (element i + nex (j + ney k) has nodes i + nax j + pl k +
// {0, 1, 1 + nax, nax} and the same plus pl) with one byte of Dirichlet
// flags per element (bit s: local node s) -- 1 byte read instead of 32.
struct ConnView {
  const int *conn = nullptr;
  const unsigned char *emask = nullptr;  // structured when set
  int nex = 0, ney = 0, nax = 0, pl = 0;
};

// The 8 node numbers (| MASK_BIT on Dirichlet nodes) of one element:
// loaded from the table, or (STRUCT) formed on use from the element's first
// node and its Dirichlet bits, which keeps 4 registers live instead of 8.
template <bool STRUCT>
struct ElemNodes;
template <>
struct ElemNodes<false> {
  int c[8];
  __device__ __forceinline__ void load(const ConnView &cv, int E, long p) {
#pragma unroll
    for (int s = 0; s < 8; s++) c[s] = __ldg(cv.conn + (size_t)s * E + p);
  }
  __device__ __forceinline__ int operator[](int s) const { return c[s]; }
};
template <>
struct ElemNodes<true> {
  int base, nax, pl;
  unsigned m;
  __device__ __forceinline__ void load(const ConnView &cv, int E, long p) {
    const unsigned u = (unsigned)p, nx = (unsigned)cv.nex;
    const unsigned r = u / nx, i = u - r * nx;
    const unsigned k = r / (unsigned)cv.ney, j = r - k * (unsigned)cv.ney;
    nax = cv.nax;
    pl = cv.pl;
    base = (int)i + nax * (int)j + pl * (int)k;
    m = __ldg(cv.emask + p);
  }
  __device__ __forceinline__ int operator[](int s) const {
    const int s2 = s & 3;
    const int n = base + ((s2 == 1 || s2 == 2) ? 1 : 0) + ((s2 >> 1) ? nax : 0) +
                  ((s >> 2) ? pl : 0);
    return ((m >> s) & 1u) ? (n | MASK_BIT) : n;
  }
};

// Element-wise fields, device pointers in storage order.
struct Fields {
  const double *vel = nullptr;   // [3][E]
  const double *lam = nullptr;   // [E]
  const double *pdec = nullptr;  // [E] (nullable -> 0)
  const double *q = nullptr;     // [E] (nullable -> 0)
  const unsigned char *robin = nullptr;  // [E] (nullable -> none)
  double robin_alpha = 0.0;
};

// Everything an operator kernel needs, by value.
struct OpArgs {
  int E = 0, N = 0, variant = VDR_DR_VF;
  const int *conn = nullptr;  // [8][E]
  const double *xx = nullptr, *yy = nullptr, *zz = nullptr;
  const float *xx32 = nullptr, *yy32 = nullptr, *zz32 = nullptr;
  Fields f;
  const float *vel32 = nullptr, *lam32 = nullptr, *pdec32 = nullptr;
  double aH = 1.0, aM = 0.0;
};

// Candidate launch shapes of the apply tuner (tune.cu).
constexpr int TUNE_GRIDS = 5;   // resident blocks per SM: 2, 4, 8, 16, 32
constexpr int TUNE_TILES = 4;   // block apply: node tile (box height, column halves) (2,2)
                                // (2,1) (4,2), and the tcgen05 box apply
constexpr int TUNE_GRID_PER_SM[TUNE_GRIDS] = {2, 4, 8, 16, 32};

// Geometric factors of the double-float build, formed once per mesh (a
// handle's coordinates never change), double-float pairs (h, l), element
// index fastest:
//   Ji[(9 q + 3 a + b) E + p]  (J^-1)_{ab} = d xi_a / d x_b at Gauss point q
//   Dj[q E + p]                detJ at Gauss point q
//   K[t E + p]                 int gradN_i . gradN_j dOmega (unit
//                              diffusivity), t = i (15 - i) / 2 + j, i <= j
// 116 pairs = 928 bytes per element.
constexpr int GEO_PAIRS = 72 + 8 + 36;
struct GeoFactors {
  float2 *Ji = nullptr, *Dj = nullptr, *K = nullptr;
};

struct Handle {
  int N = 0, E = 0;
  int nax = 0, nay = 0, naz = 0;  // > 0 when the mesh is the canonical structured numbering
  int device = 0;
  cudaStream_t stream = nullptr;
  vdr_options opt{};
  // launch shapes chosen by measurement (tune.cu): resident blocks per SM
  // of the stored single-product applies' grids and of the binary16 apply,
  // the node-tile block apply's box height and column split (K = 64)
  int apply_per_sm = 8, half_per_sm = 8;
  bool apply_tuned = false, half_tuned = false;
  float apply_tune_ms[TUNE_GRIDS] = {}, half_tune_ms[TUNE_GRIDS] = {};
  int blk_ty = 2, blk_halves = 2;
  bool blk_use_tc = false;  // the tcgen05 box apply measured fastest (K = 64)
  bool blk_tuned = false;
  float blk_tune_ms[TUNE_TILES] = {};
  int scatter = VDR_SCATTER_ATOMIC;  // ATOMIC or COLOR (WARP is ATOMIC + warp_agg)
  bool warp_agg = false;  // warp-aggregated atomics on the structured numbering
  int apply_mode = VDR_APPLY_STORED;
  bool apply_fp32 = false;  // operator applies use the FP32 operator
  int storage = VDR_STORE_DF;  // element-matrix store (resolved, never AUTO)
  bool exact_build = false;    // H/M rows in FP64 (values outside the pair window)
  // the double-float build from the mesh's geometric factors, formed once
  // (geo_state 1), or from the coordinates at every build (build_mode
  // VDR_BUILD_RECOMPUTE, or geo_state -1: no room for them, a factor outside
  // the pair window)
  int build_mode = VDR_BUILD_AUTO;
  int geo_state = 0;
  GeoFactors geo;

  // geometry / topology (device, storage order)
  double *xx = nullptr, *yy = nullptr, *zz = nullptr;
  float *xx32 = nullptr, *yy32 = nullptr, *zz32 = nullptr;
  int *conn = nullptr;               // [8][E] 0-based | MASK_BIT
  unsigned char *emask = nullptr;    // [E] Dirichlet bits per element (structured)
  std::vector<int> perm;             // storage position -> element id
  std::vector<int> color_off;        // colour c occupies [off[c], off[c+1])
  int ncolors = 0;
  unsigned char *mask = nullptr;     // [N] 1 = Dirichlet
  bool mask_set = false;

  // fields (device, storage order)
  double *vel = nullptr, *lam = nullptr, *pdec = nullptr, *q = nullptr;
  float *vel32 = nullptr, *lam32 = nullptr, *pdec32 = nullptr;
  unsigned char *robin = nullptr;
  double robin_alpha = 0.0;
  bool fields_set = false;

  // operator state
  double aH = 1.0, aM = 0.0;
  bool op64_valid = false, op32_valid = false, diag_valid = false;
  double2 *A64 = nullptr;  // [32][E] stored element matrices (row-major pairs)
  float4 *A32 = nullptr;   // [16][E]
  const float4 *A32v = nullptr;  // the FP32 operator the FP32 apply reads (A32 or Ahi)
  int mixed_op = VDR_MIXED_HALF;
  // 16-bit inner operator of the mixed solve (half.cu): A^ = P A P D^-1 per
  // element in binary16 rows, uint4 A16[i*E + p], with a power-of-two
  // exponent per element; use_half once built and in range
  uint4 *A16 = nullptr;
  signed char *e16 = nullptr;
  bool use_half = false;
  float4 *Ahi = nullptr;   // [16][E] double-float store: hi parts
  float4 *Alo = nullptr;   // [16][E] double-float store: lo parts
  int *flag = nullptr;     // device flag: an entry left the FP32 range
  double *diag = nullptr;  // [N] assembled diagonal, 1 on Dirichlet nodes
  double *dinv = nullptr;  // [N] 1/diag (the Jacobi preconditioner)

  // solver workspace
  double *work = nullptr;
  int nwork = 0;
  // FP32-vector inner BiCGStab of the mixed solve: [10][N] floats (b, x, r,
  // rh, p, v, ph, s, sh, t) and its captured iterations
  float *work32 = nullptr;
  cudaGraphExec_t graph32 = nullptr;
  const void *graph32_key = nullptr;
  // the FP32 inner iteration with the binary16 operator, and the FP64
  // Jacobi-BiCGStab iteration, as two fused cooperative vector kernels each
  // (krylov.cu); off after a failed capture
  bool fused32 = true, fused64 = true;
  KState *st = nullptr;
  KState *h_st = nullptr;  // pinned mirror
  double *partials = nullptr;
  int red_blocks = 0;
  static constexpr int NGRAPH = 8;
  cudaGraphExec_t graph_exec[NGRAPH] = {};
  long long graph_size[NGRAPH] = {};  // (N << 32) | E the graph was captured for
  const void *graph_key[NGRAPH] = {};
  cudaEvent_t ev[2] = {nullptr, nullptr};

  // host staging
  double *h_stage = nullptr;
  size_t h_stage_bytes = 0;
  double *stage_d = nullptr;  // [3E] device staging of uploaded fields
  double *drs = nullptr;      // [5E] per-element DR scalars of the build
  float2 *gsc = nullptr;      // [10E] the same as pairs, with the fields (geometric-factor build)
  // time loop: the mass matrix M (double-float store) and the source vector
  // F = sum_e f_e of the current fields, so that later steps form their
  // right-hand side from two applies; rhs_tmp holds A T and M T
  float4 *Mhi = nullptr, *Mlo = nullptr;
  double *Fvec = nullptr, *rhs_tmp = nullptr;
  bool mass_valid = false;
  double *massw = nullptr;  // [8][E] integrate_mass weights (fixed geometry)

  vdr_solve_stats last{};

  // many right-hand sides (block.cu)
  float4 *Aaos = nullptr;    // element-major FP32 copy [E][64] for the TF32 apply
  bool aos_valid = false;
  bool aos_scaled = false;   // Aaos carries the Jacobi scale (block solve)
  double *phi = nullptr;     // [8][E] source weights (1/vol) int W_i
  bool want_phi = false, phi_valid = false;
  int *perm_d = nullptr;     // storage position -> caller element (colour mode)
  float *dinv32 = nullptr;
  int bk_K = 0;
  float *bk_f = nullptr;
  double *bk_d = nullptr;
  cudaGraphExec_t bk_graph = nullptr;
  bool bk_graph_split = false;
  bool block_tma = false;     // bulk-copy block apply
  bool block_tile = true;     // node-tile block apply on structured meshes (default)
  int blk_tc_mode = -1;       // K = 64 on the tile path: -1 by measurement, 0 node tile, 1 tcgen05
  int *block_err = nullptr;   // set when a bounded device wait ran out

  // many meshes as segments (batch.cu)
  std::vector<int> seg_off;  // node offsets, nseg + 1
  int seg_tile = 0, seg_threads = 256;  // autotuned tile shape (0: not yet)
  double *seg_d = nullptr;
  size_t seg_dwords = 0;
  int *seg_i = nullptr;
  size_t seg_iwords = 0;
  unsigned *seg_ticket = nullptr;
  int seg_ticket_n = 0;
  cudaGraphExec_t seg_graph = nullptr;
  const void *seg_key = nullptr;
  long seg_graph_launches = 0;
  int *seg_of_elem = nullptr;         // [E] storage order
  const int *gate_eseg = nullptr;     // apply gate while a segmented solve runs
  const int *gate_active = nullptr;

  // restarted GCR (gcr.cu)
  double *gcr_work = nullptr;
  size_t gcr_words = 0;
  cudaGraphExec_t gcr_graph = nullptr;
  const void *gcr_key = nullptr;
  long gcr_cycle_launches = 0;
};

// The connectivity view of the stored applies (structured when the mesh
// is in the canonical numbering, natural order and emask is built; the
// FP32-vector apply uses the structured form, the double-float ones the
// table).
ConnView conn_view(const Handle &h);
cudaError_t launch_emask(Handle &h);

// SM count of the current device, cached once (thread-safe).
int device_sm_count();

// Process-wide count of kernels launched by this library (graph nodes
// included), for the benchmark's launch accounting.
void count_launches(long n);
long long launches_so_far();
int apply_launches(const Handle &h);  // kernels per operator apply

OpArgs op_args(const Handle &h);

// Outputs of one element-build pass (any pointer may be null).
struct BuildArgs {
  double aH = 1.0, aM = 0.0;     // A_e = aH*H + aM*M
  double2 *A64 = nullptr;        // FP64 element-matrix store
  float4 *A32 = nullptr;         // FP32 element-matrix store
  float4 *Ahi = nullptr, *Alo = nullptr;  // double-float store
  int *bad = nullptr;            // set when an entry is outside FP32 range
  double *diag = nullptr;        // += diag(A_e)
  double cf = 1.0, rM = 0.0;     // b += cf*f - (H - rM*M) T_old
  const double *told = nullptr;
  double *b = nullptr;
  bool exact_fp64 = false;  // H/M rows accumulated in FP64, not double-float
  double *phi = nullptr;     // [8][E] (1/vol) int W_i dOmega, per element
  double *drs = nullptr;     // [5][E] per-element DR scalars (double-float build)
  // time loop: M kept as its own double-float store, and f = sum_e f_e
  float4 *Mhi = nullptr, *Mlo = nullptr;
  double *f = nullptr;
  // the mesh's geometric factors (element.cu, GeoFactors): given, the
  // double-float build reads them instead of recomputing the Jacobians
  const float2 *gJi = nullptr, *gDj = nullptr, *gK = nullptr;
  float2 *gsc = nullptr;  // [10][E] per-element scalars of that build, as pairs
};


// ---- launchers (element.cu) ----
cudaError_t launch_build(const OpArgs &a, const BuildArgs &ba, bool fp32,
                         cudaStream_t s);
// The mesh's geometric factors into g (arrays of E * 72, E * 8, E * 36
// pairs); sets bit 2 of *bad when a coordinate difference or detJ lies
// outside the pairs' safe window (the factors are then not to be used).
cudaError_t launch_geo_factors(const OpArgs &a, const GeoFactors &g, int *bad,
                               cudaStream_t s);
// The build's double-float beta of the VF variant on n host values.
cudaError_t diag_beta_vf(int n, const double *pe, double *beta);
cudaError_t launch_mf_apply(const OpArgs &a, bool fp32, bool transpose,
                            const double *x, double *y, const int *skip,
                            const int *skip2, cudaStream_t s);
cudaError_t launch_mass(Handle &h, const double *c, double *partials,
                        double *out, cudaStream_t s);

// ---- launchers (apply.cu) ----
cudaError_t launch_stored_apply(const Handle &h, bool fp32, bool transpose,
                                const double *x, double *y, const int *skip,
                                const int *skip2, cudaStream_t s);
// Time loop: b = cf F - (H - rM M) t from the stored A and M (t zero on
// Dirichlet nodes), as b = cf F - (A t)/aH + (aM/aH + rM) M t.
cudaError_t launch_rhs_from_mass(Handle &h, double cf, double rM, const double *t,
                                 double *b, cudaStream_t s);
// y1 += A x1 and y2 += A^T x2 in one pass (BiCG), when can_apply_both.
bool can_apply_both(const Handle &h);
cudaError_t launch_apply_both(const Handle &h, const double *x1, double *y1,
                              const double *x2, double *y2, const int *skip,
                              cudaStream_t s);
// Runs a one-warp mbarrier wait that nothing completes with a short budget:
// VDR_TIMEOUT when the bound tripped and was reported (block.cu).
int diag_wait_timeout(Handle &h);
// The same for the grid barrier of the fused inner kernels (krylov.cu).
int diag_barrier_timeout(Handle &h);
// The FP32 operator (A32v) on FP32 vectors, y += A x (stored mode only).
cudaError_t launch_stored_apply32v(const Handle &h, const float *x, float *y,
                                   const int *skip, const int *skip2,
                                   cudaStream_t s);
cudaError_t launch_apply(const Handle &h, bool transpose, const double *x,
                         double *y, const int *skip, const int *skip2,
                         cudaStream_t s);
cudaError_t launch_mask_conn(int *conn, int E, const unsigned char *mask,
                             cudaStream_t s);
cudaError_t launch_legacy_bb(const double *bb_ref, int E, double2 *A64,
                             cudaStream_t s);
// The stored element matrices in the reference's BB layout (FP64, caller's
// element order); the operator must be stored and valid.
cudaError_t launch_export_bb(const Handle &h, double *bb, cudaStream_t s);
// Reference BB -> double-float store; bit 2 of *bad when an entry is
// outside the store window (use launch_legacy_bb instead).
cudaError_t launch_legacy_bb_df(const double *bb_ref, int E, float4 *Ahi, float4 *Alo,
                                int *bad, cudaStream_t s);
cudaError_t launch_legacy_conn(const int *iss_ref, int E, int N, const int *bc,
                               int *conn, int *bad, cudaStream_t s);
// diag = 1 on Dirichlet nodes (when mask != null); dinv = 1/diag.
cudaError_t launch_diag_fix(double *diag, double *dinv,
                            const unsigned char *mask, int N, cudaStream_t s);
// Masks v and clears *all_zero when a nonzero entry remains.
cudaError_t launch_mask_vec_flag(double *v, const unsigned char *mask, int N,
                                 int *all_zero, cudaStream_t s);
cudaError_t launch_mask_vec(double *v, const unsigned char *mask, int N,
                            cudaStream_t s);
cudaError_t launch_bc_to_mask(const int *bc, unsigned char *mask, int N,
                              cudaStream_t s);

// ---- the 16-bit inner operator (half.cu) ----
// Builds A^ = P A P D^-1 in the binary16 store from the current FP64
// operator (hi parts of the double-float store, or the FP64 store) and the
// Jacobi diagonal; bit 0 of *bad when an element's scale leaves the range.
cudaError_t launch_half_store(Handle &h, int *bad, cudaStream_t s);
// y += A^ x on FP32 vectors (x, y of length N).
cudaError_t launch_apply_half(const Handle &h, const float *x, float *y,
                              const int *skip, const int *skip2, cudaStream_t s);

// ---- launch-shape tuning (tune.cu) ----
// Times the stored apply's grid candidates on the current operator and keeps
// the fastest in h.apply_per_sm (once per handle; not while the stream is
// being captured; meshes below 65,536 elements keep the default).
int tune_stored_apply(Handle &h);
// The same for the binary16 inner operator's apply (h.half_per_sm).
int tune_half_apply(Handle &h);
// The node-tile block apply's (box height, column halves) for K = 64, timed
// on X -> Y scratch columns of N x 64 floats (h.blk_ty, h.blk_halves).
int tune_block_apply(Handle &h, const float *X, float *Y, const float4 *Aaos);
// The tcgen05 box block apply (block_tc.cu): K = 64, Y += A X with boxes of
// 4 x 4 x 4 elements; needs the structured numbering, the error flag and
// the driver's tensor-map encoder.
bool block_tc_supported(const Handle &h);
int launch_block_tc(const Handle &h, bool split, const float *A, const float *X, float *Y,
                    const int *skip, const unsigned char *mask, cudaStream_t s);

// ---- solvers (krylov.cu) ----
int solve_device(Handle &h, int method, const double *b, double *x,
                 double tol, int itmax, int *iter, double *err,
                 const Precond *prec = nullptr, int stall_window = 0,
                 double *hist = nullptr, int max_hist = 0,
                 int *n_hist = nullptr);
// FP64 iterative refinement around an inner solve with the FP32 operator.
struct MixedStats {
  int outer = 0, inner = 0;
  double err = 0.0;
};
int solve_mixed_device(Handle &h, int method, const double *b, double *x,
                       double tol, double inner_tol, int max_outer,
                       int inner_itmax, MixedStats *ms);
cudaError_t ensure_solver_workspace(Handle &h, int nvec);

// Restarted GCR(m) with Jacobi and, if given, the preconditioner `prec`
// (gcr.cu).
int solve_gcr_device(Handle &h, const double *b, double *x, double tol,
                     int itmax, int m, const Precond *prec, int stall_window,
                     int *iter, double *err, double *hist = nullptr,
                     int max_hist = 0, int *n_hist = nullptr);

// Segments (independent meshes in one handle) and their batched solve
// (batch.cu).
int set_segments(Handle &h, int nseg, const int *node_off);
int solve_segmented_device(Handle &h, const double *b, double *x, double tol,
                           int itmax, int *iters, double *errs, int *statuses);

// Builds the element matrices and the Jacobi diagonal if stale (abi.cu).
int prepare_operator(Handle &h);
Handle &handle_of(vdr_handle *H);

// ---- many right-hand sides (block.cu) ----
int solve_block_device(Handle &h, int K, int precision, const double *B,
                       double *X, double tol, double inner_tol, int max_outer,
                       int inner_itmax, int *outer_iters, int *inner_iters,
                       double *errs_host);
cudaError_t launch_block_apply64(const Handle &h, int K, const double *X,
                                 double *Y, cudaStream_t s);
// x_clean: X is known to be zero on Dirichlet rows (the block solve's
// vectors), so the node-tile apply skips its mask reads.
int block_apply_launches_tf32(const Handle &h, int K, bool split,
                              const float *X, const float *dscale, float *Y,
                              const float4 *Aaos, const int *skip,
                              cudaStream_t s, bool x_clean = false);
cudaError_t launch_block_rhs(const Handle &h, const double *phi, int K,
                             const double *Q, double cf, double *B,
                             cudaStream_t s);
cudaError_t ensure_aos(Handle &h, bool scaled, float4 **out);

// ---- errors ----
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

}  // namespace vdr
