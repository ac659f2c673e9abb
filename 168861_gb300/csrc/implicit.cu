// Implicit (backward Euler) path: assembly + preconditioned GMRES(m), one persistent
// kernel per chunk of time steps.
//
// Replaces SolverImGPU::update / ::calculate (src/solverIm-gpu.cpp:687-843: Update_HH,
// Update_Mat, Update_B, then BiCGSTAB over cuSPARSE csrmv and cuBLAS dot/axpy with a
// host sync every 30 iterations) and computes the system of SolverImCPU::createMatrix
// (src/solverIm-cpu.cpp:29-183):
//
//   row j (physical):  -g_j V_mother + d_j V_j - g_DR V_DR - b_j g_DL V_DL = rhs_j
//   d_j   = c_j + b_j g_DL + [DR column] g_DR + [mother column] g_j,  c_j = c_m dX/dT - W dX
//   rhs_j = c_m dX V^n_j/dT + K dX + I_j,      g_x = 1/(r_a dX)_x
//
// with the reference's sealed ends: row 1 has no mother column, a row whose next element
// is a terminal has no DR column, and rows 0, N-1 and terminals are identity rows whose
// right-hand side is the stale second buffer -- so they keep their value from two steps
// back, exactly as the CPU reference leaves them.  The matrix is symmetric; it is stored
// as the diagonal plus the per-row conductance to the mother (the value of the (j,
// mother) and (mother, j) entries), which is the reference's CSR without the duplicated
// off-diagonals.  nrt_export_system expands it to the reference's CSR layout.
//
// Solver: right-preconditioned GMRES(m) (Saad), classical Gram-Schmidt, Givens
// rotations.  Each cycle starts from the true FP64 residual b - A x, so in mixed precision
// (FP32 basis, SpMV, orthogonalisation update and preconditioner) every restart is one
// step of iterative refinement.  Inner products and norms: per-thread partial sums in the
// basis precision over the thread's rows, then FP64 across threads and CTAs in a fixed
// order (deterministic, identical in every CTA).  Initial guess: V^n extrapolated
// linearly from V^{n-1}.  In mixed precision with the tree preconditioner a refinement
// cycle is one preconditioned Richardson step, x += M^-1 r (see implicit_one_step), with
// GMRES cycles taking over when a cycle lowers the true residual less than tenfold.
//
// Preconditioners: the exact tree factorisation (Hines order, see tree_factor), an exact
// tridiagonal solve of every unbranched segment piece, Jacobi, or none.
//
// Memory-level parallelism: every row loop keeps several rows per thread in flight and
// issues all of a row's independent loads before it uses any: a compact per-row flag
// byte replaces the topology record, the neighbours j-1 and j+1 are loaded speculatively
// (the mother is j-1 except on the first row of a DL child), and only the rare rows with
// a far neighbour make a second, dependent load.  The SpMV is fused with up to kG
// Gram-Schmidt products; the update and the norm share a pass.
//
// Two launch shapes from one template:
//  * kGrid  (one tree): a cooperative launch over the whole GPU; rows are split into
//    contiguous per-CTA ranges aligned with segment pieces; grid-wide syncs separate the
//    phases (two per Arnoldi step).
//  * block  (batches): a persistent block-per-instance scheduler; each CTA takes the next
//    instance (largest first) from an atomic queue and runs all of its steps with
//    __syncthreads only.
#include <cooperative_groups.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "hh.cuh"
#include "nrt_solver.h"
#include "pdl.cuh"
#include "record.cuh"
#include "tma.cuh"

namespace cg = cooperative_groups;

namespace nrt {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxPiece = 256;                 // longest segment piece one sweep handles
constexpr int kMaxDots = kMaxRestart + 1;
constexpr int kTileBytes = 44 * 1024;          // shared-memory staging for the sweeps
constexpr int kU = 4;                          // rows per thread in flight: SpMV + products
constexpr int kV = 4;                          // rows per thread in flight: streaming passes
constexpr int kA = 1;                          // rows per thread in flight: assembly
constexpr int kR = 2;                          // rows per thread in flight: FP64 residual
constexpr int kG = 8;                          // Gram-Schmidt products per pass over the rows

// Per-row flags of the implicit system (ImView::rowf).
enum : uint8_t {
  R_IDENT = 1,   // identity row
  R_UP = 2,      // column at the mother
  R_DOWNR = 4,   // column at DR == j + 1
  R_DOWNL = 8,   // column at DL
  R_FAR = 16,    // the mother is not j - 1 (first row of a DL child)
  R_HH = 32,     // Hodgkin_Huxley element
  R_INP = 64,    // nonzero injected current
};

struct InstStat {
  int64_t iters;
  int32_t last_iters;
  int32_t nonconv;
  double last_res;
  // passes over the rows (GMRES), for bandwidth accounting: FP64 residuals after the one
  // fused into the assembly, preconditioner applications, solution updates, basis
  // vectors read by the Arnoldi steps (sum of j + 1), and Richardson refinement steps
  int64_t residuals, applies, xupdates, basis, rich;
};

struct ImView {
  int64_t ntot;
  int m;             // GMRES restart (BiCGSTAB: sizes the shared work vectors only)
  int krylov;        // NRT_GMRES or NRT_BICGSTAB
  int scheme;        // NRT_BACKWARD_EULER or NRT_CRANK_NICOLSON
  int precond;
  int tol_mode;
  double tol;
  int max_iter;      // per step per instance; 0 -> instance size; < 0 -> assembly only
  double inner_rel;  // a refinement cycle's inner target relative to its starting residual
  int rich;          // refinement cycles start as preconditioned Richardson steps
  int ninst;
  int tile_rows;     // rows per shared-memory tile (segment preconditioner)
  const uint8_t *rowf;
  const double *cmdt;  // c_m dX / dT
  const double *g64;   // 1 / (r_a dX)
  const float *gf;
  const double *wdx64, *kdx64, *inp64;
  double *diag;
  double *rhs;
  void *Wb, *Z, *yv, *pcd, *pcc;  // T-typed workspace
  const int2 *pieces;             // (first row, length) of every segment piece
  const int *tiles;               // piece index where each tile starts (sentinel at end)
  const int *cta_row;             // kGrid: per-CTA row range [cta_row[c], cta_row[c+1])
  const int *cta_tile;            // kGrid: per-CTA tile range
  const int64_t *inst_row;        // per instance row range (ninst + 1)
  const int *inst_tile;           // per instance tile range (ninst + 1)
  const int *order;               // batch: instance processing order
  int *queue;                     // batch: next index into order
  double *partials;               // kGrid: 2 x gridDim x kMaxDots
  InstStat *stats;
  int *err;                       // set when a bounded wait gives up (device fault report)
  // exact tree preconditioner (NRT_PRECOND_TREE).  Segments in tile order; per-slot
  // arrays in slot order (slots: the rows of a worker's segments, level by level, deepest
  // level first; every tile starts on a multiple of 16 slots, padding slots have row -1).
  void *cdiag;                    // T[ntot]: c_j = c_m dX / dT - W dX, written by the assembly
  const int *seg_len, *seg_c1, *seg_c2, *seg_prow, *seg_soff;
  const int *tile_seg;            // segments of tree tile q: [tile_seg[q], tile_seg[q+1])
  const int *tile_slot;           // slots of tree tile q: [tile_slot[q], tile_slot[q+1])
  const int *srow;                // row behind each slot (-1: padding)
  const uint8_t *sflag;           // SL_* flags per slot
  const int *lev_tile;            // tree tiles of level entry e: [lev_tile[e], lev_tile[e+1])
  const int *work_lev;            // level entries of a worker (CTA or instance), deepest first
  const void *sg;                 // T per slot: conductance to the mother (0 without a column)
  void *sinv, *se, *sy;           // T per slot: 1 / pivot, g / pivot, eliminated right side
  void *exp_d, *exp_b;            // T per segment: what it passes to its parent row
  int tree_cap;                   // staging slots per tree tile (multiple of 16)
  int local_top;                  // one tree: levels 0 .. local_top all belong to CTA 0, which
                                  // passes between them with CTA barriers only (-1: none)
};

template <typename T>
struct Work {
  T *Wb, *Z, *y, *pd, *pc;
};

struct Shared {
  double *H, *cs, *sn, *g, *s, *y, *red, *warp;
  void *coef;      // T[kMaxDots]: update / solution coefficients
  int *flag;       // [0] convergence, [1] queue slot, [2] tile barrier phase
  uint64_t *bar;   // mbarrier of the tile bulk copies
  void *tile;      // staging area
};

__host__ __device__ inline size_t shared_fixed_bytes(int m) {
  return sizeof(double) * ((size_t)(m + 1) * m + 2 * m + 2 * (m + 1) + m + kMaxDots +
                           kWarps * kMaxDots + kMaxDots) + 32;
}

// The dynamic shared memory of the launch.
__device__ __forceinline__ double *dyn_smem() {
  extern __shared__ __align__(16) double nrt_dyn_smem[];
  return nrt_dyn_smem;
}

__device__ Shared carve(double *base, int m) {
  Shared S;
  S.H = base;
  S.cs = S.H + (m + 1) * m;
  S.sn = S.cs + m;
  S.g = S.sn + m;
  S.s = S.g + (m + 1);
  S.y = S.s + (m + 1);
  S.red = S.y + m;
  S.warp = S.red + kMaxDots;
  S.coef = (void *)(S.warp + kWarps * kMaxDots);
  S.flag = (int *)((double *)S.coef + kMaxDots);
  S.bar = (uint64_t *)(S.flag + 4);
  S.tile = (void *)((char *)base + ((shared_fixed_bytes(m) + 127) & ~(size_t)127));
  return S;
}

// ---------------------------------------------------------------- reductions

// Reduces the first k register accumulators of every thread over the CTA into out[0..k)
// (FP64, fixed order: warp shuffle tree, then warps in index order).
template <typename T, int kN>
__device__ __forceinline__ void block_reduce(const T (&acc)[kN], int k, double *warp_part,
                                             double *out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < kN; i++) {
    if (i < k) {
      double v = (double)acc[i];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) warp_part[w * kMaxDots + i] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < k) {
    double s = 0;
    for (int q = 0; q < kWarps; q++) s += warp_part[q * kMaxDots + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// Grid-wide completion: per-CTA sums -> global partials -> grid sync -> every CTA sums
// all CTAs' partials in the same order.
__device__ void grid_finish(cg::grid_group &grid, int k, double *cta_sums, double *partials,
                            int &parity) {
  double *buf = partials + (size_t)parity * gridDim.x * kMaxDots;
  parity ^= 1;
  if (threadIdx.x < k) buf[(size_t)blockIdx.x * kMaxDots + threadIdx.x] = cta_sums[threadIdx.x];
  __syncthreads();
  __threadfence();
  grid.sync();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = w; i < k; i += kWarps) {
    double v = 0;
    for (int c = lane; c < (int)gridDim.x; c += 32) v += buf[(size_t)c * kMaxDots + i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) cta_sums[i] = v;
  }
  __syncthreads();
}

// Sums k accumulators over the group into S.red[off .. off + k).
template <bool kGrid, typename T, int kN>
__device__ __forceinline__ void group_reduce(cg::grid_group &grid, const T (&acc)[kN], int k,
                                             Shared &S, double *partials, int &parity,
                                             int off = 0) {
  block_reduce(acc, k, S.warp, S.red + off);
  if (kGrid) grid_finish(grid, k, S.red + off, partials, parity);
}

template <bool kGrid>
__device__ __forceinline__ void group_sync(cg::grid_group &grid) {
  if (kGrid) {
    __threadfence();
    grid.sync();
  } else {
    __syncthreads();
  }
}

// ---------------------------------------------------------------- row kernels

// b_r - (A x)_r for the kN rows r = rb + u * stride (rows >= r1 give 0, flag R_IDENT), in
// FP64 as fused multiply-adds: b - d x first (one rounding for the two terms that nearly
// cancel), then + g x_q for each neighbour.  D / G: diagonal and conductance arrays, x the
// vector.  All independent loads of the kN rows are issued before any use.
template <int kN>
__device__ __forceinline__ void residual_rows(const PackView &pv, const ImView &iv,
                                              const double *__restrict__ B,
                                              const double *__restrict__ D,
                                              const double *__restrict__ G, const double *x,
                                              int64_t rb, int64_t stride, int64_t r1,
                                              double (&out)[kN], uint8_t (&fl)[kN]) {
  using C = double;
  using X = double;
  const int64_t N = pv.ntot;
  C dg[kN], gm[kN], gp[kN], bb[kN];
  X xs[kN], xm[kN], xp[kN];
#pragma unroll
  for (int u = 0; u < kN; u++) {
    const int64_t r = rb + u * stride;
    const bool ok = r < r1;
    const int64_t rm = r > 0 ? r - 1 : r, rp = r + 1 < N ? r + 1 : r;
    fl[u] = ok ? iv.rowf[r] : (uint8_t)R_IDENT;
    bb[u] = ok ? B[r] : (C)0;
    dg[u] = ok ? D[r] : (C)0;
    gm[u] = ok ? G[r] : (C)0;
    gp[u] = ok ? G[rp] : (C)0;
    xs[u] = ok ? x[r] : (X)0;
    xm[u] = ok ? x[rm] : (X)0;
    xp[u] = ok ? x[rp] : (X)0;
  }
#pragma unroll
  for (int u = 0; u < kN; u++) {
    const uint8_t f = fl[u];
    X s = 0;
    if (!(f & R_IDENT)) {
      X mo = xm[u], xl = 0;
      C gl = 0;
      if (f & (R_FAR | R_DOWNL)) {
        const Topo t = pv.topo[rb + u * stride];
        if (f & R_FAR) mo = x[t.mother];
        if (f & R_DOWNL) {
          gl = G[t.dl];
          xl = x[t.dl];
        }
      }
      s = fma(-dg[u], xs[u], bb[u]);
      if (f & R_UP) s = fma(gm[u], mo, s);
      if (f & R_DOWNR) s = fma(gp[u], xp[u], s);
      if (f & R_DOWNL) s = fma(gl, xl, s);
    }
    out[u] = s;
  }
}

// (A x)_r in the difference form c_r x_r + sum over the row's neighbours q of
// g_q (x_r - x_q): the same product as apply_rows (the diagonal is c_r plus the row's
// conductances), without its cancellation.  For the smooth vectors of a stiff cable,
// d_r x_r and g x_q are each ~g/c times larger than their difference, so the diagonal
// form loses that factor of precision in FP32; here each difference of neighbouring
// values is formed first (exactly, when they are within a factor of two).
template <int kN, typename C, typename X>
__device__ __forceinline__ void apply_rows_c(const PackView &pv, const ImView &iv,
                                             const C *__restrict__ Cc, const C *__restrict__ G,
                                             const X *x, int64_t rb, int64_t stride, int64_t r1,
                                             X (&out)[kN], uint8_t (&fl)[kN]) {
  const int64_t N = pv.ntot;
  C cc[kN], gm[kN], gp[kN];
  X xs[kN], xm[kN], xp[kN];
#pragma unroll
  for (int u = 0; u < kN; u++) {
    const int64_t r = rb + u * stride;
    const bool ok = r < r1;
    const int64_t rm = r > 0 ? r - 1 : r, rp = r + 1 < N ? r + 1 : r;
    fl[u] = ok ? iv.rowf[r] : (uint8_t)R_IDENT;
    cc[u] = ok ? Cc[r] : (C)0;
    gm[u] = ok ? G[r] : (C)0;
    gp[u] = ok ? G[rp] : (C)0;
    xs[u] = ok ? x[r] : (X)0;
    xm[u] = ok ? x[rm] : (X)0;
    xp[u] = ok ? x[rp] : (X)0;
  }
#pragma unroll
  for (int u = 0; u < kN; u++) {
    const uint8_t f = fl[u];
    X s = 0;
    if (!(f & R_IDENT)) {
      X mo = xm[u], xl = 0;
      C gl = 0;
      if (f & (R_FAR | R_DOWNL)) {
        const Topo t = pv.topo[rb + u * stride];
        if (f & R_FAR) mo = x[t.mother];
        if (f & R_DOWNL) {
          gl = G[t.dl];
          xl = x[t.dl];
        }
      }
      s = cc[u] * xs[u];
      if (f & R_UP) s += gm[u] * (xs[u] - mo);
      if (f & R_DOWNR) s += gp[u] * (xs[u] - xp[u]);
      if (f & R_DOWNL) s += gl * (xs[u] - xl);
    }
    out[u] = s;
  }
}

// ---------------------------------------------------------------- kernel context

template <typename T, bool kGrid>
struct Ctx {
  // device-memory copies of the launch's views: phases read the fields they need
  const PackView *pv;
  const ImView *iv;
  Work<T> w;
  int64_t r0, r1;   // rows of this CTA (kGrid) or instance (batch)
  int t0, t1;       // segment-preconditioner tiles
  int l0, l1;       // tree-preconditioner level entries (deepest first)
};

template <bool kGrid>
__device__ __forceinline__ void level_sync(cg::grid_group &grid) {
  if (kGrid) {
    __threadfence();
    grid.sync();
  }
}

// ---------------------------------------------------------------- tree preconditioner
//
// Exact factorisation of the tree matrix in Hines order (leaves to root), written for
// the input conductance eta of the subtree below each row: with d_k = g_k + eta_k (g_k
// the conductance to the mother, 0 on a row without that column),
//
//   eta_k = c_k + sum over children ch of g_ch eta_ch / (g_ch + eta_ch),
//
// which is d_k = D_k - sum g_ch^2 / d_ch rewritten without the cancellation between D_k
// and the children's terms (every term is positive), so the pivots keep full relative
// precision in FP32.  Per slot it stores inv_k = 1 / d_k and e_k = g_k / d_k; a segment
// passes e_first * eta_first (= g eta / (g + eta)) to its parent row.  Solve: elimination
// y_k = v_k + e_{k+1} y_{k+1} leaves to root, then x_k = inv_k y_k + e_k x_mother root to
// leaves.
//
// Work order: the segments of one level at a time (deepest first for the factorisation
// and the elimination), tile by tile through shared memory.  Inside a tile the
// recurrences along the segments run as segmented parallel scans over all the tile's
// slots, so a long unbranched cable costs a few scan rounds, not one thread walking it:
// the elimination and the substitution are first-order affine recurrences (maps
// y -> A + M y compose associatively), and the pivot recurrence is a Moebius map of eta,
// i.e. a product of 2x2 matrices acting on (p, q) with eta = p / q, normalised by powers
// of two as it goes.

enum : uint8_t { SL_FIRST = 1, SL_LAST = 2, SL_PAD = 4 };  // slot flags (ImView::sflag)

// bulk (TMA) copies, mbarriers and the bounded wait: tma.cuh

// Shared-memory tile of the tree preconditioner: three T rows, the slot flags and the
// slot rows, `cap` slots each.
template <typename T>
struct TreeTile {
  T *a, *b, *d;
  uint8_t *f;
  int *r;
};

template <typename T>
__device__ __forceinline__ TreeTile<T> tree_tile(const Shared &S, int cap) {
  TreeTile<T> t;
  t.a = (T *)S.tile;
  t.b = t.a + cap;
  t.d = t.b + cap;
  t.r = (int *)(t.d + cap);
  t.f = (uint8_t *)(t.r + cap);
  return t;
}

// Bulk-copies slots [s0, s0 + cnt) of the slot rows, the slot flags and up to three T
// arrays (null sources are skipped) into the tile, then waits for them.  s0 is a multiple
// of 16 slots and the slot arrays are padded, so every copy starts 16-byte aligned and
// its size rounded up to 16 bytes stays inside the arrays and the tile.
// Tile q_next (-1: none) is the one this CTA stages after this one: its arrays are
// prefetched into L2 while this tile is worked on.
template <typename T>
__device__ __forceinline__ void tile_bulk_load(const ImView &iv, const Shared &S,
                                               const TreeTile<T> &t, int s0, int cnt,
                                               const T *x0, T *d0, const T *x1, T *d1,
                                               const T *x2, T *d2, int q_next = -1) {
  const uint32_t nt = ((uint32_t)cnt * sizeof(T) + 15u) & ~15u;
  const uint32_t nr = ((uint32_t)cnt * 4u + 15u) & ~15u;
  const uint32_t nf = ((uint32_t)cnt + 15u) & ~15u;
  if (threadIdx.x == 0) {
    fence_proxy_async();
    const uint32_t total = nr + nf + (x0 ? nt : 0) + (x1 ? nt : 0) + (x2 ? nt : 0);
    mbar_expect_tx(S.bar, total);
    bulk_load(t.r, iv.srow + s0, nr, S.bar);
    bulk_load(t.f, iv.sflag + s0, nf, S.bar);
    if (x0) bulk_load(d0, x0 + s0, nt, S.bar);
    if (x1) bulk_load(d1, x1 + s0, nt, S.bar);
    if (x2) bulk_load(d2, x2 + s0, nt, S.bar);
    if (q_next >= 0) {
      const int s1 = iv.tile_slot[q_next], c1 = iv.tile_slot[q_next + 1] - s1;
      const uint32_t mt = ((uint32_t)c1 * sizeof(T) + 15u) & ~15u;
      prefetch_l2(iv.srow + s1, ((uint32_t)c1 * 4u + 15u) & ~15u);
      prefetch_l2(iv.sflag + s1, ((uint32_t)c1 + 15u) & ~15u);
      if (x0) prefetch_l2(x0 + s1, mt);
      if (x1) prefetch_l2(x1 + s1, mt);
      if (x2) prefetch_l2(x2 + s1, mt);
    }
  }
  const uint32_t ph = (uint32_t)S.flag[2];
  mbar_wait(S.bar, ph, iv.err);
  __syncthreads();
  if (threadIdx.x == 0) S.flag[2] = (int)(ph ^ 1u);
}

// dst[k] = src[row of slot k] for the slots of the tile (0 for padding slots).
template <typename T>
__device__ __forceinline__ void tile_gather(T *dst, const int *rows, const T *src, int cnt) {
  for (int k = threadIdx.x; k < cnt; k += 8 * blockDim.x) {
    T v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int kk = k + u * blockDim.x;
      const int r = kk < cnt ? rows[kk] : -1;
      v[u] = r >= 0 ? src[r] : (T)0;
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int kk = k + u * blockDim.x;
      if (kk < cnt) dst[kk] = v[u];
    }
  }
}

// dst[s0 + k] = src[k] for the tile's slots.
template <typename T>
__device__ __forceinline__ void store_contig(T *dst, const T *src, int s0, int count) {
  for (int k = threadIdx.x; k < count; k += blockDim.x) dst[s0 + k] = src[k];
}

// dst[row of slot k] = src[k] for the real slots of the tile.
template <typename T>
__device__ __forceinline__ void tile_scatter(T *dst, const int *rows, const T *src, int cnt) {
  for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
    const int r = rows[k];
    if (r >= 0) dst[r] = src[k];
  }
}

// The contiguous run of slots thread t owns in a tile scan.  The run length is odd, so
// the threads of a warp touch distinct shared-memory banks.
__device__ __forceinline__ void scan_run(int cnt, int &k0, int &k1) {
  const int R = ((cnt + (int)blockDim.x - 1) / (int)blockDim.x) | 1;
  k0 = min(cnt, (int)threadIdx.x * R);
  k1 = min(cnt, k0 + R);
}

// Segmented first-order recurrence over a tile's slots, in place in a[]:
//   kDesc:  y_k = a_k + m_k y_{k+1}, k = cnt-1 .. 0 (nothing enters the top)
//   !kDesc: y_k = a_k + m_k y_{k-1}, k = 0 .. cnt-1
// with m_k = link(k) (0 where a segment starts in scan order).  Each thread composes the
// maps of its run, a warp shuffle scan and one pass over the warps give every run its
// entering value, and the run is then evaluated.  scratch: 3 * warps T values.
// Links of the two solve recurrences: elimination (descending) uses e_{k+1} unless slot k
// ends its segment; substitution (ascending) uses e_k unless slot k starts one.
template <typename T, bool kDesc>
struct SlotLink {
  const T *e;
  const uint8_t *f;
  __device__ __forceinline__ T operator()(int k) const {
    if (kDesc) return (f[k] & SL_LAST) ? (T)0 : e[k + 1];
    return (f[k] & SL_FIRST) ? (T)0 : e[k];
  }
};

template <typename T, bool kDesc>
__device__ __noinline__ void tile_affine_scan(T *a, int cnt, SlotLink<T, kDesc> link, T *scratch) {
  int k0, k1;
  scan_run(cnt, k0, k1);
  T A = 0, M = 1;  // the run's map y_in -> A + M y_in
  if (kDesc) {
    for (int k = k1 - 1; k >= k0; k--) {
      const T m = link(k);
      A = a[k] + m * A;
      M = m * M;
    }
  } else {
    for (int k = k0; k < k1; k++) {
      const T m = link(k);
      A = a[k] + m * A;
      M = m * M;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int sl = kDesc ? 31 - lane : lane;  // position in scan order inside the warp
  T iA = A, iM = M;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int src = (kDesc ? lane + off : lane - off) & 31;
    const T pA = __shfl_sync(0xffffffffu, iA, src), pM = __shfl_sync(0xffffffffu, iM, src);
    if (sl >= off) {  // (this part) after (the earlier part)
      iA = iA + iM * pA;
      iM = iM * pM;
    }
  }
  const int prv = (kDesc ? lane + 1 : lane - 1) & 31;
  T eA = __shfl_sync(0xffffffffu, iA, prv), eM = __shfl_sync(0xffffffffu, iM, prv);
  if (sl == 0) {
    eA = 0;
    eM = 1;
  }
  if (sl == 31) {
    scratch[2 * w] = iA;
    scratch[2 * w + 1] = iM;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    T y = 0;
    for (int q = 0; q < nw; q++) {
      const int ww = kDesc ? nw - 1 - q : q;
      scratch[2 * nw + ww] = y;
      y = scratch[2 * ww] + scratch[2 * ww + 1] * y;
    }
  }
  __syncthreads();
  T y = eA + eM * scratch[2 * nw + w];
  if (kDesc) {
    for (int k = k1 - 1; k >= k0; k--) {
      y = a[k] + link(k) * y;
      a[k] = y;
    }
  } else {
    for (int k = k0; k < k1; k++) {
      y = a[k] + link(k) * y;
      a[k] = y;
    }
  }
  __syncthreads();
}

// 2x2 matrices and vectors of the pivot recurrence, scaled by powers of two.
template <typename T>
struct Mob {
  T a, b, c, d;  // [[a, b], [c, d]]
};

template <typename T>
__device__ __forceinline__ T pow2_scale_of(T m) {
  int e;
  frexp(m, &e);
  return ldexp((T)1, -e);
}

template <typename T>
__device__ __forceinline__ Mob<T> mob_mul(const Mob<T> &x, const Mob<T> &y) {  // x * y
  Mob<T> r{x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c,
           x.c * y.b + x.d * y.d};
  const T m = fmax(fmax(r.a, r.b), fmax(r.c, r.d));  // entries are non-negative
  if (m > (T)0) {
    const T s = pow2_scale_of(m);
    r.a *= s;
    r.b *= s;
    r.c *= s;
    r.d *= s;
  }
  return r;
}

// Per-slot map of the pivot recurrence.  The vector entering slot k is (a, b) with
// a / b = g_{k+1} eta_{k+1} / (g_{k+1} + eta_{k+1}) when slot k+1 continues the segment;
// the slot forms (p, q) = (a + c b, b) (or (c b, b) at a segment's last slot, where c
// already holds the children's terms), eta_k = p / q, and passes (g p, p + g q) on.
template <typename T>
__device__ __forceinline__ Mob<T> slot_map(T c, T g, uint8_t f) {
  if (f & SL_PAD) return Mob<T>{1, 0, 0, 1};
  if (f & SL_LAST) return Mob<T>{0, g * c, 0, c + g};
  return Mob<T>{g, g * c, 1, c + g};
}

// One tile of the factorisation: sc = c (in) -> 1/pivot, sg = g -> e = g / pivot,
// sh -> e * eta; scratch: 12 * warps T values.
template <typename T>
__device__ __noinline__ void tile_factor_scan(T *sc, T *sg, T *sh, const uint8_t *sf, int cnt,
                                              T *scratch) {
  int k0, k1;
  scan_run(cnt, k0, k1);
  Mob<T> P{1, 0, 0, 1};  // the run's map, scan order = descending slots
  for (int k = k1 - 1; k >= k0; k--) P = mob_mul(slot_map(sc[k], sg[k], sf[k]), P);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int sl = 31 - lane;
  Mob<T> I = P;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int src = (lane + off) & 31;
    Mob<T> Q{__shfl_sync(0xffffffffu, I.a, src), __shfl_sync(0xffffffffu, I.b, src),
             __shfl_sync(0xffffffffu, I.c, src), __shfl_sync(0xffffffffu, I.d, src)};
    if (sl >= off) I = mob_mul(I, Q);
  }
  const int prv = (lane + 1) & 31;
  Mob<T> E{__shfl_sync(0xffffffffu, I.a, prv), __shfl_sync(0xffffffffu, I.b, prv),
           __shfl_sync(0xffffffffu, I.c, prv), __shfl_sync(0xffffffffu, I.d, prv)};
  if (sl == 0) E = Mob<T>{1, 0, 0, 1};
  if (sl == 31) {
    scratch[4 * w] = I.a;
    scratch[4 * w + 1] = I.b;
    scratch[4 * w + 2] = I.c;
    scratch[4 * w + 3] = I.d;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // vector entering each warp; (0, 1) enters the tile's top slot
    T va = 0, vb = 1;
    for (int q = nw - 1; q >= 0; q--) {
      scratch[4 * nw + 2 * q] = va;
      scratch[4 * nw + 2 * q + 1] = vb;
      const T na = scratch[4 * q] * va + scratch[4 * q + 1] * vb;
      const T nb = scratch[4 * q + 2] * va + scratch[4 * q + 3] * vb;
      const T s = pow2_scale_of(fmax(na, nb));
      va = na * s;
      vb = nb * s;
    }
  }
  __syncthreads();
  T va = scratch[4 * nw + 2 * w], vb = scratch[4 * nw + 2 * w + 1];
  {
    const T na = E.a * va + E.b * vb, nb = E.c * va + E.d * vb;
    const T s = pow2_scale_of(fmax(na, nb));
    va = na * s;
    vb = nb * s;
  }
  for (int k = k1 - 1; k >= k0; k--) {
    const uint8_t f = sf[k];
    const T c = sc[k], g = sg[k];
    if (f & SL_PAD) {
      sc[k] = 0;
      sg[k] = 0;
      sh[k] = 0;
      continue;
    }
    const T p = (f & SL_LAST) ? c * vb : va + c * vb;
    const T eta = p / vb;
    const T inv = (T)1 / (g + eta);
    const T e = g * inv;
    sc[k] = inv;
    sg[k] = e;
    sh[k] = e * eta;
    const T na = g * p, nb = p + g * vb;
    const T s = pow2_scale_of(fmax(na, nb));
    va = na * s;
    vb = nb * s;
  }
  __syncthreads();
}

template <typename T, bool kGrid>
__device__ __noinline__ void tree_factor(Ctx<T, kGrid> c) {
  const ImView &iv = *c.iv;
  cg::grid_group grid = cg::this_grid();
  Shared S = carve(dyn_smem(), iv.m);
  const TreeTile<T> t = tree_tile<T>(S, iv.tree_cap);
  T *scratch = (T *)S.warp;
  T *exp_d = (T *)iv.exp_d;
  for (int e = c.l0; e < c.l1; e++) {
    for (int q = iv.lev_tile[e]; q < iv.lev_tile[e + 1]; q++) {
      const int s0 = iv.tile_slot[q], cnt = iv.tile_slot[q + 1] - s0;
      const int qn = q + 1 < iv.lev_tile[c.l1] ? q + 1 : -1;
      tile_bulk_load<T>(iv, S, t, s0, cnt, (const T *)iv.sg, t.b, nullptr, nullptr, nullptr,
                        nullptr, qn);
      tile_gather(t.a, t.r, (const T *)iv.cdiag, cnt);  // c of every slot's row
      __syncthreads();
      for (int s = iv.tile_seg[q] + threadIdx.x; s < iv.tile_seg[q + 1]; s += blockDim.x) {
        const int last = iv.seg_soff[s] + iv.seg_len[s] - 1;
        const int c1 = iv.seg_c1[s], c2 = iv.seg_c2[s];
        T add = 0;
        if (c1 >= 0) add += exp_d[c1];
        if (c2 >= 0) add += exp_d[c2];
        t.a[last] += add;
      }
      __syncthreads();
      tile_factor_scan(t.a, t.b, t.d, t.f, cnt, scratch);
      for (int s = iv.tile_seg[q] + threadIdx.x; s < iv.tile_seg[q + 1]; s += blockDim.x)
        exp_d[s] = t.d[iv.seg_soff[s]];  // 0 when the first row has no mother column
      store_contig((T *)iv.sinv, t.a, s0, cnt);
      store_contig((T *)iv.se, t.b, s0, cnt);
      fence_proxy_async();  // the solves read sinv / se back with bulk copies
      __syncthreads();
    }
    // entry e is level c.l1 - 1 - e; the next (shallower) one is CTA 0's alone when this
    // one is (every CTA evaluates the same test, so all take the same grid syncs)
    if (c.l1 - 1 - e > iv.local_top) level_sync<kGrid>(grid);
  }
}

// z = A^-1 v (up to rounding) with the factors of tree_factor.
template <typename T, bool kGrid>
__device__ __noinline__ void tree_apply(Ctx<T, kGrid> c, const T *v, T *z) {
  const ImView &iv = *c.iv;
  cg::grid_group grid = cg::this_grid();
  Shared S = carve(dyn_smem(), iv.m);
  const TreeTile<T> t = tree_tile<T>(S, iv.tree_cap);
  T *scratch = (T *)S.warp;
  T *exp_b = (T *)iv.exp_b;
  // elimination, deepest level first: y_k = v_k + e_{k+1} y_{k+1} inside a segment
  for (int e = c.l0; e < c.l1; e++) {
    for (int q = iv.lev_tile[e]; q < iv.lev_tile[e + 1]; q++) {
      const int s0 = iv.tile_slot[q], cnt = iv.tile_slot[q + 1] - s0;
      const int qn = q + 1 < iv.lev_tile[c.l1] ? q + 1 : -1;
      tile_bulk_load<T>(iv, S, t, s0, cnt, (const T *)iv.se, t.b, nullptr, nullptr, nullptr,
                        nullptr, qn);
      tile_gather(t.a, t.r, v, cnt);
      __syncthreads();
      for (int s = iv.tile_seg[q] + threadIdx.x; s < iv.tile_seg[q + 1]; s += blockDim.x) {
        const int last = iv.seg_soff[s] + iv.seg_len[s] - 1;
        const int c1 = iv.seg_c1[s], c2 = iv.seg_c2[s];
        T add = 0;
        if (c1 >= 0) add += exp_b[c1];
        if (c2 >= 0) add += exp_b[c2];
        t.a[last] += add;
      }
      __syncthreads();
      tile_affine_scan<T, true>(t.a, cnt, SlotLink<T, true>{t.b, t.f}, scratch);
      for (int s = iv.tile_seg[q] + threadIdx.x; s < iv.tile_seg[q + 1]; s += blockDim.x) {
        const int o = iv.seg_soff[s];
        exp_b[s] = t.b[o] * t.a[o];
      }
      store_contig((T *)iv.sy, t.a, s0, cnt);
      fence_proxy_async();  // the substitution reads sy back with bulk copies
      __syncthreads();
    }
    // as in tree_factor; after level 0 the substitution starts at level 0, in CTA 0
    if (c.l1 - 1 - e > iv.local_top) level_sync<kGrid>(grid);
  }
  // substitution, root level first: x_k = inv_k y_k + e_k x_{k-1} (x_mother on a first row)
  for (int e = c.l1 - 1; e >= c.l0; e--) {
    for (int q = iv.lev_tile[e]; q < iv.lev_tile[e + 1]; q++) {
      const int s0 = iv.tile_slot[q], cnt = iv.tile_slot[q + 1] - s0;
      // next: the following tile of this level, else the first tile of the level above
      const int qn = q + 1 < iv.lev_tile[e + 1] ? q + 1
                                                : (e > c.l0 ? iv.lev_tile[e - 1] : -1);
      tile_bulk_load<T>(iv, S, t, s0, cnt, (const T *)iv.sy, t.a, (const T *)iv.se, t.b,
                        (const T *)iv.sinv, t.d, qn);
      for (int k = threadIdx.x; k < cnt; k += blockDim.x) t.a[k] *= t.d[k];
      __syncthreads();
      for (int s = iv.tile_seg[q] + threadIdx.x; s < iv.tile_seg[q + 1]; s += blockDim.x) {
        const int pr = iv.seg_prow[s];
        if (pr >= 0) {
          const int o = iv.seg_soff[s];
          t.a[o] += t.b[o] * z[pr];
        }
      }
      __syncthreads();
      tile_affine_scan<T, false>(t.a, cnt, SlotLink<T, false>{t.b, t.f}, scratch);
      tile_scatter(z, t.r, t.a, cnt);
      __syncthreads();
    }
    // the next (deeper) level is CTA 0's alone when it is within the top levels
    if (c.l1 - 1 - e >= iv.local_top) level_sync<kGrid>(grid);
  }
}

// ---------------------------------------------------------------- segment preconditioner

// Rows covered by tile q: from its first piece's start to its last piece's end.
__device__ __forceinline__ void tile_rows(const ImView &iv, int q, int64_t &a, int64_t &b) {
  const int pa = iv.tiles[q], pb = iv.tiles[q + 1];
  a = iv.pieces[pa].x;
  const int2 last = iv.pieces[pb - 1];
  b = (int64_t)last.x + last.y;
}

// Thomas factorisation of every piece (once per step): pd = 1/pivot, pc = c'.
// Staged through shared memory tile by tile; one thread per piece.
template <typename T, bool kGrid>
__device__ __noinline__ void factor_pieces(Ctx<T, kGrid> c) {
  Shared S = carve(dyn_smem(), c.iv->m);
  T *sd = (T *)S.tile;                          // diag, then pivots^-1
  T *sg = sd + c.iv->tile_rows;                  // conductance to the mother
  T *sc = sg + c.iv->tile_rows;                  // c'
  for (int q = c.t0; q < c.t1; q++) {
    int64_t a, b;
    tile_rows(*c.iv, q, a, b);
    for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
      sd[r - a] = (T)c.iv->diag[r];
      sg[r - a] = (T)c.iv->g64[r];
    }
    __syncthreads();
    for (int p = c.iv->tiles[q] + threadIdx.x; p < c.iv->tiles[q + 1]; p += blockDim.x) {
      const int2 pc = c.iv->pieces[p];
      const int o = (int)(pc.x - a);
      double cprev = 0;
      for (int k = 0; k < pc.y; k++) {
        const double sub = k ? -(double)sg[o + k] : 0.0;                  // (j, j-1)
        const double sup = k + 1 < pc.y ? -(double)sg[o + k + 1] : 0.0;   // (j, j+1)
        const double d = 1.0 / ((double)sd[o + k] - sub * cprev);
        cprev = sup * d;
        sd[o + k] = (T)d;
        sc[o + k] = (T)cprev;
      }
    }
    __syncthreads();
    for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
      c.w.pd[r] = sd[r - a];
      c.w.pc[r] = sc[r - a];
    }
    __syncthreads();
  }
}

// z = M^-1 v over this CTA's rows (identity rows: v and z are 0).
template <typename T, bool kGrid>
__device__ __noinline__ void apply_precond(Ctx<T, kGrid> c, const T *v, T *z) {
  cg::grid_group grid = cg::this_grid();
  Shared S = carve(dyn_smem(), c.iv->m);
  if (c.iv->precond == NRT_PRECOND_TREE) {
    level_sync<kGrid>(grid);  // v of every row visible (tree tiles span other CTAs' rows)
    tree_apply(c, v, z);
  } else if (c.iv->precond == NRT_PRECOND_SEGMENT) {
    T *sv = (T *)S.tile;
    T *sd = sv + c.iv->tile_rows;
    T *sc = sd + c.iv->tile_rows;
    T *sg = sc + c.iv->tile_rows;
    for (int q = c.t0; q < c.t1; q++) {
      int64_t a, b;
      tile_rows(*c.iv, q, a, b);
      for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
        sv[r - a] = v[r];
        sd[r - a] = c.w.pd[r];
        sc[r - a] = c.w.pc[r];
        sg[r - a] = (T)c.iv->g64[r];
      }
      __syncthreads();
      for (int p = c.iv->tiles[q] + threadIdx.x; p < c.iv->tiles[q + 1]; p += blockDim.x) {
        const int2 pc = c.iv->pieces[p];
        const int o = (int)(pc.x - a);
        T y = sv[o] * sd[o];
        sv[o] = y;
        for (int k = 1; k < pc.y; k++) {  // forward: y_k = (v_k + g_k y_{k-1}) d_k
          y = (sv[o + k] + sg[o + k] * y) * sd[o + k];
          sv[o + k] = y;
        }
        for (int k = pc.y - 2; k >= 0; k--) {  // backward: z_k = y_k - c'_k z_{k+1}
          y = sv[o + k] - sc[o + k] * y;
          sv[o + k] = y;
        }
      }
      __syncthreads();
      for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) z[r] = sv[r - a];
      __syncthreads();
    }
  } else {
    for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x) {
      const uint8_t f = c.iv->rowf[j];
      if (f & R_IDENT) {
        z[j] = 0;
        continue;
      }
      z[j] = c.iv->precond == NRT_PRECOND_JACOBI ? (T)((double)v[j] / c.iv->diag[j]) : v[j];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- one step
//
// The row passes below are separate (not inlined) functions: each keeps its own rows in
// flight in registers, and none of them has to share the register file with the state
// of the others.

template <typename T>
struct DotAcc {
  T v[kG];
};

// The initial guess of a step: V^n extrapolated from V^{n-1} (which Vout holds until the
// first solution update writes it).
__device__ __forceinline__ double x0_of(const double *Vin, const double *Vout, int64_t j) {
  return 2.0 * Vin[j] - Vout[j];
}

// Assembly: gates (from V^n), W, K, diagonal, c and right-hand side, fused with the first
// true residual r = b - A x0 (into W_0).  Nothing writes V here, so the neighbours' x0 are
// formed from V^n and V^{n-1} directly (a row's columns are never identity rows).  Returns
// the thread's parts of ||b||^2 and ||r||^2.
template <typename T, bool kGrid>
__device__ __noinline__ double2 ph_assemble(Ctx<T, kGrid> c, const double *Vin,
                                            const double *Vout, int active, int inst) {
  const PackView &pv = *c.pv;
  const ImView &iv = *c.iv;
  const int64_t N = pv.ntot, stride = blockDim.x;
  T *cdiag = (T *)iv.cdiag;
  // ||b|| needs a few digits only and its terms are far from FP32's range limits: it
  // accumulates in T.  Residual entries near convergence are tiny (their squares leave
  // FP32's normal range), so ||r|| stays in FP64.
  T bacc = 0;
  double racc = 0;
  // gates of this precision (the mixed path keeps them in FP32)
  T *gate = sizeof(T) == 4 ? (T *)(void *)pv.gatef : (T *)(void *)pv.gate;
  const bool cn = iv.scheme == NRT_CRANK_NICOLSON;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kA * stride) {
    uint8_t f[kA];
    double v[kA], vo[kA], cm[kA], gj[kA], gn[kA], inp[kA], xm[kA], xp[kA], vm[kA], vp[kA];
    int64_t hc[kA];
    T g0[kA], g1[kA], g2[kA];
    // every load that does not depend on the row's flags goes out in this first round
#pragma unroll
    for (int u = 0; u < kA; u++) {
      const int64_t r = rb + u * stride;
      const bool ok = r < c.r1;
      const int64_t rp = r + 1 < N ? r + 1 : r, rm = r > 0 ? r - 1 : r;
      hc[u] = ok && pv.hp_cls ? (int64_t)pv.hp_cls[r] : (pv.hp_inst ? (int64_t)inst : r);
      const bool gl = ok && pv.hh_dense;
      g0[u] = gl ? gate[r] : (T)0;
      g1[u] = gl ? gate[N + r] : (T)0;
      g2[u] = gl ? gate[2 * N + r] : (T)0;
      f[u] = ok ? iv.rowf[r] : (uint8_t)R_IDENT;
      v[u] = ok ? Vin[r] : 0.0;
      vo[u] = ok ? Vout[r] : 0.0;
      cm[u] = ok ? iv.cmdt[r] : 0.0;
      gj[u] = ok ? iv.g64[r] : 0.0;
      gn[u] = ok ? iv.g64[rp] : 0.0;
      inp[u] = 0.0;
      xm[u] = ok ? x0_of(Vin, Vout, rm) : 0.0;
      xp[u] = ok ? x0_of(Vin, Vout, rp) : 0.0;
      vm[u] = ok && cn ? Vin[rm] : 0.0;  // Crank-Nicolson: V^n of the neighbours
      vp[u] = ok && cn ? Vin[rp] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kA; u++) {
      const int64_t r = rb + u * stride;
      if (r >= c.r1) continue;
      double wdx, kdx;
      if (f[u] & R_HH) {
        const int64_t L = pv.hp_ld;
        if (!pv.hh_dense) {
          g0[u] = gate[r];
          g1[u] = gate[N + r];
          g2[u] = gate[2 * N + r];
        }
        if (sizeof(T) == 4) {
          const HHParams32 q = hh_params32(pv.hpq, hc[u]);
          const float dv = (float)(v[u] - (double)q.v[HP_REST]);
          GateStep32 g = hh_step32(dv + q.v[HP_LSNA], dv + q.v[HP_LSK], (float)g0[u],
                                   (float)g1[u], (float)g2[u], q.v[HP_DTMS], q.v[HP_GNA],
                                   q.v[HP_GK], q.v[HP_GL], q.v[HP_ENA], q.v[HP_EK], q.v[HP_EL]);
          gate[r] = (T)g.m;
          gate[N + r] = (T)g.h;
          gate[2 * N + r] = (T)g.n;
          const float dx = q.v[HP_DX];
          wdx = (double)(g.W * dx);  // FP32 inputs: the product in FP32 loses nothing
          kdx = (double)(g.K * dx);
        } else {
          const double *hp = pv.hp + hc[u];
          GateStep64 g = hh_step64(v[u], (double)g0[u], (double)g1[u], (double)g2[u],
                                   hp[HP_LSNA * L], hp[HP_LSK * L], hp[HP_REST * L],
                                   hp[HP_DTMS * L], hp[HP_GNA * L], hp[HP_GK * L],
                                   hp[HP_GL * L], hp[HP_ENA * L], hp[HP_EK * L],
                                   hp[HP_EL * L]);
          gate[r] = (T)g.m;
          gate[N + r] = (T)g.h;
          gate[2 * N + r] = (T)g.n;
          const double dx = hp[HP_DX * L];
          wdx = g.W * dx;
          kdx = g.K * dx;
        }
      } else {
        wdx = iv.wdx64[r];
        kdx = iv.kdx64[r];
      }
      if (f[u] & R_IDENT) {
        c.w.y[r] = 0;
        c.w.Wb[r] = 0;
        continue;
      }
      // backward Euler: c = c_m dX/dT - W dX; Crank-Nicolson (doubled): 2 c_m dX/dT - W dX
      const double cj = (cn ? 2.0 * cm[u] : cm[u]) - wdx;
      double d = cj, gl = 0.0, xl = 0.0, xmo = xm[u], vmo = vm[u], vl = 0.0;
      if (f[u] & (R_DOWNL | R_FAR)) {
        const Topo t = pv.topo[r];
        if (f[u] & R_DOWNL) {
          gl = iv.g64[t.dl];
          xl = x0_of(Vin, Vout, t.dl);
          if (cn) vl = Vin[t.dl];
          d += gl;
        }
        if (f[u] & R_FAR) {
          xmo = x0_of(Vin, Vout, t.mother);
          if (cn) vmo = Vin[t.mother];
        }
      }
      if (f[u] & R_DOWNR) d += gn[u];
      if (f[u] & R_UP) d += gj[u];
      iv.diag[r] = d;
      cdiag[r] = (T)cj;
      if (active && (f[u] & R_INP)) inp[u] = iv.inp64[r];  // one row or a few per tree
      double b;
      if (!cn) {
        b = cm[u] * v[u] + kdx;
        if (active && (f[u] & R_INP)) b += inp[u];  // other rows would add an exact 0
      } else {  // (2 c_m dX/dT + W dX) V^n - sum g (V^n - V^n_q) + 2 (K dX + I)
        b = (2.0 * cm[u] + wdx) * v[u];
        if (f[u] & R_UP) b -= gj[u] * (v[u] - vmo);
        if (f[u] & R_DOWNR) b -= gn[u] * (v[u] - vp[u]);
        if (f[u] & R_DOWNL) b -= gl * (v[u] - vl);
        b += 2.0 * kdx;
        if (active && (f[u] & R_INP)) b += 2.0 * inp[u];
      }
      iv.rhs[r] = b;
      bacc += (T)b * (T)b;
      // r = b - A x0 as residual_rows forms it: b - d x0, then mother, DR, DL
      double rr = fma(-d, 2.0 * v[u] - vo[u], b);
      if (f[u] & R_UP) rr = fma(gj[u], xmo, rr);
      if (f[u] & R_DOWNR) rr = fma(gn[u], xp[u], rr);
      if (f[u] & R_DOWNL) rr = fma(gl, xl, rr);
      c.w.Wb[r] = (T)rr;
      racc += rr * rr;
    }
  }
  return make_double2((double)bacc, racc);
}

// Vout = x0 for the rows of this group (when a step ends before any solution update).
template <typename T, bool kGrid>
__device__ __noinline__ void ph_x0(Ctx<T, kGrid> c, const double *Vin, double *Vout) {
  const uint8_t *rowf = c.iv->rowf;
  for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x)
    if (!(rowf[j] & R_IDENT)) Vout[j] = x0_of(Vin, Vout, j);
}

// True residual r = b - A x in FP64 into W_0 (identity rows 0); returns the thread's
// part of ||r||^2, or with scale > 0 of ||scale r||^2 summed in FP32.  That form is for
// the mixed GMRES and Richardson cycles, where the norm only decides convergence and scales
// an FP32 basis: it keeps the sum off the FP64 pipe, and the caller passes a power of two
// near 1 / (the previous residual norm), which keeps the entries in FP32's range.  FP64
// solves and BiCGSTAB (whose rho_0 is this norm squared) take the FP64 sum.
template <typename T, bool kGrid>
__device__ __noinline__ double ph_residual(Ctx<T, kGrid> c, const double *x, float scale) {
  const PackView &pv = *c.pv;
  const ImView &iv = *c.iv;
  const int64_t stride = blockDim.x;
  float acc = 0;
  double acc64 = 0;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kR * stride) {
    double rr[kR];
    uint8_t fl[kR];
    residual_rows<kR>(pv, iv, iv.rhs, iv.diag, iv.g64, x, rb, stride, c.r1, rr, fl);
#pragma unroll
    for (int u = 0; u < kR; u++) {
      const int64_t r = rb + u * stride;
      if (r >= c.r1) continue;
      if (fl[u] & R_IDENT) {
        c.w.Wb[r] = 0;
        continue;
      }
      c.w.Wb[r] = (T)rr[u];
      if (scale > 0) {
        const float e = (float)rr[u] * scale;
        acc = fmaf(e, e, acc);
      } else {
        acc64 += rr[u] * rr[u];
      }
    }
  }
  return scale > 0 ? (double)acc : acc64;
}

// y = s_j A Z_j, fused with the thread's parts of <y, W_i> for i < g1.
template <typename T, bool kGrid>
__device__ __noinline__ DotAcc<T> ph_spmv(Ctx<T, kGrid> c, int j, T sj, int g1) {
  const PackView &pv = *c.pv;
  const ImView &iv = *c.iv;
  const int64_t N = pv.ntot, stride = blockDim.x;
  const T *CT = (const T *)iv.cdiag;
  const T *GT = sizeof(T) == 4 ? (const T *)(const void *)iv.gf : (const T *)(const void *)iv.g64;
  const T *Zj = c.w.Z + (size_t)j * N;
  DotAcc<T> acc;
#pragma unroll
  for (int i = 0; i < kG; i++) acc.v[i] = 0;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kU * stride) {
    T y[kU];
    uint8_t fl[kU];
    apply_rows_c<kU>(pv, iv, CT, GT, Zj, rb, stride, c.r1, y, fl);
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int64_t r = rb + u * stride;
      y[u] *= sj;
      if (r < c.r1) c.w.y[r] = y[u];
    }
#pragma unroll
    for (int i = 0; i < kG; i++) {
      if (i < g1) {
        const T *Wi = c.w.Wb + (size_t)i * N;
#pragma unroll
        for (int u = 0; u < kU; u++) {
          const int64_t r = rb + u * stride;
          if (r < c.r1) acc.v[i] += y[u] * Wi[r];
        }
      }
    }
  }
  return acc;
}

// The thread's parts of <y, W_{i0+i}> for i < gk.
template <typename T, bool kGrid>
__device__ __noinline__ DotAcc<T> ph_products(Ctx<T, kGrid> c, int i0, int gk) {
  const int64_t N = c.pv->ntot, stride = blockDim.x;
  DotAcc<T> acc;
#pragma unroll
  for (int i = 0; i < kG; i++) acc.v[i] = 0;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kV * stride) {
    T y[kV];
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t r = rb + u * stride;
      y[u] = r < c.r1 ? c.w.y[r] : (T)0;
    }
#pragma unroll
    for (int i = 0; i < kG; i++) {
      if (i < gk) {
        const T *Wi = c.w.Wb + (size_t)(i0 + i) * N;
#pragma unroll
        for (int u = 0; u < kV; u++) {
          const int64_t r = rb + u * stride;
          if (r < c.r1) acc.v[i] += y[u] * Wi[r];
        }
      }
    }
  }
  return acc;
}

// W_{j+1} = y - sum_{i <= j} coef_i W_i; returns the thread's part of ||W_{j+1}||^2.
template <typename T, bool kGrid>
__device__ __noinline__ T ph_update(Ctx<T, kGrid> c, int j, const T *coef) {
  const int64_t N = c.pv->ntot, stride = blockDim.x;
  T *Wn = c.w.Wb + (size_t)(j + 1) * N;
  T nacc = 0;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kV * stride) {
    T a[kV];
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t r = rb + u * stride;
      a[u] = r < c.r1 ? c.w.y[r] : (T)0;
    }
#pragma unroll 1
    for (int i = 0; i <= j; i++) {
      const T ci = coef[i];
      const T *Wi = c.w.Wb + (size_t)i * N;
      T w[kV];
#pragma unroll
      for (int u = 0; u < kV; u++) {
        const int64_t r = rb + u * stride;
        w[u] = r < c.r1 ? Wi[r] : (T)0;
      }
#pragma unroll
      for (int u = 0; u < kV; u++) a[u] -= ci * w[u];
    }
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t r = rb + u * stride;
      if (r < c.r1) {
        Wn[r] = a[u];
        nacc += a[u] * a[u];
      }
    }
  }
  return nacc;
}

// V += sum_{i < k} coef_i Z_i (identity rows keep their value).  With Vin non-null this is
// the step's first update and V starts from x0 = 2 Vin - V.
template <typename T, bool kGrid>
__device__ __noinline__ void ph_xupdate(Ctx<T, kGrid> c, int k, const T *coef, double *Vout,
                                        const double *Vin) {
  const int64_t N = c.pv->ntot, stride = blockDim.x;
  const uint8_t *rowf = c.iv->rowf;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kV * stride) {
    T a[kV];
    uint8_t fl[kV];
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t r = rb + u * stride;
      a[u] = 0;
      fl[u] = r < c.r1 ? rowf[r] : (uint8_t)R_IDENT;
    }
#pragma unroll 1
    for (int i = 0; i < k; i++) {
      const T ci = coef[i];
      const T *Zi = c.w.Z + (size_t)i * N;
      T z[kV];
#pragma unroll
      for (int u = 0; u < kV; u++) {
        const int64_t r = rb + u * stride;
        z[u] = r < c.r1 ? Zi[r] : (T)0;
      }
#pragma unroll
      for (int u = 0; u < kV; u++) a[u] += ci * z[u];
    }
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t r = rb + u * stride;
      if (!(fl[u] & R_IDENT)) {
        const double base = Vin ? x0_of(Vin, Vout, r) : Vout[r];
        Vout[r] = base + (double)a[u];
      }
    }
  }
}

// A Richardson step's update V += Z_0 (identity rows keep their value), with every load of
// a thread's kV rows issued before any use.  With Vin non-null this is the step's first
// update and V starts from x0 = 2 Vin - V.  Equal bit for bit to ph_xupdate with k = 1 and
// coefficient 1.
template <typename T, bool kGrid>
__device__ __noinline__ void ph_rich_update(Ctx<T, kGrid> c, double *Vout, const double *Vin) {
  const int64_t stride = blockDim.x;
  const uint8_t *rowf = c.iv->rowf;
  const T *Z = c.w.Z;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kV * stride) {
    uint8_t fl[kV];
    T z[kV];
    double v[kV], w[kV];
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t r = rb + u * stride;
      const bool ok = r < c.r1;
      fl[u] = ok ? rowf[r] : (uint8_t)R_IDENT;
      z[u] = ok ? Z[r] : (T)0;
      v[u] = ok ? Vout[r] : 0.0;
      w[u] = ok && Vin ? Vin[r] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t r = rb + u * stride;
      if (!(fl[u] & R_IDENT)) Vout[r] = (Vin ? 2.0 * w[u] - v[u] : v[u]) + (double)z[u];
    }
  }
}

// ---- BiCGSTAB (right-preconditioned, on the correction equation of one refinement cycle)

// p = r + beta (p - omega v); beta == 0 gives p = r.
template <typename T, bool kGrid>
__device__ __noinline__ void ph_bicg_dir(Ctx<T, kGrid> c, const T *r, T *p, const T *v, T beta,
                                         T omega) {
  const int64_t stride = blockDim.x;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kV * stride) {
    T a[kV], b[kV], d[kV];
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t q = rb + u * stride;
      const bool ok = q < c.r1;
      a[u] = ok ? r[q] : (T)0;
      b[u] = ok && beta != (T)0 ? p[q] : (T)0;
      d[u] = ok && beta != (T)0 ? v[q] : (T)0;
    }
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t q = rb + u * stride;
      if (q < c.r1) p[q] = a[u] + beta * (b[u] - omega * d[u]);
    }
  }
}

// out = A x; returns the thread's parts of <out, d0> and <out, d1> (d1 may be null).
template <typename T, bool kGrid>
__device__ __noinline__ DotAcc<T> ph_matvec(Ctx<T, kGrid> c, const T *x, T *out, const T *d0,
                                            const T *d1) {
  const PackView &pv = *c.pv;
  const ImView &iv = *c.iv;
  const int64_t stride = blockDim.x;
  const T *CT = (const T *)iv.cdiag;
  const T *GT = sizeof(T) == 4 ? (const T *)(const void *)iv.gf : (const T *)(const void *)iv.g64;
  DotAcc<T> acc;
#pragma unroll
  for (int i = 0; i < kG; i++) acc.v[i] = 0;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kU * stride) {
    T y[kU], e0[kU], e1[kU];
    uint8_t fl[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int64_t q = rb + u * stride;
      e0[u] = q < c.r1 ? d0[q] : (T)0;
      e1[u] = q < c.r1 && d1 ? d1[q] : (T)0;
    }
    apply_rows_c<kU>(pv, iv, CT, GT, x, rb, stride, c.r1, y, fl);
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int64_t q = rb + u * stride;
      if (q < c.r1) out[q] = y[u];
      acc.v[0] += y[u] * e0[u];
      acc.v[1] += y[u] * e1[u];
    }
  }
  return acc;
}

// s = r - alpha v; returns the thread's part of ||s||^2.
template <typename T, bool kGrid>
__device__ __noinline__ T ph_bicg_s(Ctx<T, kGrid> c, const T *r, const T *v, T alpha, T *s) {
  const int64_t stride = blockDim.x;
  T acc = 0;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kV * stride) {
    T a[kV], b[kV];
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t q = rb + u * stride;
      a[u] = q < c.r1 ? r[q] : (T)0;
      b[u] = q < c.r1 ? v[q] : (T)0;
    }
#pragma unroll
    for (int u = 0; u < kV; u++) {
      const int64_t q = rb + u * stride;
      const T x = a[u] - alpha * b[u];
      if (q < c.r1) s[q] = x;
      acc += x * x;
    }
  }
  return acc;
}

// V += alpha ph + omega sh (FP64 accumulation; identity rows keep their value) and
// r = s - omega t; returns the thread's parts of ||r||^2 and <rh, r>.
template <typename T, bool kGrid>
__device__ __noinline__ DotAcc<T> ph_bicg_x(Ctx<T, kGrid> c, const T *ph, const T *sh,
                                            const T *s, const T *t, T alpha, T omega, T *r,
                                            const T *rh, double *Vout) {
  const int64_t stride = blockDim.x;
  const uint8_t *rowf = c.iv->rowf;
  DotAcc<T> acc;
#pragma unroll
  for (int i = 0; i < kG; i++) acc.v[i] = 0;
  for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kU * stride) {
    T a[kU], b[kU], e[kU], f[kU], h[kU];
    uint8_t fl[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int64_t q = rb + u * stride;
      const bool ok = q < c.r1;
      a[u] = ok ? ph[q] : (T)0;
      b[u] = ok ? sh[q] : (T)0;
      e[u] = ok ? s[q] : (T)0;
      f[u] = ok ? t[q] : (T)0;
      h[u] = ok ? rh[q] : (T)0;
      fl[u] = ok ? rowf[q] : (uint8_t)R_IDENT;
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int64_t q = rb + u * stride;
      const T rn = e[u] - omega * f[u];
      if (q < c.r1) r[q] = rn;
      if (!(fl[u] & R_IDENT)) Vout[q] += (double)(alpha * a[u] + omega * b[u]);
      acc.v[0] += rn * rn;
      acc.v[1] += rn * h[u];
    }
  }
  return acc;
}

// One refinement cycle of BiCGSTAB on A d = r0 (r0 in W_0, ||r0|| = res), accumulating
// d into V.  Stops at the cycle target, at the budget, or on a breakdown (the next cycle
// restarts from the true residual).  Every pass through the loop counts against the
// budget, so repeated breakdowns still end the step.
// Not inlined, so that the GMRES path's register allocation does not carry it.
// Returns {parity, iters}.
template <typename T, bool kGrid>
__device__ __noinline__ int2 bicgstab_cycle(Ctx<T, kGrid> c, int parity, double res,
                                            double cycle_target, int budget, int iters,
                                            double *Vout) {
  const ImView &iv = *c.iv;
  cg::grid_group grid = cg::this_grid();
  Shared S = carve(dyn_smem(), iv.m);
  const int64_t N = c.pv->ntot;
  T *rh = c.w.Wb, *r1 = c.w.Wb + N, *p = c.w.Wb + 2 * N, *v = c.w.Wb + 3 * N;
  T *ph = c.w.Z, *sh = c.w.Z + N, *s = c.w.Z + 2 * N, *t = c.w.Z + 3 * N;
  const T *r = rh;  // the first iteration reads r0 itself
  double rho = res * res, rho_prev = 1.0, alpha = 1.0, omega = 1.0;
  for (int it = 0; iters < budget; it++) {
    const double beta = it == 0 ? 0.0 : (rho / rho_prev) * (alpha / omega);
    ph_bicg_dir(c, r, p, v, (T)beta, (T)omega);
    group_sync<kGrid>(grid);
    apply_precond(c, p, ph);
    group_sync<kGrid>(grid);
    {
      DotAcc<T> acc = ph_matvec(c, ph, v, rh, (const T *)nullptr);
      group_reduce<kGrid>(grid, acc.v, 1, S, iv.partials, parity);
    }
    const double rv = S.red[0];
    if (rv == 0.0 || !(rv == rv) || !(rho == rho)) {  // breakdown: restart from r0
      iters++;
      break;
    }
    alpha = rho / rv;
    {
      T acc[1] = {ph_bicg_s(c, r, v, (T)alpha, s)};
      group_reduce<kGrid>(grid, acc, 1, S, iv.partials, parity);
    }
    iters++;
    if (sqrt(S.red[0]) <= cycle_target) {  // x += alpha ph completes the cycle
      ph_bicg_x(c, ph, ph, s, s, (T)alpha, (T)0, r1, rh, Vout);
      group_sync<kGrid>(grid);
      break;
    }
    apply_precond(c, s, sh);
    group_sync<kGrid>(grid);
    {
      DotAcc<T> acc = ph_matvec(c, sh, t, s, t);
      group_reduce<kGrid>(grid, acc.v, 2, S, iv.partials, parity);
    }
    const double ts = S.red[0], tt = S.red[1];
    omega = tt > 0.0 ? ts / tt : 0.0;
    {
      DotAcc<T> acc = ph_bicg_x(c, ph, sh, s, t, (T)alpha, (T)omega, r1, rh, Vout);
      group_reduce<kGrid>(grid, acc.v, 2, S, iv.partials, parity);
    }
    r = r1;
    const double rn = sqrt(S.red[0]);
    rho_prev = rho;
    rho = S.red[1];
    if (rn <= cycle_target || omega == 0.0 || rho == 0.0) break;
  }
  group_sync<kGrid>(grid);  // V complete before the next true residual
  return make_int2(parity, iters);
}

// One backward-Euler step of one group (CTA or grid) for instance `inst`.
template <typename T, bool kGrid>
__device__ __forceinline__ void implicit_one_step(Ctx<T, kGrid> &c, cg::grid_group &grid,
                                                  Shared &S, int &parity, const double *Vin,
                                                  double *Vout, bool active, int64_t inst_n,
                                                  int inst) {
  const ImView &iv = *c.iv;
  const int m = iv.m;
  T *coef = (T *)S.coef;
  // ---- assembly, fused with the first true residual (W_0); V still holds V^{n-1}
  const double2 br = ph_assemble(c, Vin, Vout, active ? 1 : 0, inst);
  __syncthreads();
  if (iv.precond == NRT_PRECOND_SEGMENT) {
    factor_pieces(c);
  } else if (iv.precond == NRT_PRECOND_TREE) {
    level_sync<kGrid>(grid);  // c of every row visible before the elimination
    tree_factor(c);
  }
  double target = iv.tol, res0 = 0;
  {
    double acc[2] = {br.x, br.y};
    group_reduce<kGrid>(grid, acc, 2, S, iv.partials, parity);  // also publishes W_0
    if (iv.tol_mode == NRT_TOL_REL) target = iv.tol * sqrt(S.red[0]);
    res0 = sqrt(S.red[1]);
    if (!kGrid) __syncthreads();
  }
  const int budget = iv.max_iter > 0 ? iv.max_iter : (iv.max_iter < 0 ? 0 : (int)inst_n);
  const double inner_rel = iv.inner_rel;
  int iters = 0, n_res = 0, n_app = 0, n_xup = 0, n_basis = 0, n_rich = 0;
  double res = 0, prev_res = 0;
  bool converged = false;
  bool x0_pending = true;  // V holds V^{n-1} until the first solution update
  // Mixed precision with the tree preconditioner: M is the FP32 factorisation of A itself,
  // so GMRES's one Arnoldi step per cycle takes x += y M^-1 r with y within rounding of 1.
  // A Richardson step takes x += M^-1 r without the SpMV, the products and the basis
  // update.  The FP64 residual that opens the next cycle checks it: a cycle that does not
  // lower the true residual tenfold hands the rest of the step to GMRES cycles.
  bool rich = iv.rich != 0;
  for (int cycle = 0;; cycle++) {
    // ---- cycle start: true residual r = b - A x in FP64, W_0 = r, Z_0 = M^-1 r
    if (cycle == 0) {
      res = res0;
    } else {
      // res > 0 here (a zero residual has converged); the scale stays a normal FP32 number
      const bool f32 = sizeof(T) == 4 && iv.krylov == NRT_GMRES;
      const int e = f32 ? max(-126, min(126, ilogb(res))) : 0;
      double acc[1] = {ph_residual(c, Vout, f32 ? exp2f((float)-e) : 0.0f)};
      group_reduce<kGrid>(grid, acc, 1, S, iv.partials, parity);
      res = sqrt(S.red[0]) * exp2((double)e);
      n_res++;
    }
    if (res <= target) {
      converged = true;
      break;
    }
    if (iters + n_rich >= budget || !(res == res)) break;  // budget spent, or not finite
    if (rich && cycle > 0 && res > 0.1 * prev_res) rich = false;
    if (iv.krylov == NRT_BICGSTAB) {
      if (x0_pending) {
        ph_x0(c, Vin, Vout);
        x0_pending = false;
        group_sync<kGrid>(grid);
      }
      const int2 pi = bicgstab_cycle(c, parity, res, fmax(target, inner_rel * res), budget,
                                     iters, Vout);
      parity = pi.x;
      iters = pi.y;
      continue;
    }
    apply_precond(c, c.w.Wb, c.w.Z);
    n_app++;
    group_sync<kGrid>(grid);  // Z_0 of every row visible before the SpMV
    if (rich) {  // x += M^-1 r
      ph_rich_update(c, Vout, x0_pending ? Vin : (const double *)nullptr);
      group_sync<kGrid>(grid);
      n_xup++;
      n_rich++;
      x0_pending = false;
      prev_res = res;
      continue;
    }
    if (threadIdx.x == 0) {
      S.g[0] = res;
      for (int i = 1; i <= m; i++) S.g[i] = 0;
      S.s[0] = 1.0 / res;
    }
    __syncthreads();
    const double cycle_target = fmax(target, inner_rel * res);
    int k = 0;
    for (int j = 0; j < m; j++) {
      // y = s_j A Z_j fused with p_i = <y, W_i> for the first kG of i <= j
      const int g1 = min(j + 1, kG);
      {
        DotAcc<T> acc = ph_spmv(c, j, (T)S.s[j], g1);
        group_reduce<kGrid>(grid, acc.v, g1, S, iv.partials, parity);
      }
      for (int i0 = kG; i0 <= j; i0 += kG) {  // remaining products, kG at a time
        const int gk = min(j + 1 - i0, kG);
        DotAcc<T> acc = ph_products(c, i0, gk);
        group_reduce<kGrid>(grid, acc.v, gk, S, iv.partials, parity, i0);
      }
      if (threadIdx.x <= j) {
        const double h = S.s[threadIdx.x] * S.red[threadIdx.x];
        S.H[threadIdx.x * m + j] = h;
        coef[threadIdx.x] = (T)(h * S.s[threadIdx.x]);
      }
      __syncthreads();
      // w = y - sum_i h_ij s_i W_i -> W_{j+1}; ||w||^2
      T nacc[1] = {ph_update(c, j, coef)};
      group_reduce<kGrid>(grid, nacc, 1, S, iv.partials, parity);  // publishes W_{j+1}
      if (threadIdx.x == 0) {
        const double hn = sqrt(S.red[0]);
        S.s[j + 1] = hn > 0 ? 1.0 / hn : 0.0;
        for (int i = 0; i < j; i++) {
          const double a = S.H[i * m + j], b = S.H[(i + 1) * m + j];
          S.H[i * m + j] = S.cs[i] * a + S.sn[i] * b;
          S.H[(i + 1) * m + j] = -S.sn[i] * a + S.cs[i] * b;
        }
        const double a = S.H[j * m + j];
        const double den = sqrt(a * a + hn * hn);
        S.cs[j] = den == 0 ? 1.0 : a / den;
        S.sn[j] = den == 0 ? 0.0 : hn / den;
        S.H[j * m + j] = den;
        S.g[j + 1] = -S.sn[j] * S.g[j];
        S.g[j] = S.cs[j] * S.g[j];
        S.flag[0] = (fabs(S.g[j + 1]) <= cycle_target || hn == 0) ? 1 : 0;
      }
      __syncthreads();
      k = j + 1;
      iters++;
      n_basis += j + 1;
      if (S.flag[0] || iters + n_rich >= budget || k >= m) break;
      // Z_{j+1} = M^-1 W_{j+1}, only when another Arnoldi step will use it
      apply_precond(c, c.w.Wb + (size_t)(j + 1) * c.pv->ntot, c.w.Z + (size_t)(j + 1) * c.pv->ntot);
      n_app++;
      group_sync<kGrid>(grid);  // Z_{j+1} of every row visible before the next SpMV
    }
    // ---- x += sum_i y_i s_i Z_i
    if (threadIdx.x == 0) {
      for (int i = k - 1; i >= 0; i--) {
        double a = S.g[i];
        for (int l = i + 1; l < k; l++) a -= S.H[i * m + l] * S.y[l];
        S.y[i] = a / S.H[i * m + i];
      }
      for (int i = 0; i < k; i++) coef[i] = (T)(S.y[i] * S.s[i]);
    }
    __syncthreads();
    ph_xupdate(c, k, coef, Vout, x0_pending ? Vin : (const double *)nullptr);
    group_sync<kGrid>(grid);
    n_xup++;
    x0_pending = false;
  }
  if (x0_pending) ph_x0(c, Vin, Vout);  // converged (or out of budget) at x0 itself
  if (threadIdx.x == 0 && (!kGrid || blockIdx.x == 0)) {
    InstStat &st = iv.stats[inst];
    st.iters += iters;
    st.last_iters = iters;
    st.last_res = res;
    if (!converged) st.nonconv += 1;
    st.residuals += n_res;
    st.applies += n_app;
    st.xupdates += n_xup;
    st.basis += n_basis;
    st.rich += n_rich;
  }
  group_sync<kGrid>(grid);  // V^{n+1} complete before the next step reads it
}

// Recording at the probes of instance `inst` after the step at loop index i (V is that
// step's output, complete in this CTA's view).  Each thread keeps the same probes for the
// whole launch.
__device__ __noinline__ void ph_record(const RecView *rp, int inst, int64_t i, const double *V,
                                       double dT) {
  const RecView r = *rp;
  const int a = r.p0[inst], b = r.p0[inst + 1];
  for (int p = a + threadIdx.x; p < b; p += blockDim.x) record_probe(r, p, i, V[r.src[p]], dT);
}

template <typename T, bool kGrid>
__global__ void __launch_bounds__(kThreads, 4) implicit_steps(const PackView *pvp, const ImView *ivp,
                                                           int nsteps, int force, double *V0,
                                                           double *V1, int cur,
                                                           const RecView *rec) {
  const ImView &iv = *ivp;
  Shared S = carve(dyn_smem(), iv.m);
  cg::grid_group grid = cg::this_grid();
  int parity = 0;
  if (threadIdx.x == 0) {
    mbar_init(S.bar, 1);
    S.flag[2] = 0;
  }
  __syncthreads();
  Ctx<T, kGrid> c;
  c.pv = pvp;
  c.iv = ivp;
  c.w.Wb = (T *)iv.Wb;
  c.w.Z = (T *)iv.Z;
  c.w.y = (T *)iv.yv;
  c.w.pd = (T *)iv.pcd;
  c.w.pc = (T *)iv.pcc;
  if (kGrid) {
    c.r0 = iv.cta_row[blockIdx.x];
    c.r1 = iv.cta_row[blockIdx.x + 1];
    c.t0 = iv.cta_tile[blockIdx.x];
    c.t1 = iv.cta_tile[blockIdx.x + 1];
    c.l0 = iv.work_lev ? iv.work_lev[blockIdx.x] : 0;
    c.l1 = iv.work_lev ? iv.work_lev[blockIdx.x + 1] : 0;
    const InstDev in = pvp->inst[0];
    const int64_t inst_n = iv.inst_row[1] - iv.inst_row[0];
    int s = 0;
    for (; s < nsteps; s++) {
      const int64_t i = in.base + s;
      if (i >= in.iend) break;
      const bool active = force >= 0 ? force != 0
                                     : (i >= in.ion && i <= in.ioff);
      implicit_one_step<T, kGrid>(c, grid, S, parity, ((cur + s) & 1) ? V1 : V0,
                                  ((cur + s + 1) & 1) ? V1 : V0, active, inst_n, 0);
      if (rec && blockIdx.x == 0) ph_record(rec, 0, i, ((cur + s + 1) & 1) ? V1 : V0, in.dT);
    }
    if ((nsteps - s) & 1) {  // the run ended inside the launch: each CTA moves its rows
      double *dst = ((cur + nsteps) & 1) ? V1 : V0;
      const double *src = ((cur + s) & 1) ? V1 : V0;
      for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x) dst[j] = src[j];
    }
  } else {
    for (;;) {
      if (threadIdx.x == 0) S.flag[1] = atomicAdd(iv.queue, 1);
      __syncthreads();
      const int q = S.flag[1];
      __syncthreads();
      if (q >= iv.ninst) break;
      const int inst = iv.order[q];
      c.r0 = iv.inst_row[inst];
      c.r1 = iv.inst_row[inst + 1];
      c.t0 = iv.inst_tile[inst];
      c.t1 = iv.inst_tile[inst + 1];
      c.l0 = iv.work_lev ? iv.work_lev[inst] : 0;
      c.l1 = iv.work_lev ? iv.work_lev[inst + 1] : 0;
      const InstDev in = pvp->inst[inst];
      int s = 0;
      for (; s < nsteps; s++) {
        const int64_t i = in.base + s;
        if (i >= in.iend) break;
        const bool active = force >= 0 ? force != 0
                                       : (i >= in.ion && i <= in.ioff);
        implicit_one_step<T, kGrid>(c, grid, S, parity, ((cur + s) & 1) ? V1 : V0,
                                    ((cur + s + 1) & 1) ? V1 : V0, active, c.r1 - c.r0, inst);
        if (rec) ph_record(rec, inst, i, ((cur + s + 1) & 1) ? V1 : V0, in.dT);
      }
      if ((nsteps - s) & 1) {  // finished early: put its latest V where the others' is
        double *dst = ((cur + nsteps) & 1) ? V1 : V0;
        const double *src = ((cur + s) & 1) ? V1 : V0;
        for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x) dst[j] = src[j];
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------- host side

// Schedule of the exact tree preconditioner.  Segments are maximal runs of physical rows
// each linked to the previous row (mother == j - 1), broken after every branch point and
// at `cap` rows; a segment's parent row (the mother of its first row) is then always the
// last row of its parent segment.  Level = number of segments above.  Each worker (one
// CTA of the cooperative launch, or one instance of a batch) gets, per level (deepest
// first), tiles of whole segments whose slots fit the shared-memory staging area; every
// tile starts on a multiple of 16 slots (padding slots in between have row -1).
struct TreeSchedule {  // sized without a fill: every entry is written by the builders
  hvec<int> seg_len, seg_c1, seg_c2, seg_prow, seg_soff;  // tile order
  hvec<int> tile_seg, tile_slot, slot_row, lev_tile, work_lev;
  hvec<uint8_t> slot_flag;
  int local_top = -1;  // ImView::local_top
};

struct ImplicitState {
  ImView iv{};
  PackView *d_pv = nullptr;  // device copies the kernel reads
  ImView *d_iv = nullptr;
  hvec<uint8_t> rowf;  // sized without a fill: implicit_plan writes every row
  hvec<int2> pieces;
  std::vector<int> tiles, cta_row, cta_tile, inst_tile, order;
  std::vector<int64_t> inst_row;
  TreeSchedule tree;
  int grid_blocks = 0;
  bool grid_mode = false;
  int tile_rows = 0;
  size_t smem = 0;
};

static size_t smem_bytes(int m) { return ((shared_fixed_bytes(m) + 127) & ~(size_t)127) + kTileBytes; }

template <typename X>
static int up(Arena &a, X *&dst, const X *src, size_t count, cudaStream_t st) {
  dst = (X *)a.take(sizeof(X) * (count ? count : 1));
  if (!dst) {
    set_error("arena exhausted");
    return NRT_ENOMEM;
  }
  if (src && count) NRT_CUDA(cudaMemcpyAsync(dst, src, sizeof(X) * count, cudaMemcpyHostToDevice, st));
  return NRT_OK;
}

#define TRYI(x)                     \
  do {                              \
    int _rc = (x);                  \
    if (_rc != NRT_OK) return _rc;  \
  } while (0)

static void build_tree_schedule(const HostPack &host, int cap, bool grid_mode, int ctas,
                                TreeSchedule &T) {
  struct Seg {
    int start, len, prow, parent, level, c1, c2;
  };
  std::vector<Seg> segs;
  std::vector<int> seg_of(host.ntot, -1);
  std::vector<int> inst_seg(host.ninst + 1, 0);
  for (int32_t i = 0; i < host.ninst; i++) {
    const int64_t o = host.off[i], n = host.num_elem[i];
    int cur = -1;
    for (int64_t jl = 0; jl < n; jl++) {
      const int64_t j = o + jl;
      const Topo &t = host.topo[j];
      if (t.flags & F_IDENT) {
        cur = -1;
        continue;
      }
      const bool linked = cur >= 0 && (t.flags & F_UP) && t.mother == j - 1 &&
                          !(host.topo[j - 1].flags & F_BRANCH) && segs[cur].len < cap;
      if (linked) {
        segs[cur].len++;
      } else {
        Seg s;
        s.start = (int)j;
        s.len = 1;
        s.prow = (t.flags & F_UP) ? t.mother : -1;
        s.parent = s.prow >= 0 ? seg_of[s.prow] : -1;
        s.level = s.parent >= 0 ? segs[s.parent].level + 1 : 0;
        s.c1 = s.c2 = -1;
        segs.push_back(s);
        cur = (int)segs.size() - 1;
        if (s.parent >= 0) {
          Seg &p = segs[s.parent];
          (p.c1 < 0 ? p.c1 : p.c2) = cur;
        }
      }
      seg_of[j] = cur;
    }
    inst_seg[i + 1] = (int)segs.size();
  }
  // Workers: instances (batch) or CTAs (one tree; each level's segments dealt out to the
  // CTAs by rows).  Every worker of a cooperative launch sees the same number of levels.
  const int nwork = grid_mode ? ctas : host.ninst;
  int max_level = 0;
  for (const Seg &s : segs) max_level = std::max(max_level, s.level);
  std::vector<std::vector<std::vector<int>>> lists(nwork);  // [worker][level] -> segments
  if (grid_mode) {
    std::vector<std::vector<int>> by_level(max_level + 1);
    for (int s = 0; s < (int)segs.size(); s++) by_level[segs[s].level].push_back(s);
    for (int w = 0; w < nwork; w++) lists[w].resize(max_level + 1);
    std::vector<int64_t> level_rows(max_level + 1, 0);
    for (int L = 0; L <= max_level; L++)
      for (int s : by_level[L]) level_rows[L] += segs[s].len;
    // The top levels, while together they fit one tile, all go to CTA 0: a grid-wide sync
    // between two of them would wait on CTAs that have nothing to do there.
    int64_t top_rows = 0;
    T.local_top = -1;
    for (int L = 0; L <= max_level && top_rows + level_rows[L] <= cap; L++) {
      top_rows += level_rows[L];
      T.local_top = L;
    }
    for (int L = 0; L <= max_level; L++) {
      int64_t acc = 0;
      for (int s : by_level[L]) {
        const int w = L <= T.local_top ? 0
                                       : (int)std::min<int64_t>(nwork - 1, acc * nwork /
                                                                std::max<int64_t>(level_rows[L], 1));
        lists[w][L].push_back(s);
        acc += segs[s].len;
      }
    }
  } else {
    for (int32_t i = 0; i < host.ninst; i++) {
      int ml = 0;
      for (int s = inst_seg[i]; s < inst_seg[i + 1]; s++) ml = std::max(ml, segs[s].level);
      lists[i].resize(ml + 1);
      for (int s = inst_seg[i]; s < inst_seg[i + 1]; s++) lists[i][segs[s].level].push_back(s);
    }
  }
  // Emit in (worker, level deepest first, tile) order; renumber segments accordingly.
  std::vector<int> newid(segs.size(), -1);
  std::vector<int> order;
  auto pad = [&]() {
    T.slot_row.push_back(-1);
    T.slot_flag.push_back(SL_PAD | SL_FIRST | SL_LAST);
  };
  auto new_tile = [&]() {
    while (T.slot_row.size() & 15) pad();
    T.tile_seg.push_back((int)order.size());
    T.tile_slot.push_back((int)T.slot_row.size());
  };
  T.work_lev.assign(nwork + 1, 0);
  for (int w = 0; w < nwork; w++) {
    T.work_lev[w] = (int)T.lev_tile.size();
    for (int L = (int)lists[w].size() - 1; L >= 0; L--) {
      T.lev_tile.push_back((int)T.tile_seg.size());
      int used = cap;  // forces a new tile for the first segment
      for (int s : lists[w][L]) {
        if (used + segs[s].len > cap) {
          new_tile();
          used = 0;
        }
        newid[s] = (int)order.size();
        order.push_back(s);
        T.seg_soff.push_back(used);
        for (int k = 0; k < segs[s].len; k++) {
          T.slot_row.push_back(segs[s].start + k);
          T.slot_flag.push_back((k == 0 ? SL_FIRST : 0) | (k == segs[s].len - 1 ? SL_LAST : 0));
        }
        used += segs[s].len;
      }
    }
  }
  T.work_lev[nwork] = (int)T.lev_tile.size();
  T.lev_tile.push_back((int)T.tile_seg.size());
  new_tile();  // sentinel: end of the last tile
  for (int k = 0; k < 16; k++) pad();  // bulk copies round their size up to 16 bytes
  for (int s : order) {
    const Seg &g = segs[s];
    T.seg_len.push_back(g.len);
    T.seg_prow.push_back(g.prow);
    T.seg_c1.push_back(g.c1 >= 0 ? newid[g.c1] : -1);
    T.seg_c2.push_back(g.c2 >= 0 ? newid[g.c2] : -1);
  }
}

// The same schedule for a batch (one worker per instance), built per instance on all host
// cores and concatenated: every instance's slots are padded to a multiple of 16, which is
// where the sequential builder's next tile would start, so the result is the same.
struct InstSchedule {
  std::vector<int> seg_len, seg_c1, seg_c2, seg_prow, seg_soff, tile_seg, tile_slot, slot_row,
      lev_tile;
  std::vector<uint8_t> slot_flag;
};

static void instance_schedule(const HostPack &host, int cap, int32_t i, InstSchedule &L) {
  struct Seg {
    int start, len, prow, parent, level, c1, c2;
  };
  const int64_t o = host.off[i], n = host.num_elem[i];
  std::vector<Seg> segs;
  std::vector<int> seg_of(n, -1);
  int cur = -1;
  for (int64_t jl = 0; jl < n; jl++) {
    const int64_t j = o + jl;
    const Topo &t = host.topo[j];
    if (t.flags & F_IDENT) {
      cur = -1;
      continue;
    }
    const bool linked = cur >= 0 && (t.flags & F_UP) && t.mother == j - 1 &&
                        !(host.topo[j - 1].flags & F_BRANCH) && segs[cur].len < cap;
    if (linked) {
      segs[cur].len++;
    } else {
      Seg s;
      s.start = (int)j;
      s.len = 1;
      s.prow = (t.flags & F_UP) ? t.mother : -1;
      s.parent = s.prow >= 0 ? seg_of[s.prow - o] : -1;
      s.level = s.parent >= 0 ? segs[s.parent].level + 1 : 0;
      s.c1 = s.c2 = -1;
      segs.push_back(s);
      cur = (int)segs.size() - 1;
      if (s.parent >= 0) {
        Seg &p = segs[s.parent];
        (p.c1 < 0 ? p.c1 : p.c2) = cur;
      }
    }
    seg_of[jl] = cur;
  }
  int ml = 0;
  for (const Seg &s : segs) ml = std::max(ml, s.level);
  std::vector<std::vector<int>> lists(segs.empty() ? 0 : ml + 1);
  for (int s = 0; s < (int)segs.size(); s++) lists[segs[s].level].push_back(s);
  std::vector<int> newid(segs.size(), -1), order;
  auto pad = [&]() {
    L.slot_row.push_back(-1);
    L.slot_flag.push_back(SL_PAD | SL_FIRST | SL_LAST);
  };
  for (int lv = (int)lists.size() - 1; lv >= 0; lv--) {
    L.lev_tile.push_back((int)L.tile_seg.size());
    int used = cap;
    for (int s : lists[lv]) {
      if (used + segs[s].len > cap) {
        while (L.slot_row.size() & 15) pad();
        L.tile_seg.push_back((int)order.size());
        L.tile_slot.push_back((int)L.slot_row.size());
        used = 0;
      }
      newid[s] = (int)order.size();
      order.push_back(s);
      L.seg_soff.push_back(used);
      for (int q = 0; q < segs[s].len; q++) {
        L.slot_row.push_back(segs[s].start + q);
        L.slot_flag.push_back((q == 0 ? SL_FIRST : 0) | (q == segs[s].len - 1 ? SL_LAST : 0));
      }
      used += segs[s].len;
    }
  }
  while (L.slot_row.size() & 15) pad();
  for (int s : order) {
    const Seg &g = segs[s];
    L.seg_len.push_back(g.len);
    L.seg_prow.push_back(g.prow);
    L.seg_c1.push_back(g.c1 >= 0 ? newid[g.c1] : -1);
    L.seg_c2.push_back(g.c2 >= 0 ? newid[g.c2] : -1);
  }
}

static void build_tree_schedule_batch(const HostPack &host, int cap, TreeSchedule &T) {
  const int32_t ni = host.ninst;
  std::vector<InstSchedule> loc(ni);
  parallel_for(ni, [&](int64_t i) { instance_schedule(host, cap, (int32_t)i, loc[i]); });
  // bases: segments, slots, tiles, level entries
  std::vector<size_t> sb(ni + 1, 0), lb(ni + 1, 0), tb(ni + 1, 0), eb(ni + 1, 0);
  for (int32_t i = 0; i < ni; i++) {
    sb[i + 1] = sb[i] + loc[i].seg_len.size();
    lb[i + 1] = lb[i] + loc[i].slot_row.size();
    tb[i + 1] = tb[i] + loc[i].tile_seg.size();
    eb[i + 1] = eb[i] + loc[i].lev_tile.size();
  }
  T.seg_len.resize(sb[ni]); T.seg_c1.resize(sb[ni]); T.seg_c2.resize(sb[ni]);
  T.seg_prow.resize(sb[ni]); T.seg_soff.resize(sb[ni]);
  T.slot_row.resize(lb[ni]); T.slot_flag.resize(lb[ni]);
  T.tile_seg.resize(tb[ni]); T.tile_slot.resize(tb[ni]);
  T.lev_tile.resize(eb[ni]);
  T.work_lev.assign(ni + 1, 0);
  parallel_for(ni, [&](int64_t i) {
    const InstSchedule &L = loc[i];
    const int s0 = (int)sb[i], l0 = (int)lb[i], t0 = (int)tb[i];
    for (size_t q = 0; q < L.seg_len.size(); q++) {
      T.seg_len[s0 + q] = L.seg_len[q];
      T.seg_prow[s0 + q] = L.seg_prow[q];
      T.seg_soff[s0 + q] = L.seg_soff[q];
      T.seg_c1[s0 + q] = L.seg_c1[q] >= 0 ? L.seg_c1[q] + s0 : -1;
      T.seg_c2[s0 + q] = L.seg_c2[q] >= 0 ? L.seg_c2[q] + s0 : -1;
    }
    std::copy(L.slot_row.begin(), L.slot_row.end(), T.slot_row.begin() + l0);
    std::copy(L.slot_flag.begin(), L.slot_flag.end(), T.slot_flag.begin() + l0);
    for (size_t q = 0; q < L.tile_seg.size(); q++) {
      T.tile_seg[t0 + q] = L.tile_seg[q] + s0;
      T.tile_slot[t0 + q] = L.tile_slot[q] + l0;
    }
    for (size_t q = 0; q < L.lev_tile.size(); q++) T.lev_tile[eb[i] + q] = L.lev_tile[q] + t0;
    T.work_lev[i] = (int)eb[i];
  });
  T.work_lev[ni] = (int)T.lev_tile.size();
  T.lev_tile.push_back((int)T.tile_seg.size());
  // sentinel tile (the slot count is already a multiple of 16), then the copy overrun pad
  T.tile_seg.push_back((int)T.seg_len.size());
  T.tile_slot.push_back((int)T.slot_row.size());
  for (int q = 0; q < 16; q++) {
    T.slot_row.push_back(-1);
    T.slot_flag.push_back(SL_PAD | SL_FIRST | SL_LAST);
  }
}

// Groups pieces [pa, pb) into tiles whose row span fits the shared-memory staging area.
static void make_tiles(const hvec<int2> &pieces, int pa, int pb, int tile_rows,
                       std::vector<int> &tiles) {
  int64_t start_row = -1;
  for (int p = pa; p < pb; p++) {
    const int64_t end = (int64_t)pieces[p].x + pieces[p].y;
    if (start_row < 0 || end - start_row > tile_rows) {
      tiles.push_back(p);
      start_row = pieces[p].x;
    }
  }
}

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// Row structure, launch shape and preconditioner schedule; the exact device bytes the
// implicit workspace takes from the arena.
int Engine::implicit_plan(size_t &bytes) {
  im = new ImplicitState();
  ImplicitState &S = *im;
  const int64_t N = host.ntot;
  const int32_t ni = host.ninst;
  // Row structure (flags) per element.  The validator guaranteed the reference
  // numbering: mother < j, DR == j + 1 off terminals, terminals follow their mother.
  S.rowf.resize(N);
  parallel_for(ni, [&](int64_t i) {
    const int64_t o = host.off[i], n = host.num_elem[i];
    for (int64_t jl = 0; jl < n; jl++) {
      const int64_t j = o + jl;
      Topo &t = host.topo[j];
      t.flags &= ~(uint32_t)(F_UP | F_DOWNR | F_DOWNL | F_IDENT);
      uint8_t rf = (t.flags & F_HH) ? R_HH : 0;
      if (host.inp[j] != 0.0) rf |= R_INP;
      const bool ident = jl == 0 || jl == n - 1 || (t.flags & F_TERM);
      if (ident) {
        t.flags |= F_IDENT;
        S.rowf[j] = rf | R_IDENT;
        continue;
      }
      if (jl != 1) {
        t.flags |= F_UP;
        rf |= R_UP;
        if (t.mother != j - 1) rf |= R_FAR;
      }
      if (!(host.topo[j + 1].flags & F_TERM)) {  // j + 1 is in this instance (j < o + n - 1)
        t.flags |= F_DOWNR;
        rf |= R_DOWNR;
      }
      if (t.flags & F_BRANCH) {
        t.flags |= F_DOWNL;
        rf |= R_DOWNL;
      }
      S.rowf[j] = rf;
    }
  });
  // Segment pieces: maximal runs of consecutive physical rows linked to their
  // predecessor (mother == j - 1 with a mother column), cut at kMaxPiece rows.
  S.inst_row.assign(host.off.begin(), host.off.end());
  std::vector<int> inst_piece(ni + 1, 0);
  {
    std::vector<std::vector<int2>> ip(ni);  // per instance, then concatenated in order
    parallel_for(ni, [&](int64_t i) {
      const int64_t o = host.off[i], n = host.num_elem[i];
      int64_t start = -1;
      for (int64_t jl = 0; jl < n; jl++) {
        const int64_t j = o + jl;
        const Topo &t = host.topo[j];
        const bool ident = t.flags & F_IDENT;
        const bool linked = !ident && (t.flags & F_UP) && t.mother == j - 1 && start >= 0 &&
                            (j - start) < kMaxPiece;
        if (!linked && start >= 0) {
          ip[i].push_back(make_int2((int)start, (int)(j - start)));
          start = -1;
        }
        if (!ident && start < 0) start = j;
      }
      if (start >= 0) ip[i].push_back(make_int2((int)start, (int)(o + n - start)));
    });
    for (int32_t i = 0; i < ni; i++) inst_piece[i + 1] = inst_piece[i] + (int)ip[i].size();
    S.pieces.resize(inst_piece[ni]);
    parallel_for(ni, [&](int64_t i) {
      std::copy(ip[i].begin(), ip[i].end(), S.pieces.begin() + inst_piece[i]);
    });
  }
  const int np = (int)S.pieces.size();
  const size_t tb = opt.precision == NRT_MIXED ? 4 : 8;
  S.tile_rows = (int)(kTileBytes / (4 * tb));
  int dev_sms = 0;
  NRT_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device));
  S.smem = smem_bytes(opt.restart);
  const bool mixed = opt.precision == NRT_MIXED;
  S.grid_mode = ni == 1 && opt.schedule == 0;
  if (S.grid_mode) {
    // One tree: cooperative grid, row ranges aligned with pieces.
    int per_sm = 0;
    auto kern = mixed ? implicit_steps<float, true> : implicit_steps<double, true>;
    NRT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S.smem));
    NRT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, S.smem));
    if (per_sm < 1) {
      set_error("implicit kernel does not fit on an SM");
      return NRT_EDEVICE;
    }
    const int64_t want = (N + 4 * kThreads - 1) / (4 * kThreads);
    int G = (int)std::min<int64_t>((int64_t)dev_sms * std::min(per_sm, 2), std::max<int64_t>(1, want));
    G = std::max(1, std::min(G, 4096));
    std::vector<int> cta_piece(G + 1, np);
    S.cta_row.assign(G + 1, (int)N);
    int q = 0;
    for (int c = 0; c < G; c++) {
      const int64_t goal = (N * (int64_t)c) / G;
      while (q < np && S.pieces[q].x + S.pieces[q].y <= goal) q++;
      cta_piece[c] = std::min(q, np);
      S.cta_row[c] = c == 0 ? 0 : (q < np ? S.pieces[q].x : (int)N);
    }
    S.cta_row[0] = 0;
    cta_piece[0] = 0;
    for (int c = 1; c <= G; c++) {
      S.cta_row[c] = std::max(S.cta_row[c], S.cta_row[c - 1]);
      cta_piece[c] = std::max(cta_piece[c], cta_piece[c - 1]);
    }
    S.cta_row[G] = (int)N;
    cta_piece[G] = np;
    S.cta_tile.assign(G + 1, 0);
    for (int c = 0; c < G; c++) {
      S.cta_tile[c] = (int)S.tiles.size();
      make_tiles(S.pieces, cta_piece[c], cta_piece[c + 1], S.tile_rows, S.tiles);
    }
    S.cta_tile[G] = (int)S.tiles.size();
    S.grid_blocks = G;
  } else {
    S.order.resize(ni);
    for (int32_t i = 0; i < ni; i++) S.order[i] = i;
    std::stable_sort(S.order.begin(), S.order.end(),
                     [&](int a, int b) { return host.num_elem[a] > host.num_elem[b]; });
    int per_sm = 0;
    auto kern = mixed ? implicit_steps<float, false> : implicit_steps<double, false>;
    NRT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S.smem));
    NRT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, S.smem));
    // persistent CTAs: as many per SM as fit, or at most tile_ctas_per_sm (a tuned shape;
    // each instance is one CTA's from start to end, so results do not depend on it)
    if (opt.tile_ctas_per_sm > 0) per_sm = std::min(per_sm, opt.tile_ctas_per_sm);
    S.grid_blocks = std::max(1, std::min<int>(dev_sms * std::max(per_sm, 1), ni));
    S.inst_tile.assign(ni + 1, 0);
    for (int32_t i = 0; i < ni; i++) {
      S.inst_tile[i] = (int)S.tiles.size();
      make_tiles(S.pieces, inst_piece[i], inst_piece[i + 1], S.tile_rows, S.tiles);
    }
    S.inst_tile[ni] = (int)S.tiles.size();
  }
  S.tiles.push_back(np);  // sentinel: end piece of the last tile
  const bool tree = opt.precond == NRT_PRECOND_TREE;
  S.iv.local_top = -1;
  if (tree) {
    // staging slots: three T rows, the slot row and the slot flag per slot
    S.iv.tree_cap = (int)(kTileBytes / (3 * tb + 5)) & ~15;
    if (S.grid_mode)
      build_tree_schedule(host, S.iv.tree_cap, true, S.grid_blocks, S.tree);
    else
      build_tree_schedule_batch(host, S.iv.tree_cap, S.tree);
    S.iv.local_top = S.tree.local_top;
  }
  // device bytes, in the order implicit_init takes them
  const int m = opt.restart;
  size_t b = 0;
  b += al256(N);                                            // rowf
  b += 5 * al256(8 * N);                                    // cmdt, g64, wdx64, kdx64, inp64
  b += 2 * al256(8 * N);                                    // diag, rhs
  b += al256(4 * N) + al256(tb * N);                        // gf, cdiag
  b += 2 * al256(tb * N * (m + 1)) + 3 * al256(tb * N);     // Wb, Z, y, pd, pc
  b += al256(sizeof(int2) * std::max<size_t>(1, S.pieces.size()));
  b += al256(4 * S.tiles.size());
  if (S.grid_mode)
    b += al256(4 * S.cta_row.size()) + al256(4 * S.cta_tile.size());
  else
    b += al256(4 * S.inst_tile.size()) + al256(4 * S.order.size());
  b += al256(8 * S.inst_row.size()) + 2 * al256(4) + al256(sizeof(double) * 2 * 4096 * kMaxDots);
  b += al256(sizeof(InstStat) * ni) + al256(sizeof(PackView)) + al256(sizeof(ImView));
  if (tree) {
    const TreeSchedule &T = S.tree;
    const size_t ns = T.slot_row.size(), nseg = std::max<size_t>(1, T.seg_len.size());
    b += 5 * al256(4 * nseg);                               // seg_len, c1, c2, prow, soff
    b += al256(4 * T.tile_seg.size()) + al256(4 * T.tile_slot.size()) + al256(4 * ns) + al256(ns);
    b += al256(4 * T.lev_tile.size()) + al256(4 * T.work_lev.size());
    b += 4 * al256(tb * ns);                                // sg, sinv, se, sy
    b += 2 * al256(tb * nseg);                              // exp_d, exp_b
  }
  bytes = b + 4096;
  return NRT_OK;
}

int Engine::implicit_init() {
  ImplicitState &S = *im;
  const int64_t N = host.ntot;
  const int32_t ni = host.ninst;
  const bool mixed = opt.precision == NRT_MIXED;
  const size_t tb = mixed ? 4 : 8;
  NRT_CUDA(cudaMemcpyAsync((void *)pv.topo, host.topo.data(), sizeof(Topo) * N,
                           cudaMemcpyHostToDevice, stream));
  cudaStream_t st = stream;
  ImView &iv = S.iv;
  iv.ntot = N;
  iv.m = opt.restart;
  iv.precond = opt.precond;
  iv.krylov = opt.krylov;
  iv.scheme = opt.scheme;
  iv.tol_mode = opt.tol_mode;
  iv.tol = opt.tol;
  iv.max_iter = opt.max_iter;
  iv.inner_rel = !mixed ? 0.0 : (opt.inner_tol > 0 ? opt.inner_tol : NRT_INNER_TOL_DEFAULT);
  iv.rich = mixed && opt.precond == NRT_PRECOND_TREE && opt.krylov == NRT_GMRES &&
            opt.refinement == 0;
  iv.ninst = ni;
  iv.tile_rows = S.tile_rows;
  uint8_t *pr;
  TRYI(up(arena, pr, S.rowf.data(), N, st)); iv.rowf = pr;
  // c_m dX / dT and the FP32 conductances are staged (filled in parallel, no zero fill
  // first); the other FP64 rows go up straight from the host pack
  std::unique_ptr<double[]> cmdt_b(new double[N]);
  std::unique_ptr<float[]> gf_b(new float[N]);
  double *cmdt = cmdt_b.get();
  float *gf = gf_b.get();
  parallel_ranges(N, [&](int64_t a, int64_t b) {
    for (int64_t j = a; j < b; j++) {
      cmdt[j] = host.c_m_dx[j] / host.inst[host.topo[j].flags >> INST_SHIFT].dT;
      gf[j] = (float)host.gax[j];
    }
  });
  double *p;
  TRYI(up(arena, p, cmdt, N, st)); iv.cmdt = p;
  TRYI(up(arena, p, host.gax.data(), N, st)); iv.g64 = p;
  TRYI(up(arena, p, host.wdx.data(), N, st)); iv.wdx64 = p;
  TRYI(up(arena, p, host.kdx.data(), N, st)); iv.kdx64 = p;
  TRYI(up(arena, p, host.inp.data(), N, st)); iv.inp64 = p;
  TRYI(up(arena, iv.diag, (const double *)nullptr, N, st));
  TRYI(up(arena, iv.rhs, (const double *)nullptr, N, st));
  float *pf;
  TRYI(up(arena, pf, gf, N, st)); iv.gf = pf;
  iv.cdiag = arena.take(tb * N);
  if (!iv.cdiag) {
    set_error("arena exhausted");
    return NRT_ENOMEM;
  }
  const int m = opt.restart;
  iv.Wb = arena.take(tb * N * (m + 1));
  iv.Z = arena.take(tb * N * (m + 1));
  iv.yv = arena.take(tb * N);
  iv.pcd = arena.take(tb * N);
  iv.pcc = arena.take(tb * N);
  if (!iv.Wb || !iv.Z || !iv.yv || !iv.pcd || !iv.pcc) {
    set_error("arena exhausted (Krylov workspace)");
    return NRT_ENOMEM;
  }
  NRT_CUDA(cudaMemsetAsync(iv.Wb, 0, tb * N * (m + 1), st));
  NRT_CUDA(cudaMemsetAsync(iv.Z, 0, tb * N * (m + 1), st));
  NRT_CUDA(cudaMemsetAsync(iv.yv, 0, tb * N, st));
  int2 *pc;
  TRYI(up(arena, pc, S.pieces.data(), S.pieces.size(), st)); iv.pieces = pc;
  int *pi;
  TRYI(up(arena, pi, S.tiles.data(), S.tiles.size(), st)); iv.tiles = pi;
  if (S.grid_mode) {
    TRYI(up(arena, pi, S.cta_row.data(), S.cta_row.size(), st)); iv.cta_row = pi;
    TRYI(up(arena, pi, S.cta_tile.data(), S.cta_tile.size(), st)); iv.cta_tile = pi;
  } else {
    TRYI(up(arena, pi, S.inst_tile.data(), S.inst_tile.size(), st)); iv.inst_tile = pi;
    TRYI(up(arena, pi, S.order.data(), S.order.size(), st)); iv.order = pi;
  }
  int64_t *pl;
  TRYI(up(arena, pl, S.inst_row.data(), S.inst_row.size(), st)); iv.inst_row = pl;
  TRYI(up(arena, iv.queue, (const int *)nullptr, 1, st));
  TRYI(up(arena, iv.err, (const int *)nullptr, 1, st));
  NRT_CUDA(cudaMemsetAsync(iv.err, 0, sizeof(int), st));
  TRYI(up(arena, iv.partials, (const double *)nullptr, (size_t)2 * 4096 * kMaxDots, st));
  std::vector<InstStat> zero(ni, InstStat{0, 0, 0, 0.0, 0, 0, 0, 0, 0});
  TRYI(up(arena, iv.stats, zero.data(), ni, st));
  iv.work_lev = nullptr;
  std::vector<char> sgbuf;
  if (opt.precond == NRT_PRECOND_TREE) {
    const TreeSchedule &T = S.tree;
    const size_t ns = T.slot_row.size(), nseg = std::max<size_t>(1, T.seg_len.size());
    TRYI(up(arena, pi, T.seg_len.data(), T.seg_len.size(), st)); iv.seg_len = pi;
    TRYI(up(arena, pi, T.seg_c1.data(), T.seg_c1.size(), st)); iv.seg_c1 = pi;
    TRYI(up(arena, pi, T.seg_c2.data(), T.seg_c2.size(), st)); iv.seg_c2 = pi;
    TRYI(up(arena, pi, T.seg_prow.data(), T.seg_prow.size(), st)); iv.seg_prow = pi;
    TRYI(up(arena, pi, T.seg_soff.data(), T.seg_soff.size(), st)); iv.seg_soff = pi;
    TRYI(up(arena, pi, T.tile_seg.data(), T.tile_seg.size(), st)); iv.tile_seg = pi;
    TRYI(up(arena, pi, T.tile_slot.data(), T.tile_slot.size(), st)); iv.tile_slot = pi;
    TRYI(up(arena, pi, T.slot_row.data(), ns, st)); iv.srow = pi;
    uint8_t *pf8;
    TRYI(up(arena, pf8, T.slot_flag.data(), ns, st)); iv.sflag = pf8;
    TRYI(up(arena, pi, T.lev_tile.data(), T.lev_tile.size(), st)); iv.lev_tile = pi;
    TRYI(up(arena, pi, T.work_lev.data(), T.work_lev.size(), st)); iv.work_lev = pi;
    // static per-slot conductance to the mother (0 on a row without that column)
    sgbuf.resize(tb * ns);
    parallel_ranges((int64_t)ns, [&](int64_t a, int64_t b) {
      for (int64_t k = a; k < b; k++) {
        const int r = T.slot_row[k];
        const double g = (r >= 0 && (host.topo[r].flags & F_UP)) ? host.gax[r] : 0.0;
        if (mixed)
          ((float *)sgbuf.data())[k] = (float)g;
        else
          ((double *)sgbuf.data())[k] = g;
      }
    });
    void *sgd = arena.take(tb * ns);
    iv.sinv = arena.take(tb * ns);
    iv.se = arena.take(tb * ns);
    iv.sy = arena.take(tb * ns);
    iv.exp_d = arena.take(tb * nseg);
    iv.exp_b = arena.take(tb * nseg);
    if (!iv.cdiag || !sgd || !iv.sinv || !iv.se || !iv.sy || !iv.exp_d || !iv.exp_b) {
      set_error("arena exhausted (tree preconditioner)");
      return NRT_ENOMEM;
    }
    NRT_CUDA(cudaMemcpyAsync(sgd, sgbuf.data(), tb * ns, cudaMemcpyHostToDevice, st));
    iv.sg = sgd;
    NRT_CUDA(cudaMemsetAsync(iv.sinv, 0, tb * ns, st));
    NRT_CUDA(cudaMemsetAsync(iv.se, 0, tb * ns, st));
    NRT_CUDA(cudaMemsetAsync(iv.sy, 0, tb * ns, st));
  }
  S.d_pv = (PackView *)arena.take(sizeof(PackView));
  S.d_iv = (ImView *)arena.take(sizeof(ImView));
  if (!S.d_pv || !S.d_iv) {
    set_error("arena exhausted (views)");
    return NRT_ENOMEM;
  }
  NRT_CUDA(cudaMemcpyAsync(S.d_pv, &pv, sizeof(PackView), cudaMemcpyHostToDevice, st));
  NRT_CUDA(cudaMemcpyAsync(S.d_iv, &iv, sizeof(ImView), cudaMemcpyHostToDevice, st));
  NRT_CUDA(cudaStreamSynchronize(st));
  return NRT_OK;
}

// Runs `nsteps` implicit steps for every instance (one launch).
static int implicit_launch(Engine &e, int nsteps, int force) {
  ImplicitState &S = *e.im;
  NRT_CUDA(cudaMemsetAsync(S.iv.queue, 0, sizeof(int), e.stream));
  const PackView *pv = S.d_pv;
  const ImView *iv = S.d_iv;
  double *V0 = e.V[0], *V1 = e.V[1];
  int cur = e.cur;
  // the drop-in per-call loop (force >= 0) has no device loop index: it is not recorded
  const RecView *rec = force < 0 ? e.record_view() : nullptr;
  void *args[] = {&pv, &iv, &nsteps, &force, &V0, &V1, &cur, &rec};
  const bool mixed = e.opt.precision == NRT_MIXED;
  if (S.grid_mode) {
    const void *k = mixed ? (const void *)implicit_steps<float, true> : (const void *)implicit_steps<double, true>;
    NRT_CUDA(cudaLaunchCooperativeKernel(k, dim3(S.grid_blocks), dim3(kThreads), args, S.smem, e.stream));
  } else {
    const void *k = mixed ? (const void *)implicit_steps<float, false> : (const void *)implicit_steps<double, false>;
    NRT_CUDA(cudaLaunchKernel(k, dim3(S.grid_blocks), dim3(kThreads), args, S.smem, e.stream));
  }
  count_launch_on(e.stream);
  return NRT_OK;
}

int Engine::implicit_step(int k, int force) {
  (void)k;
  return implicit_launch(*this, 1, force);
}

int implicit_advance(Engine &e, int64_t steps) {
  const int chunk = 64;
  while (steps > 0) {
    const int n = (int)std::min<int64_t>(chunk, steps);
    TRYI(implicit_launch(e, n, -1));
    TRYI(launch_advance_base(e.pv.inst, e.pv.ninst, n, e.stream));
    if (n & 1) e.cur ^= 1;
    e.steps_done += n;
    steps -= n;
  }
  return NRT_OK;
}

int instance_stats(Engine &e, int64_t *iters, int32_t *last_iters, int32_t *nonconv,
                   double *last_res) {
  const int32_t ni = e.host.ninst;
  std::vector<InstStat> s(ni, InstStat{0, 0, 0, 0.0, 0, 0, 0, 0, 0});
  if (e.im) {
    NRT_CUDA(cudaMemcpyAsync(s.data(), e.im->iv.stats, sizeof(InstStat) * ni,
                             cudaMemcpyDeviceToHost, e.stream));
    NRT_CUDA(cudaStreamSynchronize(e.stream));
  }
  for (int32_t i = 0; i < ni; i++) {
    if (iters) iters[i] = s[i].iters;
    if (last_iters) last_iters[i] = s[i].last_iters;
    if (nonconv) nonconv[i] = s[i].nonconv;
    if (last_res) last_res[i] = s[i].last_res;
  }
  return NRT_OK;
}

int pass_counts(Engine &e, int64_t *residuals, int64_t *applies, int64_t *xupdates,
                int64_t *basis, int64_t *rich) {
  const int32_t ni = e.host.ninst;
  std::vector<InstStat> s(ni, InstStat{0, 0, 0, 0.0, 0, 0, 0, 0, 0});
  if (e.im) {
    NRT_CUDA(cudaMemcpyAsync(s.data(), e.im->iv.stats, sizeof(InstStat) * ni,
                             cudaMemcpyDeviceToHost, e.stream));
    NRT_CUDA(cudaStreamSynchronize(e.stream));
  }
  for (int32_t i = 0; i < ni; i++) {
    if (residuals) residuals[i] = s[i].residuals;
    if (applies) applies[i] = s[i].applies;
    if (xupdates) xupdates[i] = s[i].xupdates;
    if (basis) basis[i] = s[i].basis;
    if (rich) rich[i] = s[i].rich;
  }
  return NRT_OK;
}

// NRT_EDEVICE when a kernel's bounded wait gave up (an error word is set); synchronises.
int implicit_check(Engine &e) {
  int err[2] = {0, 0};
  if (e.im)
    NRT_CUDA(cudaMemcpyAsync(&err[0], e.im->iv.err, sizeof(int), cudaMemcpyDeviceToHost, e.stream));
  if (e.pv.err)
    NRT_CUDA(cudaMemcpyAsync(&err[1], e.pv.err, sizeof(int), cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaStreamSynchronize(e.stream));
  if (err[0] || err[1]) {
    set_error(err[0] ? "implicit kernel: a bounded wait for its tile copies expired"
                     : "explicit step: a bounded wait for its tile copies expired");
    return NRT_EDEVICE;
  }
  return NRT_OK;
}

// Sum of non-converged steps over all instances (-1 on a device error).
int64_t nonconverged_total(Engine &e) {
  if (!e.im) return 0;
  if (implicit_check(e) != NRT_OK) return -1;
  std::vector<InstStat> s(e.host.ninst);
  if (cudaMemcpyAsync(s.data(), e.im->iv.stats, sizeof(InstStat) * e.host.ninst,
                      cudaMemcpyDeviceToHost, e.stream) != cudaSuccess ||
      cudaStreamSynchronize(e.stream) != cudaSuccess)
    return -1;
  int64_t t = 0;
  for (const InstStat &x : s) t += x.nonconv;
  return t;
}

void Engine::implicit_release() {
  delete im;
  im = nullptr;
}

int Engine::get_stats(nrt_stats *st) {
  memset(st, 0, sizeof(*st));
  st->steps = steps_done;
  st->device_bytes = (int64_t)arena.cap;
  if (opt.mode == NRT_IMPLICIT_BE && im) {
    std::vector<InstStat> s(host.ninst);
    NRT_CUDA(cudaMemcpyAsync(s.data(), im->iv.stats, sizeof(InstStat) * host.ninst,
                             cudaMemcpyDeviceToHost, stream));
    NRT_CUDA(cudaStreamSynchronize(stream));
    for (const InstStat &x : s) {
      st->krylov_iters += x.iters;
      st->nonconverged_steps += x.nonconv;
      st->last_iters = std::max(st->last_iters, x.last_iters);
      st->last_residual = std::max(st->last_residual, x.last_res);
    }
  }
  return NRT_OK;
}

// Expands the stored symmetric system to the reference's CSR (src/solverIm-cpu.cpp:29-183
// column order: mother, diagonal, DR, DL; identity rows 1).  Runs an assembly-only pass
// for the next step and restores the state it touched.
int export_system(Engine &e, int input_active, int32_t *row_ptr, int32_t *col, double *val,
                  double *rhs, int32_t *nnz_out) {
  if (e.opt.mode != NRT_IMPLICIT_BE || e.host.ninst != 1) {
    set_error("export_system needs a single-tree implicit solver");
    return NRT_EINVAL;
  }
  const int64_t N = e.host.ntot;
  const bool mixed = e.opt.precision == NRT_MIXED;
  const size_t gb = (mixed ? 4 : 8) * 3 * N;
  void *gate = mixed ? (void *)e.pv.gatef : (void *)e.pv.gate;
  std::vector<char> saved(gb);
  std::vector<double> Vother(N);
  ImplicitState &S = *e.im;
  InstStat stat0;
  NRT_CUDA(cudaMemcpyAsync(saved.data(), gate, gb, cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaMemcpyAsync(Vother.data(), e.V[e.cur ^ 1], 8 * N, cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaMemcpyAsync(&stat0, S.iv.stats, sizeof(InstStat), cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaStreamSynchronize(e.stream));
  const int saved_iter = S.iv.max_iter;
  S.iv.max_iter = -1;  // assembly only
  NRT_CUDA(cudaMemcpyAsync(S.d_iv, &S.iv, sizeof(ImView), cudaMemcpyHostToDevice, e.stream));
  int rc = implicit_launch(e, 1, input_active ? 1 : 0);
  S.iv.max_iter = saved_iter;
  const cudaError_t ce = cudaMemcpyAsync(S.d_iv, &S.iv, sizeof(ImView), cudaMemcpyHostToDevice, e.stream);
  if (rc) return rc;
  NRT_CUDA(ce);
  std::vector<double> diag(N), rh(N), g(N);
  NRT_CUDA(cudaMemcpyAsync(diag.data(), S.iv.diag, 8 * N, cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaMemcpyAsync(rh.data(), S.iv.rhs, 8 * N, cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaMemcpyAsync(g.data(), S.iv.g64, 8 * N, cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaMemcpyAsync(gate, saved.data(), gb, cudaMemcpyHostToDevice, e.stream));
  NRT_CUDA(cudaMemcpyAsync(e.V[e.cur ^ 1], Vother.data(), 8 * N, cudaMemcpyHostToDevice, e.stream));
  NRT_CUDA(cudaMemcpyAsync(S.iv.stats, &stat0, sizeof(InstStat), cudaMemcpyHostToDevice, e.stream));
  NRT_CUDA(cudaStreamSynchronize(e.stream));
  int32_t nnz = 0;
  for (int64_t j = 0; j < N; j++) {
    const Topo &t = e.host.topo[j];
    row_ptr[j] = nnz;
    if (t.flags & F_IDENT) {
      col[nnz] = (int32_t)j;
      val[nnz++] = 1.0;
      rhs[j] = Vother[j];
      continue;
    }
    if (t.flags & F_UP) { col[nnz] = t.mother; val[nnz++] = -g[j]; }
    col[nnz] = (int32_t)j;
    val[nnz++] = diag[j];
    if (t.flags & F_DOWNR) { col[nnz] = (int32_t)j + 1; val[nnz++] = -g[j + 1]; }
    if (t.flags & F_DOWNL) { col[nnz] = t.dl; val[nnz++] = -g[t.dl]; }
    rhs[j] = rh[j];
  }
  row_ptr[N] = nnz;
  *nnz_out = nnz;
  return NRT_OK;
}

}  // namespace nrt
