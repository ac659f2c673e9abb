// Implicit (backward Euler) path: assembly + preconditioned GMRES(m), one persistent
// kernel per chunk of time steps.
//
// Replaces SolverImGPU::update / ::calculate (src/solverIm-gpu.cpp:687-843: Update_HH,
// Update_Mat, Update_B, then BiCGSTAB over cuSPARSE csrmv and cuBLAS dot/axpy with a
// host sync every 30 iterations) and computes the system of SolverImCPU::createMatrix
// (src/solverIm-cpu.cpp:29-183):
//
//   row j (physical):  -g_j V_mother + d_j V_j - g_DR V_DR - b_j g_DL V_DL = rhs_j
//   d_j   = c_m dX/dT - W dX + b_j g_DL + [DR column] g_DR + [mother column] g_j
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
// rotations.  The preconditioner is an exact tridiagonal (Thomas) solve of every
// unbranched segment piece (<= kMaxPiece rows): only the branch-point couplings are left
// to the Krylov iteration.  Each cycle starts from the true FP64 residual b - A x, so in
// mixed precision (FP32 basis, SpMV, orthogonalisation update and preconditioner) every
// restart is one step of iterative refinement.  Inner products and norms: per-thread
// partial sums in the basis precision over the thread's rows, then FP64 across threads
// and CTAs in a fixed order (deterministic, identical in every CTA).  Warm start x0 = V^n.
//
// Memory-level parallelism: the SpMV is fused with all j+1 Gram-Schmidt products (one
// pass over the rows, register accumulators), the update and the norm share a pass, and
// the sequential Thomas sweeps run on tiles of rows staged in shared memory.
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
#include <vector>

#include "hh.cuh"
#include "nrt_solver.h"

namespace cg = cooperative_groups;

namespace nrt {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxPiece = 256;                 // longest segment piece one sweep handles
constexpr int kMaxDots = kMaxRestart + 1;
constexpr int kTileBytes = 48 * 1024;          // shared-memory staging for the sweeps
constexpr int kU = 4;                          // rows per thread kept in flight in row loops

struct InstStat {
  int64_t iters;
  int32_t last_iters;
  int32_t nonconv;
  double last_res;
};

struct ImView {
  int64_t ntot;
  int m;             // restart
  int precond;
  int tol_mode;
  double tol;
  int max_iter;      // per step per instance; 0 -> instance size; < 0 -> assembly only
  int ninst;
  int tile_rows;     // rows per shared-memory tile
  const double *cmdt;  // c_m dX / dT
  const double *g64;   // 1 / (r_a dX)
  const float *gf;
  const double *wdx64, *kdx64, *inp64;
  double *diag;
  float *diagf;
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
  // exact tree preconditioner (NRT_PRECOND_TREE): segments in tile order
  const int *seg_len, *seg_c1, *seg_c2, *seg_prow, *seg_soff;
  const int *tile_seg;            // segments of tree tile q: [tile_seg[q], tile_seg[q+1])
  const int *tile_slot;           // staging slots of tree tile q
  const int *slot_row;            // global row behind each staging slot
  const int *lev_tile;            // tree tiles of level entry e: [lev_tile[e], lev_tile[e+1])
  const int *work_lev;            // level entries of a worker (CTA or instance), deepest first
  void *tinv;                     // T[ntot]: 1 / (eliminated pivot) per row
  double *exp_d;                  // per segment: g^2 / pivot exported to the parent row
  void *exp_b;                    // T per segment: g b' / pivot exported to the parent row
  int tree_cap;                   // staging slots per tree tile
};

template <typename T>
struct Work {
  T *Wb, *Z, *y, *pd, *pc;
};

struct Shared {
  double *H, *cs, *sn, *g, *s, *y, *red, *warp;
  void *coef;      // T[kMaxDots]: update / solution coefficients
  int *flag;
  void *tile;      // staging area
};

__host__ __device__ inline size_t shared_fixed_bytes(int m) {
  return sizeof(double) * ((size_t)(m + 1) * m + 2 * m + 2 * (m + 1) + m + kMaxDots +
                           kWarps * kMaxDots + kMaxDots) + 16;
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
  S.tile = (void *)((char *)base + ((shared_fixed_bytes(m) + 127) & ~(size_t)127));
  return S;
}

// ---------------------------------------------------------------- reductions

// Reduces the first k register accumulators of every thread over the CTA into out[0..k)
// (FP64, fixed order: warp shuffle tree, then warps in index order).
template <typename T>
__device__ __forceinline__ void block_reduce(const T (&acc)[kMaxDots], int k, double *warp_part,
                                             double *out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < kMaxDots; i++) {
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

template <bool kGrid, typename T>
__device__ __forceinline__ void group_reduce(cg::grid_group &grid, const T (&acc)[kMaxDots], int k,
                                             Shared &S, double *partials, int &parity) {
  block_reduce(acc, k, S.warp, S.red);
  if (kGrid) grid_finish(grid, k, S.red, partials, parity);
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

// ---------------------------------------------------------------- kernel body

template <typename T, bool kGrid>
struct Ctx {
  PackView pv;
  ImView iv;
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
  } else {
    __syncthreads();
  }
}

// Exact tree factorisation (Hines elimination order, leaves to root): for every segment,
// the parent rows' pivots absorb g^2 / pivot of their child segments; one thread per
// segment, the segments of one level at a time, staged in shared memory.
template <typename T, bool kGrid>
__device__ void tree_factor(Ctx<T, kGrid> &c, cg::grid_group &grid, Shared &S) {
  const ImView &iv = c.iv;
  double *sd = (double *)S.tile;
  double *sg = sd + iv.tree_cap;
  T *tinv = (T *)iv.tinv;
  for (int e = c.l0; e < c.l1; e++) {
    for (int q = iv.lev_tile[e]; q < iv.lev_tile[e + 1]; q++) {
      const int s0 = iv.tile_slot[q], s1 = iv.tile_slot[q + 1];
      for (int k = s0 + threadIdx.x; k < s1; k += blockDim.x) {
        const int r = iv.slot_row[k];
        sd[k - s0] = iv.diag[r];
        sg[k - s0] = iv.g64[r];
      }
      __syncthreads();
      for (int s = iv.tile_seg[q] + threadIdx.x; s < iv.tile_seg[q + 1]; s += blockDim.x) {
        const int o = iv.seg_soff[s], L = iv.seg_len[s];
        double d = sd[o + L - 1];
        if (iv.seg_c1[s] >= 0) d -= iv.exp_d[iv.seg_c1[s]];
        if (iv.seg_c2[s] >= 0) d -= iv.exp_d[iv.seg_c2[s]];
        for (int k = L - 1; k >= 1; k--) {
          const double inv = 1.0 / d;
          sd[o + k] = inv;
          const double gk = sg[o + k];
          d = sd[o + k - 1] - gk * gk * inv;
        }
        const double inv0 = 1.0 / d;
        sd[o] = inv0;
        iv.exp_d[s] = iv.seg_prow[s] >= 0 ? sg[o] * sg[o] * inv0 : 0.0;
      }
      __syncthreads();
      for (int k = s0 + threadIdx.x; k < s1; k += blockDim.x) tinv[iv.slot_row[k]] = (T)sd[k - s0];
      __syncthreads();
    }
    level_sync<kGrid>(grid);
  }
}

// z = A^-1 v (up to rounding) with the factors of tree_factor: elimination of every
// segment into its parent row, leaves to root, then back-substitution root to leaves.
template <typename T, bool kGrid>
__device__ void tree_apply(Ctx<T, kGrid> &c, cg::grid_group &grid, Shared &S, const T *v, T *z) {
  const ImView &iv = c.iv;
  T *sb = (T *)S.tile;
  T *si = sb + iv.tree_cap;
  T *sg = si + iv.tree_cap;
  const T *tinv = (const T *)iv.tinv;
  const T *g = sizeof(T) == 4 ? (const T *)(const void *)iv.gf : (const T *)(const void *)iv.g64;
  T *exp_b = (T *)iv.exp_b;
  for (int pass = 0; pass < 2; pass++) {
    for (int ee = 0; ee < c.l1 - c.l0; ee++) {
      const int e = pass == 0 ? c.l0 + ee : c.l1 - 1 - ee;  // deepest first, then root first
      for (int q = iv.lev_tile[e]; q < iv.lev_tile[e + 1]; q++) {
        const int s0 = iv.tile_slot[q], s1 = iv.tile_slot[q + 1];
        for (int k = s0 + threadIdx.x; k < s1; k += blockDim.x) {
          const int r = iv.slot_row[k];
          sb[k - s0] = pass == 0 ? v[r] : z[r];
          si[k - s0] = tinv[r];
          sg[k - s0] = g[r];
        }
        __syncthreads();
        for (int s = iv.tile_seg[q] + threadIdx.x; s < iv.tile_seg[q + 1]; s += blockDim.x) {
          const int o = iv.seg_soff[s], L = iv.seg_len[s];
          if (pass == 0) {
            T b = sb[o + L - 1];
            if (iv.seg_c1[s] >= 0) b += exp_b[iv.seg_c1[s]];
            if (iv.seg_c2[s] >= 0) b += exp_b[iv.seg_c2[s]];
            sb[o + L - 1] = b;
            for (int k = L - 1; k >= 1; k--) {
              b = sb[o + k - 1] + sg[o + k] * b * si[o + k];
              sb[o + k - 1] = b;
            }
            exp_b[s] = iv.seg_prow[s] >= 0 ? sg[o] * sb[o] * si[o] : (T)0;
          } else {
            const int pr = iv.seg_prow[s];
            T x = (sb[o] + (pr >= 0 ? sg[o] * z[pr] : (T)0)) * si[o];
            sb[o] = x;
            for (int k = 1; k < L; k++) {
              x = (sb[o + k] + sg[o + k] * x) * si[o + k];
              sb[o + k] = x;
            }
          }
        }
        __syncthreads();
        for (int k = s0 + threadIdx.x; k < s1; k += blockDim.x) z[iv.slot_row[k]] = sb[k - s0];
        __syncthreads();
      }
      level_sync<kGrid>(grid);
    }
  }
}

// (A x)_j for a physical row, FP64 (identity rows yield 0).
__device__ __forceinline__ double row_apply64(const PackView &pv, const ImView &iv, int64_t j,
                                              const double *x) {
  const Topo t = pv.topo[j];
  if (t.flags & F_IDENT) return 0.0;
  double s = iv.diag[j] * x[j];
  if (t.flags & F_UP) s -= iv.g64[j] * x[t.mother];
  if (t.flags & F_DOWNR) s -= iv.g64[j + 1] * x[j + 1];
  if (t.flags & F_DOWNL) s -= iv.g64[t.dl] * x[t.dl];
  return s;
}

template <typename T>
__device__ __forceinline__ T row_apply(const PackView &pv, const ImView &iv, int64_t j, const T *x);

template <>
__device__ __forceinline__ double row_apply<double>(const PackView &pv, const ImView &iv, int64_t j,
                                                    const double *x) {
  return row_apply64(pv, iv, j, x);
}

template <>
__device__ __forceinline__ float row_apply<float>(const PackView &pv, const ImView &iv, int64_t j,
                                                  const float *x) {
  const Topo t = pv.topo[j];
  if (t.flags & F_IDENT) return 0.0f;
  float s = iv.diagf[j] * x[j];
  if (t.flags & F_UP) s = fmaf(-iv.gf[j], x[t.mother], s);
  if (t.flags & F_DOWNR) s = fmaf(-iv.gf[j + 1], x[j + 1], s);
  if (t.flags & F_DOWNL) s = fmaf(-iv.gf[t.dl], x[t.dl], s);
  return s;
}

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
__device__ void factor_pieces(Ctx<T, kGrid> &c, Shared &S) {
  T *sd = (T *)S.tile;                          // diag, then pivots^-1
  T *sg = sd + c.iv.tile_rows;                  // conductance to the mother
  T *sc = sg + c.iv.tile_rows;                  // c'
  for (int q = c.t0; q < c.t1; q++) {
    int64_t a, b;
    tile_rows(c.iv, q, a, b);
    for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
      sd[r - a] = (T)c.iv.diag[r];
      sg[r - a] = (T)c.iv.g64[r];
    }
    __syncthreads();
    for (int p = c.iv.tiles[q] + threadIdx.x; p < c.iv.tiles[q + 1]; p += blockDim.x) {
      const int2 pc = c.iv.pieces[p];
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
__device__ void apply_precond(Ctx<T, kGrid> &c, cg::grid_group &grid, Shared &S, const T *v, T *z) {
  if (c.iv.precond == NRT_PRECOND_TREE) {
    level_sync<kGrid>(grid);  // v of every row visible (tree tiles span other CTAs' rows)
    tree_apply(c, grid, S, v, z);
  } else if (c.iv.precond == NRT_PRECOND_SEGMENT) {
    T *sv = (T *)S.tile;
    T *sd = sv + c.iv.tile_rows;
    T *sc = sd + c.iv.tile_rows;
    T *sg = sc + c.iv.tile_rows;
    for (int q = c.t0; q < c.t1; q++) {
      int64_t a, b;
      tile_rows(c.iv, q, a, b);
      for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) {
        sv[r - a] = v[r];
        sd[r - a] = c.w.pd[r];
        sc[r - a] = c.w.pc[r];
        sg[r - a] = (T)c.iv.g64[r];
      }
      __syncthreads();
      for (int p = c.iv.tiles[q] + threadIdx.x; p < c.iv.tiles[q + 1]; p += blockDim.x) {
        const int2 pc = c.iv.pieces[p];
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
      const uint32_t f = c.pv.topo[j].flags;
      if (f & F_IDENT) {
        z[j] = 0;
        continue;
      }
      z[j] = c.iv.precond == NRT_PRECOND_JACOBI ? (T)((double)v[j] / c.iv.diag[j]) : v[j];
    }
    __syncthreads();
  }
}

// One backward-Euler step of one group (CTA or grid) for instance `inst`.
template <typename T, bool kGrid>
__device__ void implicit_one_step(Ctx<T, kGrid> &c, cg::grid_group &grid, Shared &S, int &parity,
                                  const double *Vin, double *Vout, bool active, int64_t inst_n,
                                  int inst) {
  const PackView &pv = c.pv;
  const ImView &iv = c.iv;
  const int64_t N = pv.ntot;
  const int m = iv.m;
  T *coef = (T *)S.coef;
  // ---- assembly: gates (from V^n), W, K, diagonal, right-hand side, x0 = V^n
  double bacc = 0;
  for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x) {
    const Topo t = pv.topo[j];
    const double v = Vin[j];
    double wdx, kdx;
    if (t.flags & F_HH) {
      if (pv.hpf) {
        const float *hp = pv.hpf;
        const float dv = (float)(v - (double)hp[HP_REST * N + j]);
        GateStep32 g = hh_step32(dv + hp[HP_LSNA * N + j], dv + hp[HP_LSK * N + j], pv.gatef[j],
                                 pv.gatef[N + j], pv.gatef[2 * N + j], hp[HP_DTMS * N + j],
                                 hp[HP_GNA * N + j], hp[HP_GK * N + j], hp[HP_GL * N + j],
                                 hp[HP_ENA * N + j], hp[HP_EK * N + j], hp[HP_EL * N + j]);
        pv.gatef[j] = g.m;
        pv.gatef[N + j] = g.h;
        pv.gatef[2 * N + j] = g.n;
        const double dx = (double)hp[HP_DX * N + j];
        wdx = (double)g.W * dx;
        kdx = (double)g.K * dx;
      } else {
        const double *hp = pv.hp;
        GateStep64 g = hh_step64(v, pv.gate[j], pv.gate[N + j], pv.gate[2 * N + j],
                                 hp[HP_LSNA * N + j], hp[HP_LSK * N + j], hp[HP_REST * N + j],
                                 hp[HP_DTMS * N + j], hp[HP_GNA * N + j], hp[HP_GK * N + j],
                                 hp[HP_GL * N + j], hp[HP_ENA * N + j], hp[HP_EK * N + j],
                                 hp[HP_EL * N + j]);
        pv.gate[j] = g.m;
        pv.gate[N + j] = g.h;
        pv.gate[2 * N + j] = g.n;
        const double dx = hp[HP_DX * N + j];
        wdx = g.W * dx;
        kdx = g.K * dx;
      }
    } else {
      wdx = iv.wdx64[j];
      kdx = iv.kdx64[j];
    }
    if (t.flags & F_IDENT) {
      c.w.y[j] = 0;
      continue;
    }
    double d = iv.cmdt[j] - wdx;
    if (t.flags & F_DOWNL) d += iv.g64[t.dl];
    if (t.flags & F_DOWNR) d += iv.g64[j + 1];
    if (t.flags & F_UP) d += iv.g64[j];
    iv.diag[j] = d;
    if (iv.diagf) iv.diagf[j] = (float)d;
    double b = iv.cmdt[j] * v + kdx;
    if (active) b += iv.inp64[j];
    iv.rhs[j] = b;
    bacc += b * b;
    Vout[j] = 2.0 * v - Vout[j];  // x0: linear extrapolation from V^{n-1} (held in Vout)
  }
  __syncthreads();
  if (iv.precond == NRT_PRECOND_SEGMENT) {
    factor_pieces(c, S);
  } else if (iv.precond == NRT_PRECOND_TREE) {
    level_sync<kGrid>(grid);  // diagonal of every row visible before the elimination
    tree_factor(c, grid, S);
  }
  double target = iv.tol;
  {
    double acc[kMaxDots];
    acc[0] = bacc;
    group_reduce<kGrid>(grid, acc, 1, S, iv.partials, parity);  // also publishes x0
    if (iv.tol_mode == NRT_TOL_REL) target = iv.tol * sqrt(S.red[0]);
    if (!kGrid) __syncthreads();
  }
  const int budget = iv.max_iter > 0 ? iv.max_iter : (iv.max_iter < 0 ? 0 : (int)inst_n);
  const double inner_rel = sizeof(T) == 4 ? 1e-5 : 0.0;
  int iters = 0;
  double res = 0;
  bool converged = false;
  for (;;) {
    // ---- cycle start: true residual r = b - A x in FP64, W_0 = r, Z_0 = M^-1 r
    {
      double acc[kMaxDots];
      acc[0] = 0;
      for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x) {
        if (pv.topo[j].flags & F_IDENT) {
          c.w.Wb[j] = 0;
          continue;
        }
        const double r = iv.rhs[j] - row_apply64(pv, iv, j, Vout);
        c.w.Wb[j] = (T)r;
        acc[0] += r * r;
      }
      group_reduce<kGrid>(grid, acc, 1, S, iv.partials, parity);
    }
    res = sqrt(S.red[0]);
    if (res <= target) {
      converged = true;
      break;
    }
    if (iters >= budget) break;
    apply_precond(c, grid, S, c.w.Wb, c.w.Z);
    group_sync<kGrid>(grid);  // Z_0 of every row visible before the SpMV
    if (threadIdx.x == 0) {
      S.g[0] = res;
      for (int i = 1; i <= m; i++) S.g[i] = 0;
      S.s[0] = 1.0 / res;
    }
    __syncthreads();
    const double cycle_target = fmax(target, inner_rel * res);
    int k = 0;
    for (int j = 0; j < m; j++) {
      const T *Zj = c.w.Z + (size_t)j * N;
      const T sj = (T)S.s[j];
      // y = s_j A Z_j fused with p_i = <y, W_i>, i <= j
      T acc[kMaxDots];
#pragma unroll
      for (int i = 0; i < kMaxDots; i++) acc[i] = 0;
      const int64_t stride = (int64_t)blockDim.x;
      for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kU * stride) {
        T y[kU];  // kU rows per thread in flight
#pragma unroll
        for (int u = 0; u < kU; u++) {
          const int64_t r = rb + u * stride;
          y[u] = r < c.r1 ? sj * row_apply<T>(pv, iv, r, Zj) : (T)0;
        }
#pragma unroll
        for (int u = 0; u < kU; u++)
          if (rb + u * stride < c.r1) c.w.y[rb + u * stride] = y[u];
#pragma unroll
        for (int i = 0; i < kMaxDots; i++) {
          if (i <= j) {
            const T *Wi = c.w.Wb + (size_t)i * N;
#pragma unroll
            for (int u = 0; u < kU; u++)
              if (rb + u * stride < c.r1) acc[i] += y[u] * Wi[rb + u * stride];
          }
        }
      }
      group_reduce<kGrid>(grid, acc, j + 1, S, iv.partials, parity);
      if (threadIdx.x <= j) {
        const double h = S.s[threadIdx.x] * S.red[threadIdx.x];
        S.H[threadIdx.x * m + j] = h;
        coef[threadIdx.x] = (T)(h * S.s[threadIdx.x]);
      }
      __syncthreads();
      // w = y - sum_i h_ij s_i W_i -> W_{j+1}; ||w||^2; then Z_{j+1} = M^-1 w
      T *Wn = c.w.Wb + (size_t)(j + 1) * N;
      T nacc[kMaxDots];
      nacc[0] = 0;
      for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kU * stride) {
        T a[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) a[u] = rb + u * stride < c.r1 ? c.w.y[rb + u * stride] : (T)0;
#pragma unroll
        for (int i = 0; i < kMaxDots; i++) {
          if (i <= j) {
            const T ci = coef[i];
            const T *Wi = c.w.Wb + (size_t)i * N;
#pragma unroll
            for (int u = 0; u < kU; u++)
              if (rb + u * stride < c.r1) a[u] -= ci * Wi[rb + u * stride];
          }
        }
#pragma unroll
        for (int u = 0; u < kU; u++)
          if (rb + u * stride < c.r1) {
            Wn[rb + u * stride] = a[u];
            nacc[0] += a[u] * a[u];
          }
      }
      __syncthreads();
      apply_precond(c, grid, S, Wn, c.w.Z + (size_t)(j + 1) * N);
      group_reduce<kGrid>(grid, nacc, 1, S, iv.partials, parity);  // publishes Z_{j+1}
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
      if (S.flag[0] || iters >= budget) break;
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
    {
      const int64_t stride = (int64_t)blockDim.x;
      for (int64_t rb = c.r0 + threadIdx.x; rb < c.r1; rb += kU * stride) {
        T a[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) a[u] = 0;
#pragma unroll
        for (int i = 0; i < kMaxDots; i++) {
          if (i < k) {
            const T ci = coef[i];
            const T *Zi = c.w.Z + (size_t)i * N;
#pragma unroll
            for (int u = 0; u < kU; u++)
              if (rb + u * stride < c.r1) a[u] += ci * Zi[rb + u * stride];
          }
        }
#pragma unroll
        for (int u = 0; u < kU; u++) {
          const int64_t r = rb + u * stride;
          if (r < c.r1 && !(pv.topo[r].flags & F_IDENT)) Vout[r] += (double)a[u];
        }
      }
    }
    group_sync<kGrid>(grid);
  }
  if (threadIdx.x == 0 && (!kGrid || blockIdx.x == 0)) {
    InstStat &st = iv.stats[inst];
    st.iters += iters;
    st.last_iters = iters;
    st.last_res = res;
    if (!converged) st.nonconv += 1;
  }
  group_sync<kGrid>(grid);  // V^{n+1} complete before the next step reads it
}

template <typename T, bool kGrid>
__global__ void __launch_bounds__(kThreads) implicit_steps(PackView pv, ImView iv, int nsteps,
                                                           int force, double *V0, double *V1,
                                                           int cur) {
  extern __shared__ __align__(16) double smem[];
  Shared S = carve(smem, iv.m);
  cg::grid_group grid = cg::this_grid();
  int parity = 0;
  Ctx<T, kGrid> c;
  c.pv = pv;
  c.iv = iv;
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
    const InstDev in = pv.inst[0];
    const int64_t inst_n = iv.inst_row[1] - iv.inst_row[0];
    for (int s = 0; s < nsteps; s++) {
      const int64_t i = in.base + s;
      if (i >= in.iend) break;
      const bool active = force >= 0 ? force != 0
                                     : (i >= in.ion && i <= in.ioff);
      implicit_one_step<T, kGrid>(c, grid, S, parity, ((cur + s) & 1) ? V1 : V0,
                                  ((cur + s + 1) & 1) ? V1 : V0, active, inst_n, 0);
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
      const InstDev in = pv.inst[inst];
      int s = 0;
      for (; s < nsteps; s++) {
        const int64_t i = in.base + s;
        if (i >= in.iend) break;
        const bool active = force >= 0 ? force != 0
                                       : (i >= in.ion && i <= in.ioff);
        implicit_one_step<T, kGrid>(c, grid, S, parity, ((cur + s) & 1) ? V1 : V0,
                                    ((cur + s + 1) & 1) ? V1 : V0, active, c.r1 - c.r0, inst);
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

struct ImplicitState {
  ImView iv{};
  std::vector<int2> pieces;
  std::vector<int> tiles, cta_row, cta_tile, inst_tile, order;
  std::vector<int64_t> inst_row;
  int grid_blocks = 0;
  bool grid_mode = false;
  size_t smem = 0;
};

static size_t smem_bytes(int m) { return ((shared_fixed_bytes(m) + 127) & ~(size_t)127) + kTileBytes; }

size_t Engine::implicit_bytes() const {
  const int64_t N = host.ntot;
  const size_t tb = opt.precision == NRT_MIXED ? 4 : 8;
  const int m = opt.restart;
  size_t b = 0;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  b += 6 * al(8 * N);                                   // cmdt, g64, wdx64, kdx64, inp64, diag
  b += al(8 * N) + al(4 * N) + al(4 * N);               // rhs, diagf, gf
  b += 2 * al(tb * N * (m + 1)) + 3 * al(tb * N);       // Wb, Z, y, pd, pc
  b += al(8 * (N + 2)) + al(4 * (N + 2));               // pieces, tiles (upper bounds)
  b += al(4 * 4100) * 2 + al(8 * (host.ninst + 1)) + al(4 * (host.ninst + 1)) + al(4 * host.ninst);
  b += al(sizeof(double) * 2 * 4096 * kMaxDots);
  b += al(sizeof(InstStat) * host.ninst) + al(64);
  if (opt.precond == NRT_PRECOND_TREE)  // schedule arrays, factors, export slots (bounds)
    b += 12 * al(4 * (N + 8)) + al(tb * N) + al(8 * N) + al(tb * N) + al(4 * (4096 + 8));
  return b;
}

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

// Schedule of the exact tree preconditioner.  Segments are maximal runs of physical rows
// each linked to the previous row (mother == j - 1), broken after every branch point and
// at `cap` rows; a segment's parent row (the mother of its first row) is then always the
// last row of its parent segment.  Level = number of segments above.  Each worker (one
// CTA of the cooperative launch, or one instance of a batch) gets, per level (deepest
// first), tiles of whole segments whose rows fit the shared-memory staging area.
struct TreeSchedule {
  std::vector<int> seg_len, seg_c1, seg_c2, seg_prow, seg_soff;  // tile order
  std::vector<int> tile_seg, tile_slot, slot_row, lev_tile, work_lev;
};

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
    for (int L = 0; L <= max_level; L++) {
      int64_t rows = 0;
      for (int s : by_level[L]) rows += segs[s].len;
      int64_t acc = 0;
      for (int s : by_level[L]) {
        const int w = (int)std::min<int64_t>(nwork - 1, acc * nwork / std::max<int64_t>(rows, 1));
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
  T.work_lev.assign(nwork + 1, 0);
  for (int w = 0; w < nwork; w++) {
    T.work_lev[w] = (int)T.lev_tile.size();
    for (int L = (int)lists[w].size() - 1; L >= 0; L--) {
      T.lev_tile.push_back((int)T.tile_seg.size());
      int used = cap;  // forces a new tile for the first segment
      for (int s : lists[w][L]) {
        if (used + segs[s].len > cap) {
          T.tile_seg.push_back((int)order.size());
          T.tile_slot.push_back((int)T.slot_row.size());
          used = 0;
        }
        newid[s] = (int)order.size();
        order.push_back(s);
        T.seg_soff.push_back(used);
        for (int k = 0; k < segs[s].len; k++) T.slot_row.push_back(segs[s].start + k);
        used += segs[s].len;
      }
    }
  }
  T.work_lev[nwork] = (int)T.lev_tile.size();
  T.lev_tile.push_back((int)T.tile_seg.size());
  T.tile_seg.push_back((int)order.size());
  T.tile_slot.push_back((int)T.slot_row.size());
  for (int s : order) {
    const Seg &g = segs[s];
    T.seg_len.push_back(g.len);
    T.seg_prow.push_back(g.prow);
    T.seg_c1.push_back(g.c1 >= 0 ? newid[g.c1] : -1);
    T.seg_c2.push_back(g.c2 >= 0 ? newid[g.c2] : -1);
  }
}

// Groups pieces [pa, pb) into tiles whose row span fits the shared-memory staging area.
static void make_tiles(const std::vector<int2> &pieces, int pa, int pb, int tile_rows,
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

int Engine::implicit_init() {
  im = new ImplicitState();
  ImplicitState &S = *im;
  const int64_t N = host.ntot;
  const int32_t ni = host.ninst;
  // Row structure (flags) per element.  The validator guaranteed the reference
  // numbering: mother < j, DR == j + 1 off terminals, terminals follow their mother.
  std::vector<char> is_term(N, 0);
  for (int64_t t : host.terms) is_term[t] = 1;
  for (int32_t i = 0; i < ni; i++) {
    const int64_t o = host.off[i], n = host.num_elem[i];
    for (int64_t jl = 0; jl < n; jl++) {
      const int64_t j = o + jl;
      Topo &t = host.topo[j];
      t.flags &= ~(uint32_t)(F_UP | F_DOWNR | F_DOWNL | F_IDENT);
      const bool ident = jl == 0 || jl == n - 1 || is_term[j];
      if (ident) {
        t.flags |= F_IDENT;
        continue;
      }
      if (jl != 1) t.flags |= F_UP;
      if (!is_term[j + 1]) t.flags |= F_DOWNR;
      if (t.flags & F_BRANCH) t.flags |= F_DOWNL;
    }
  }
  NRT_CUDA(cudaMemcpyAsync((void *)pv.topo, host.topo.data(), sizeof(Topo) * N,
                           cudaMemcpyHostToDevice, stream));
  // Segment pieces: maximal runs of consecutive physical rows linked to their
  // predecessor (mother == j - 1 with a mother column), cut at kMaxPiece rows.
  S.inst_row.assign(host.off.begin(), host.off.end());
  std::vector<int> inst_piece(ni + 1, 0);
  for (int32_t i = 0; i < ni; i++) {
    const int64_t o = host.off[i], n = host.num_elem[i];
    int64_t start = -1;
    for (int64_t jl = 0; jl < n; jl++) {
      const int64_t j = o + jl;
      const Topo &t = host.topo[j];
      const bool ident = t.flags & F_IDENT;
      const bool linked = !ident && (t.flags & F_UP) && t.mother == j - 1 && start >= 0 &&
                          (j - start) < kMaxPiece;
      if (!linked && start >= 0) {
        S.pieces.push_back(make_int2((int)start, (int)(j - start)));
        start = -1;
      }
      if (!ident && start < 0) start = j;
    }
    if (start >= 0) S.pieces.push_back(make_int2((int)start, (int)(o + n - start)));
    inst_piece[i + 1] = (int)S.pieces.size();
  }
  const int np = (int)S.pieces.size();
  const size_t tb = opt.precision == NRT_MIXED ? 4 : 8;
  const int tile_rows = (int)(kTileBytes / (4 * tb));
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
      make_tiles(S.pieces, cta_piece[c], cta_piece[c + 1], tile_rows, S.tiles);
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
    S.grid_blocks = std::max(1, std::min<int>(dev_sms * std::max(per_sm, 1), ni));
    S.inst_tile.assign(ni + 1, 0);
    for (int32_t i = 0; i < ni; i++) {
      S.inst_tile[i] = (int)S.tiles.size();
      make_tiles(S.pieces, inst_piece[i], inst_piece[i + 1], tile_rows, S.tiles);
    }
    S.inst_tile[ni] = (int)S.tiles.size();
  }
  S.tiles.push_back(np);  // sentinel: end piece of the last tile
  // device buffers
  cudaStream_t st = stream;
  ImView &iv = S.iv;
  iv.ntot = N;
  iv.m = opt.restart;
  iv.precond = opt.precond;
  iv.tol_mode = opt.tol_mode;
  iv.tol = opt.tol;
  iv.max_iter = opt.max_iter;
  iv.ninst = ni;
  iv.tile_rows = tile_rows;
  std::vector<double> cmdt(N), g64(N), w64(N), k64(N), inp(N);
  std::vector<float> gf(N);
  for (int64_t j = 0; j < N; j++) {
    cmdt[j] = host.c_m_dx[j] / host.inst[host.topo[j].flags >> INST_SHIFT].dT;
    g64[j] = host.gax[j];
    gf[j] = (float)host.gax[j];
    w64[j] = host.wdx[j];
    k64[j] = host.kdx[j];
    inp[j] = host.inp[j];
  }
  double *p;
  TRYI(up(arena, p, cmdt.data(), N, st)); iv.cmdt = p;
  TRYI(up(arena, p, g64.data(), N, st)); iv.g64 = p;
  TRYI(up(arena, p, w64.data(), N, st)); iv.wdx64 = p;
  TRYI(up(arena, p, k64.data(), N, st)); iv.kdx64 = p;
  TRYI(up(arena, p, inp.data(), N, st)); iv.inp64 = p;
  TRYI(up(arena, iv.diag, (const double *)nullptr, N, st));
  TRYI(up(arena, iv.rhs, (const double *)nullptr, N, st));
  float *pf;
  TRYI(up(arena, pf, gf.data(), N, st)); iv.gf = pf;
  iv.diagf = nullptr;
  if (mixed) TRYI(up(arena, iv.diagf, (const float *)nullptr, N, st));
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
  TRYI(up(arena, iv.partials, (const double *)nullptr, (size_t)2 * 4096 * kMaxDots, st));
  std::vector<InstStat> zero(ni, InstStat{0, 0, 0, 0.0});
  TRYI(up(arena, iv.stats, zero.data(), ni, st));
  iv.work_lev = nullptr;
  if (opt.precond == NRT_PRECOND_TREE) {
    TreeSchedule T;
    // staging slots: the factorisation stages two FP64 rows, a solve three T rows
    iv.tree_cap = (int)(kTileBytes / std::max<size_t>(2 * sizeof(double), 3 * tb));
    build_tree_schedule(host, iv.tree_cap, S.grid_mode, S.grid_blocks, T);
    TRYI(up(arena, pi, T.seg_len.data(), T.seg_len.size(), st)); iv.seg_len = pi;
    TRYI(up(arena, pi, T.seg_c1.data(), T.seg_c1.size(), st)); iv.seg_c1 = pi;
    TRYI(up(arena, pi, T.seg_c2.data(), T.seg_c2.size(), st)); iv.seg_c2 = pi;
    TRYI(up(arena, pi, T.seg_prow.data(), T.seg_prow.size(), st)); iv.seg_prow = pi;
    TRYI(up(arena, pi, T.seg_soff.data(), T.seg_soff.size(), st)); iv.seg_soff = pi;
    TRYI(up(arena, pi, T.tile_seg.data(), T.tile_seg.size(), st)); iv.tile_seg = pi;
    TRYI(up(arena, pi, T.tile_slot.data(), T.tile_slot.size(), st)); iv.tile_slot = pi;
    TRYI(up(arena, pi, T.slot_row.data(), T.slot_row.size(), st)); iv.slot_row = pi;
    TRYI(up(arena, pi, T.lev_tile.data(), T.lev_tile.size(), st)); iv.lev_tile = pi;
    TRYI(up(arena, pi, T.work_lev.data(), T.work_lev.size(), st)); iv.work_lev = pi;
    const size_t nseg = std::max<size_t>(1, T.seg_len.size());
    iv.tinv = arena.take(tb * N);
    iv.exp_b = arena.take(tb * nseg);
    TRYI(up(arena, iv.exp_d, (const double *)nullptr, nseg, st));
    if (!iv.tinv || !iv.exp_b) {
      set_error("arena exhausted (tree preconditioner)");
      return NRT_ENOMEM;
    }
  }
  NRT_CUDA(cudaStreamSynchronize(st));
  return NRT_OK;
}

// Runs `nsteps` implicit steps for every instance (one launch).
static int implicit_launch(Engine &e, int nsteps, int force) {
  ImplicitState &S = *e.im;
  NRT_CUDA(cudaMemsetAsync(S.iv.queue, 0, sizeof(int), e.stream));
  PackView pv = e.pv;
  ImView iv = S.iv;
  double *V0 = e.V[0], *V1 = e.V[1];
  int cur = e.cur;
  void *args[] = {&pv, &iv, &nsteps, &force, &V0, &V1, &cur};
  const bool mixed = e.opt.precision == NRT_MIXED;
  if (S.grid_mode) {
    const void *k = mixed ? (const void *)implicit_steps<float, true> : (const void *)implicit_steps<double, true>;
    NRT_CUDA(cudaLaunchCooperativeKernel(k, dim3(S.grid_blocks), dim3(kThreads), args, S.smem, e.stream));
  } else {
    const void *k = mixed ? (const void *)implicit_steps<float, false> : (const void *)implicit_steps<double, false>;
    NRT_CUDA(cudaLaunchKernel(k, dim3(S.grid_blocks), dim3(kThreads), args, S.smem, e.stream));
  }
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
  std::vector<InstStat> s(ni, InstStat{0, 0, 0, 0.0});
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

// Sum of non-converged steps over all instances (-1 on a device error).
int64_t nonconverged_total(Engine &e) {
  if (!e.im) return 0;
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
  int rc = implicit_launch(e, 1, input_active ? 1 : 0);
  S.iv.max_iter = saved_iter;
  if (rc) return rc;
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
