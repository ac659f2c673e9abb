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
// rotations; inner products and norms accumulate in FP64 in both precisions.  The
// preconditioner is an exact tridiagonal (Thomas) solve of every unbranched segment
// piece: the branch-point couplings are the only ones left to the Krylov iteration.
// Each cycle starts from the true FP64 residual b - A x, so in mixed precision (FP32
// basis, FP32 SpMV and preconditioner) every restart is one step of iterative
// refinement.  The warm start is x0 = V^n.
//
// Two launch shapes from one template:
//  * kGrid  (one tree): a cooperative launch over the whole GPU; rows are split into
//    contiguous per-CTA ranges aligned with segment pieces; grid-wide syncs separate the
//    phases and every CTA reduces the per-CTA partial sums in the same fixed order, so
//    all CTAs hold identical Krylov scalars.
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

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxPiece = 256;  // longest segment piece one thread eliminates

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
  int max_iter;      // per step per instance; <= 0 -> instance size
  int ninst;
  const double *cmdt;  // c_m dX / dT
  const double *g64;   // 1 / (r_a dX)
  const float *gf;
  const double *wdx64, *kdx64, *inp64;
  double *diag;
  float *diagf;
  double *rhs;
  void *Wb, *Z, *yv, *pcd, *pcc;  // T-typed workspace
  const int2 *pieces;             // (first row, length) of every segment piece
  const int *cta_row;             // kGrid: per-CTA row range [cta_row[c], cta_row[c+1])
  const int *cta_piece;           // kGrid: per-CTA piece range
  const int64_t *inst_row;        // per instance row range (ninst + 1)
  const int *inst_piece;          // per instance piece range (ninst + 1)
  const int *order;               // batch: instance processing order
  int *queue;                     // batch: next index into order
  double *partials;               // kGrid: 2 x gridDim x (kMaxRestart + 1)
  InstStat *stats;
};

template <typename T>
struct Work {
  T *Wb, *Z, *y, *pd, *pc;
};

// ---------------------------------------------------------------- reductions

// Per-CTA reduction of k values: each thread passes its contribution for value i through
// `acc(i)`; warps shuffle-reduce, then warp partials are summed in fixed order.
template <class F>
__device__ void block_sums(int k, F acc, double *warp_part, double *out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < k; i++) {
    double v = acc(i);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) warp_part[w * (kMaxRestart + 1) + i] = v;
  }
  __syncthreads();
  if (threadIdx.x < k) {
    double s = 0;
    for (int q = 0; q < kWarps; q++) s += warp_part[q * (kMaxRestart + 1) + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// Grid-wide: per-CTA sums -> global partials -> grid sync -> every CTA sums all CTAs'
// partials in the same order (32 lanes per value, fixed shuffle tree).
__device__ void grid_finish(cg::grid_group &grid, int k, double *cta_sums, double *partials,
                            int &parity, double *out) {
  double *buf = partials + (size_t)parity * gridDim.x * (kMaxRestart + 1);
  parity ^= 1;
  if (threadIdx.x < k) buf[(size_t)blockIdx.x * (kMaxRestart + 1) + threadIdx.x] = cta_sums[threadIdx.x];
  __threadfence();
  grid.sync();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = w; i < k; i += kWarps) {
    double v = 0;
    for (int c = lane; c < (int)gridDim.x; c += 32) v += buf[(size_t)c * (kMaxRestart + 1) + i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) out[i] = v;
  }
  __syncthreads();
}

// ---------------------------------------------------------------- kernel body

template <typename T, bool kGrid>
struct Ctx {
  PackView pv;
  ImView iv;
  Work<T> w;
  int64_t r0, r1;   // rows of this CTA (kGrid) or instance (batch)
  int p0, p1;       // pieces
  int inst;
  int64_t ninst_rows;
};

// A x over rows [r0, r1) for the physical rows; identity rows yield 0.  FP64 form.
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

// Thomas factorisation of every piece of this CTA: pd = pivots^-1, pc = c'.
template <typename T, bool kGrid>
__device__ void factor_pieces(Ctx<T, kGrid> &c) {
  for (int q = c.p0 + threadIdx.x; q < c.p1; q += blockDim.x) {
    const int2 pc = c.iv.pieces[q];
    double cprev = 0;
    for (int k = 0; k < pc.y; k++) {
      const int64_t j = pc.x + k;
      const double a = k ? -c.iv.g64[j] : 0.0;                  // sub-diagonal (j, j-1)
      const bool last = k + 1 == pc.y;
      const double cc = last ? 0.0 : -c.iv.g64[j + 1];           // super-diagonal (j, j+1)
      double piv = c.iv.diag[j] - a * cprev;
      double d = 1.0 / piv;
      cprev = cc * d;
      c.w.pd[j] = (T)d;
      c.w.pc[j] = (T)cprev;
    }
  }
}

// z = M^-1 v over this CTA's pieces (identity rows hold 0 in both).
template <typename T, bool kGrid>
__device__ void apply_precond(Ctx<T, kGrid> &c, const T *v, T *z) {
  if (c.iv.precond == NRT_PRECOND_SEGMENT) {
    for (int q = c.p0 + threadIdx.x; q < c.p1; q += blockDim.x) {
      const int2 pc = c.iv.pieces[q];
      T yprev = 0;
      for (int k = 0; k < pc.y; k++) {  // forward: y_k = (v_k - a_k y_{k-1}) d_k
        const int64_t j = pc.x + k;
        const T a = k ? (T)(-c.iv.g64[j]) : (T)0;
        yprev = (v[j] - a * yprev) * c.w.pd[j];
        z[j] = yprev;
      }
      T znext = z[pc.x + pc.y - 1];
      for (int k = pc.y - 2; k >= 0; k--) {  // backward: z_k = y_k - c'_k z_{k+1}
        const int64_t j = pc.x + k;
        znext = z[j] - c.w.pc[j] * znext;
        z[j] = znext;
      }
    }
  } else {
    for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x) {
      const uint32_t f = c.pv.topo[j].flags;
      if (f & F_IDENT) { z[j] = 0; continue; }
      z[j] = c.iv.precond == NRT_PRECOND_JACOBI ? (T)(v[j] / c.iv.diag[j]) : v[j];
    }
  }
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

// Sums k values over the group (CTA or grid) into out[0..k).
template <bool kGrid, class F>
__device__ void group_sums(cg::grid_group &grid, int k, F acc, double *warp_part, double *cta,
                           double *partials, int &parity, double *out) {
  if (kGrid) {
    block_sums(k, acc, warp_part, cta);
    grid_finish(grid, k, cta, partials, parity, out);
  } else {
    block_sums(k, acc, warp_part, out);
  }
}

struct Shared {
  double *H, *cs, *sn, *g, *s, *y, *red, *cta, *warp;
  int *flag;
};

__device__ Shared carve(double *base, int m) {
  Shared S;
  S.H = base;
  S.cs = S.H + (m + 1) * m;
  S.sn = S.cs + m;
  S.g = S.sn + m;
  S.s = S.g + (m + 1);
  S.y = S.s + (m + 1);
  S.red = S.y + m;
  S.cta = S.red + (kMaxRestart + 2);
  S.warp = S.cta + (kMaxRestart + 2);
  S.flag = (int *)(S.warp + kWarps * (kMaxRestart + 1));
  return S;
}

size_t shared_bytes(int m) {
  return sizeof(double) * ((size_t)(m + 1) * m + 2 * m + 2 * (m + 1) + m + 2 * (kMaxRestart + 2) +
                           kWarps * (kMaxRestart + 1)) + 16;
}

// One backward-Euler step of one group (CTA or grid) for instance c.inst.
template <typename T, bool kGrid>
__device__ void implicit_one_step(Ctx<T, kGrid> &c, cg::grid_group &grid, Shared &S, int &parity,
                                  const double *Vin, double *Vout, bool active, int64_t inst_n) {
  const PackView &pv = c.pv;
  const ImView &iv = c.iv;
  const int64_t N = pv.ntot;
  const int m = iv.m;
  // ---- assembly: gates (from V^n), W, K, diagonal, right-hand side, x0 = V^n
  for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x) {
    const Topo t = pv.topo[j];
    const double v = Vin[j];
    double wdx, kdx;
    if (t.flags & F_HH) {
      if (pv.hpf) {
        const float *hp = pv.hpf;
        const double rest = (double)hp[HP_REST * N + j];
        GateStep32 g = hh_step32((float)((v + (double)hp[HP_LSNA * N + j]) - rest),
                                 (float)((v + (double)hp[HP_LSK * N + j]) - rest), pv.gatef[j],
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
    Vout[j] = v;
  }
  __syncthreads();
  if (iv.precond == NRT_PRECOND_SEGMENT) factor_pieces(c);
  // ||b|| over physical rows (relative tolerance)
  double target = iv.tol;
  if (iv.tol_mode == NRT_TOL_REL) {
    group_sums<kGrid>(grid, 1, [&](int) {
      double a = 0;
      for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x)
        if (!(pv.topo[j].flags & F_IDENT)) a += iv.rhs[j] * iv.rhs[j];
      return a;
    }, S.warp, S.cta, iv.partials, parity, S.red);
    target = iv.tol * sqrt(S.red[0]);
  } else {
    group_sync<kGrid>(grid);  // x0 of every row visible before the first residual
  }
  // max_iter < 0 is the assembly-only pass of nrt_export_system
  const int budget = iv.max_iter > 0 ? iv.max_iter : (iv.max_iter < 0 ? 0 : (int)inst_n);
  const double inner_rel = sizeof(T) == 4 ? 1e-5 : 0.0;
  int iters = 0;
  double res = 0;
  bool converged = false;
  for (;;) {
    // ---- cycle start: true residual r = b - A x in FP64, W_0 = r, Z_0 = M^-1 r
    group_sums<kGrid>(grid, 1, [&](int) {
      double a = 0;
      for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x) {
        if (pv.topo[j].flags & F_IDENT) { c.w.Wb[j] = 0; continue; }
        const double r = iv.rhs[j] - row_apply64(pv, iv, j, Vout);
        c.w.Wb[j] = (T)r;
        a += r * r;
      }
      return a;
    }, S.warp, S.cta, iv.partials, parity, S.red);
    res = sqrt(S.red[0]);
    if (res <= target) {
      converged = true;
      break;
    }
    if (iters >= budget) break;
    apply_precond(c, c.w.Wb, c.w.Z);
    group_sync<kGrid>(grid);  // Z_0 visible to neighbours
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
      // y = s_j A Z_j; p_i = <y, W_i>, i <= j
      for (int64_t r = c.r0 + threadIdx.x; r < c.r1; r += blockDim.x)
        c.w.y[r] = sj * row_apply<T>(pv, iv, r, Zj);
      group_sums<kGrid>(grid, j + 1, [&](int i) {
        const T *Wi = c.w.Wb + (size_t)i * N;
        double a = 0;
        for (int64_t r = c.r0 + threadIdx.x; r < c.r1; r += blockDim.x)
          a += (double)c.w.y[r] * (double)Wi[r];
        return a;
      }, S.warp, S.cta, iv.partials, parity, S.red);
      if (threadIdx.x <= j) S.H[threadIdx.x * m + j] = S.s[threadIdx.x] * S.red[threadIdx.x];
      __syncthreads();
      // w = y - sum_i h_ij s_i W_i -> W_{j+1}; ||w||; Z_{j+1} = M^-1 w
      T *Wn = c.w.Wb + (size_t)(j + 1) * N;
      for (int64_t r = c.r0 + threadIdx.x; r < c.r1; r += blockDim.x) {
        double a = (double)c.w.y[r];
        for (int i = 0; i <= j; i++)
          a -= S.H[i * m + j] * S.s[i] * (double)c.w.Wb[(size_t)i * N + r];
        Wn[r] = (T)a;
      }
      __syncthreads();
      apply_precond(c, Wn, c.w.Z + (size_t)(j + 1) * N);
      group_sums<kGrid>(grid, 1, [&](int) {
        double a = 0;
        for (int64_t r = c.r0 + threadIdx.x; r < c.r1; r += blockDim.x) {
          const double v = (double)Wn[r];
          a += v * v;
        }
        return a;
      }, S.warp, S.cta, iv.partials, parity, S.red);
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
      for (int i = 0; i < k; i++) S.y[i] *= S.s[i];
    }
    __syncthreads();
    for (int64_t r = c.r0 + threadIdx.x; r < c.r1; r += blockDim.x) {
      if (pv.topo[r].flags & F_IDENT) continue;
      double a = Vout[r];
      for (int i = 0; i < k; i++) a += S.y[i] * (double)c.w.Z[(size_t)i * N + r];
      Vout[r] = a;
    }
    group_sync<kGrid>(grid);
  }
  if (threadIdx.x == 0 && (!kGrid || blockIdx.x == 0)) {
    InstStat &st = iv.stats[c.inst];
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
  extern __shared__ double smem[];
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
  double *V[2] = {V0, V1};
  if (kGrid) {
    c.inst = 0;
    c.r0 = iv.cta_row[blockIdx.x];
    c.r1 = iv.cta_row[blockIdx.x + 1];
    c.p0 = iv.cta_piece[blockIdx.x];
    c.p1 = iv.cta_piece[blockIdx.x + 1];
    const InstDev in = pv.inst[0];
    const int64_t inst_n = iv.inst_row[1] - iv.inst_row[0];
    for (int s = 0; s < nsteps; s++) {
      const int64_t i = in.base + s;
      if (i >= in.iend) break;
      const bool active = force >= 0 ? force != 0
                                     : ((double)i * in.dT >= in.t0 && (double)i * in.dT <= in.t1);
      implicit_one_step<T, kGrid>(c, grid, S, parity, V[(cur + s) & 1], V[(cur + s + 1) & 1], active,
                                  inst_n);
    }
  } else {
    for (;;) {
      if (threadIdx.x == 0) S.flag[1] = atomicAdd(iv.queue, 1);
      __syncthreads();
      const int q = S.flag[1];
      __syncthreads();
      if (q >= iv.ninst) break;
      const int inst = iv.order[q];
      c.inst = inst;
      c.r0 = iv.inst_row[inst];
      c.r1 = iv.inst_row[inst + 1];
      c.p0 = iv.inst_piece[inst];
      c.p1 = iv.inst_piece[inst + 1];
      const InstDev in = pv.inst[inst];
      int s = 0;
      for (; s < nsteps; s++) {
        const int64_t i = in.base + s;
        if (i >= in.iend) break;
        const bool active = force >= 0 ? force != 0
                                       : ((double)i * in.dT >= in.t0 && (double)i * in.dT <= in.t1);
        implicit_one_step<T, kGrid>(c, grid, S, parity, V[(cur + s) & 1], V[(cur + s + 1) & 1],
                                    active, c.r1 - c.r0);
      }
      if ((nsteps - s) & 1) {  // finished early: put its latest V where the others' is
        for (int64_t j = c.r0 + threadIdx.x; j < c.r1; j += blockDim.x)
          V[(cur + nsteps) & 1][j] = V[(cur + s) & 1][j];
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------- host side

struct ImplicitState {
  ImView iv{};
  std::vector<int2> pieces;
  std::vector<int> cta_row, cta_piece, inst_piece, order;
  std::vector<int64_t> inst_row;
  int grid_blocks = 0;
  bool grid_mode = false;
  std::vector<InstStat> last_stats;
};

size_t Engine::implicit_bytes() const {
  const int64_t N = host.ntot;
  const size_t tb = opt.precision == NRT_MIXED ? 4 : 8;
  const int m = opt.restart;
  size_t b = 0;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  b += 6 * al(8 * N);                              // cmdt, g64, wdx64, kdx64, inp64, diag
  b += al(8 * N) + al(4 * N) + al(4 * N);          // rhs, diagf, gf
  b += al(tb * N * (m + 1)) + al(tb * N * (m + 1)) + 3 * al(tb * N);  // Wb, Z, y, pd, pc
  b += al(8 * (N + 2)) * 2;                        // pieces (upper bound: one per row)
  b += al(4 * (N + 2)) * 2 + al(8 * (host.ninst + 1)) + al(4 * (host.ninst + 1)) * 2 + al(4 * host.ninst);
  b += al(sizeof(double) * 2 * 4096 * (kMaxRestart + 1));
  b += al(sizeof(InstStat) * host.ninst) + al(64);
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

int Engine::implicit_init() {
  im = new ImplicitState();
  ImplicitState &S = *im;
  const int64_t N = host.ntot;
  const int32_t ni = host.ninst;
  // implicit row structure (flags) per element; the validator guaranteed the
  // reference numbering, so mother < j, DR == j + 1 off terminals.
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
  // predecessor (mother == j - 1 with a mother column), cut at kMaxPiece.
  S.inst_row.assign(host.off.begin(), host.off.end());
  S.inst_piece.assign(ni + 1, 0);
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
    S.inst_piece[i + 1] = (int)S.pieces.size();
  }
  // One tree: cooperative grid over all SMs, row ranges aligned with pieces.
  S.grid_mode = ni == 1;
  int dev_sms = 0;
  NRT_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device));
  const size_t smem = shared_bytes(opt.restart);
  if (S.grid_mode) {
    int per_sm = 0;
    auto kern = opt.precision == NRT_MIXED ? implicit_steps<float, true> : implicit_steps<double, true>;
    NRT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    NRT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    if (per_sm < 1) {
      set_error("implicit kernel does not fit on an SM");
      return NRT_EDEVICE;
    }
    // enough CTAs to cover the rows, at most one wave of co-resident CTAs
    const int64_t want = (N + 4 * kThreads - 1) / (4 * kThreads);
    int G = (int)std::min<int64_t>((int64_t)dev_sms * std::min(per_sm, 2), std::max<int64_t>(1, want));
    G = std::min(G, 4096);
    const int np = (int)S.pieces.size();
    S.cta_row.assign(G + 1, (int)N);
    S.cta_piece.assign(G + 1, np);
    int q = 0;
    for (int c = 0; c < G; c++) {
      const int64_t goal = (N * (int64_t)c) / G;
      while (q < np && S.pieces[q].x + S.pieces[q].y <= goal) q++;
      S.cta_piece[c] = std::min(q, np);
      S.cta_row[c] = c == 0 ? 0 : (q < np ? S.pieces[q].x : (int)N);
    }
    S.cta_row[0] = 0;
    S.cta_piece[0] = 0;
    for (int c = 1; c <= G; c++) {  // keep ranges monotone
      S.cta_row[c] = std::max(S.cta_row[c], S.cta_row[c - 1]);
      S.cta_piece[c] = std::max(S.cta_piece[c], S.cta_piece[c - 1]);
    }
    S.cta_row[G] = (int)N;
    S.cta_piece[G] = np;
    S.grid_blocks = G;
  } else {
    S.order.resize(ni);
    for (int32_t i = 0; i < ni; i++) S.order[i] = i;
    std::stable_sort(S.order.begin(), S.order.end(),
                     [&](int a, int b) { return host.num_elem[a] > host.num_elem[b]; });
    int per_sm = 0;
    auto kern = opt.precision == NRT_MIXED ? implicit_steps<float, false> : implicit_steps<double, false>;
    NRT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    NRT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    S.grid_blocks = std::max(1, std::min<int>(dev_sms * std::max(per_sm, 1), ni));
  }
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
  if (opt.precision == NRT_MIXED) TRYI(up(arena, iv.diagf, (const float *)nullptr, N, st));
  const size_t tb = opt.precision == NRT_MIXED ? 4 : 8;
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
  if (S.grid_mode) {
    TRYI(up(arena, pi, S.cta_row.data(), S.cta_row.size(), st)); iv.cta_row = pi;
    TRYI(up(arena, pi, S.cta_piece.data(), S.cta_piece.size(), st)); iv.cta_piece = pi;
  }
  int64_t *pl;
  TRYI(up(arena, pl, S.inst_row.data(), S.inst_row.size(), st)); iv.inst_row = pl;
  TRYI(up(arena, pi, S.inst_piece.data(), S.inst_piece.size(), st)); iv.inst_piece = pi;
  if (!S.grid_mode) {
    TRYI(up(arena, pi, S.order.data(), S.order.size(), st)); iv.order = pi;
  }
  TRYI(up(arena, iv.queue, (const int *)nullptr, 1, st));
  TRYI(up(arena, iv.partials, (const double *)nullptr, (size_t)2 * 4096 * (kMaxRestart + 1), st));
  S.last_stats.assign(ni, InstStat{0, 0, 0, 0.0});
  TRYI(up(arena, iv.stats, S.last_stats.data(), ni, st));
  return NRT_OK;
}

// Runs `nsteps` implicit steps for every instance (one launch).
static int implicit_launch(Engine &e, int nsteps, int force) {
  ImplicitState &S = *e.im;
  const size_t smem = shared_bytes(e.opt.restart);
  NRT_CUDA(cudaMemsetAsync(S.iv.queue, 0, sizeof(int), e.stream));
  PackView pv = e.pv;
  ImView iv = S.iv;
  double *V0 = e.V[0], *V1 = e.V[1];
  int cur = e.cur;
  void *args[] = {&pv, &iv, &nsteps, &force, &V0, &V1, &cur};
  const bool mixed = e.opt.precision == NRT_MIXED;
  if (S.grid_mode) {
    const void *k = mixed ? (const void *)implicit_steps<float, true> : (const void *)implicit_steps<double, true>;
    NRT_CUDA(cudaLaunchCooperativeKernel(k, dim3(S.grid_blocks), dim3(kThreads), args, smem, e.stream));
  } else {
    const void *k = mixed ? (const void *)implicit_steps<float, false> : (const void *)implicit_steps<double, false>;
    NRT_CUDA(cudaLaunchKernel(k, dim3(S.grid_blocks), dim3(kThreads), args, smem, e.stream));
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
// column order: mother, diagonal, DR, DL; identity rows 1).
int export_system(Engine &e, int input_active, int32_t *row_ptr, int32_t *col, double *val,
                  double *rhs, int32_t *nnz_out) {
  if (e.opt.mode != NRT_IMPLICIT_BE || e.host.ninst != 1) {
    set_error("export_system needs a single-tree implicit solver");
    return NRT_EINVAL;
  }
  // Assemble on copies of the state: save gates, run one assembly-only pass via a
  // zero-iteration solve, then restore.
  const int64_t N = e.host.ntot;
  const bool mixed = e.opt.precision == NRT_MIXED;
  const size_t gb = (mixed ? 4 : 8) * 3 * N;
  void *gate = mixed ? (void *)e.pv.gatef : (void *)e.pv.gate;
  std::vector<char> saved(gb);
  std::vector<double> Vsave(N), Vother(N);
  ImplicitState &S = *e.im;
  InstStat stat0;
  NRT_CUDA(cudaMemcpyAsync(saved.data(), gate, gb, cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaMemcpyAsync(Vother.data(), e.V[e.cur ^ 1], 8 * N, cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaMemcpyAsync(&stat0, S.iv.stats, sizeof(InstStat), cudaMemcpyDeviceToHost, e.stream));
  NRT_CUDA(cudaStreamSynchronize(e.stream));
  const int saved_iter = S.iv.max_iter;
  S.iv.max_iter = -1;  // budget 0 after the first residual: assembly only
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
