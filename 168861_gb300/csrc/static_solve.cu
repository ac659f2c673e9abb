// nrt_solve_csr_static: one implicit step's linear solve that allocates nothing.
//
// Who needs it: callers that cannot call cudaMalloc -- a host application that owns the
// device memory pool and forbids other allocators, a loop that must not allocate after
// start-up, or a plugin that is handed pre-allocated device buffers only.  They pass the
// system and the solution vector in their own device memory; every temporary (Krylov
// basis, preconditioned basis, SpMV result, preconditioner factors, reduction partials,
// the result record) lives in one file-scope static __device__ array of
// NRT_STATIC_SCRATCH_BYTES.  The array is reserved on a device when this file's module is
// loaded there: under CUDA's default lazy module loading that is the first call of the
// entry point on that device (or a process-wide start-up load with
// CUDA_MODULE_LOADING=EAGER).  From then on the device holds it until the process exits,
// and no later call changes the device's free memory.
//
// Method: right-preconditioned GMRES(m) with classical Gram-Schmidt and Givens rotations,
// FP64 throughout, with fixed-order grid reductions.  It is the method of the solver
// handles, over the reference's CSR system (the createMatrix layout,
// src/solverIm-cpu.cpp:29-183, as nrt_export_system returns it).  Preconditioner: an exact
// tridiagonal solve of fixed 64-row blocks, built from the (j, j-1) and (j, j+1) entries
// inside each block.  One cooperative launch on the caller's stream.
//
// Sharing: every call uses the same array and leaves its contents behind.  Each region the
// kernel reads is first written by the same call, so nothing has to be cleared between
// calls.  Calls that overlap on the GPU (different streams, or different host threads,
// without ordering) race on the array and corrupt each other's results.
#include <cooperative_groups.h>

#include <algorithm>
#include <mutex>

#include "nrt_internal.h"
#include "pdl.cuh"

namespace cg = cooperative_groups;

namespace nrt {
namespace {

constexpr int kT = 256;
constexpr int kW = kT / 32;
constexpr int kBlk = 64;                       // preconditioner block rows
constexpr int kM = NRT_STATIC_MAX_RESTART;
constexpr int kMaxG = 1024;                    // CTAs at most
constexpr int kResult = 4;                     // iterations, residual, converged, spare

static __device__ __align__(256) unsigned char g_static_scratch[NRT_STATIC_SCRATCH_BYTES];

// Offsets (in doubles) of the regions inside the scratch array.
struct Layout {
  size_t W, Z, y, pd, pc, pl, partials, result, total;
};

__host__ __device__ inline Layout layout(int n, int m) {
  Layout L;
  const size_t N = (size_t)n;
  L.W = 0;
  L.Z = L.W + N * (m + 1);
  L.y = L.Z + N * (m + 1);
  L.pd = L.y + N;
  L.pc = L.pd + N;
  L.pl = L.pc + N;
  L.partials = L.pl + N;
  L.result = L.partials + 2 * (size_t)kMaxG * (kM + 1);
  L.total = L.result + kResult;
  return L;
}

struct Args {
  int n, m, tol_mode, max_iter, rows_per_cta;
  double tol;
  const int *row_ptr, *col;
  const double *val, *b;
  double *x;
  double *scratch;
};

__device__ __forceinline__ double row_mv(const Args &a, int j, const double *v) {
  double s = 0;
  for (int p = a.row_ptr[j]; p < a.row_ptr[j + 1]; p++) s += a.val[p] * v[a.col[p]];
  return s;
}

// Diagonal and the block-local sub/super-diagonal entries of row j.
__device__ __forceinline__ void tri(const Args &a, int j, double &d, double &lo, double &hi) {
  d = lo = hi = 0;
  const int b0 = (j / kBlk) * kBlk;
  for (int p = a.row_ptr[j]; p < a.row_ptr[j + 1]; p++) {
    const int c = a.col[p];
    if (c == j) d += a.val[p];
    else if (c == j - 1 && j > b0) lo += a.val[p];
    else if (c == j + 1 && c < b0 + kBlk) hi += a.val[p];
  }
}

// z = M^-1 v over this CTA's blocks (pl: each row's block-local sub-diagonal entry, kept
// by the factorisation so that no application scans the CSR rows again).
__device__ void precond(const double *pd, const double *pc, const double *pl, const double *v,
                        double *z, int r0, int r1) {
  for (int b0 = r0 + threadIdx.x * kBlk; b0 < r1; b0 += kT * kBlk) {
    const int e = min(r1, b0 + kBlk);
    double y = 0;
    for (int j = b0; j < e; j++) {
      y = (v[j] - pl[j] * y) * pd[j];
      z[j] = y;
    }
    for (int j = e - 2; j >= b0; j--) {
      y = z[j] - pc[j] * y;
      z[j] = y;
    }
  }
}

// Sums k per-thread values over the grid; every CTA gets the same totals in out[0..k).
__device__ void grid_sums(cg::grid_group &grid, const double *acc, int k, double *partials,
                          int &parity, double *warp_part, double *out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < k; i++) {
    double v = acc[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) warp_part[w * (kM + 1) + i] = v;
  }
  __syncthreads();
  double *buf = partials + (size_t)parity * kMaxG * (kM + 1);
  parity ^= 1;
  if (threadIdx.x < k) {
    double s = 0;
    for (int q = 0; q < kW; q++) s += warp_part[q * (kM + 1) + threadIdx.x];
    buf[(size_t)blockIdx.x * (kM + 1) + threadIdx.x] = s;
  }
  __syncthreads();
  __threadfence();
  grid.sync();
  for (int i = w; i < k; i += kW) {
    double v = 0;
    for (int c = lane; c < (int)gridDim.x; c += 32) v += buf[(size_t)c * (kM + 1) + i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) out[i] = v;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kT) static_gmres(Args a) {
  __shared__ double H[(kM + 1) * kM], cs[kM], sn[kM], g[kM + 1], s[kM + 1], yv[kM],
      red[kM + 1], warp_part[kW * (kM + 1)];
  __shared__ int flag;
  cg::grid_group grid = cg::this_grid();
  const int n = a.n, m = a.m;
  const Layout L = layout(n, m);
  double *W = a.scratch + L.W, *Z = a.scratch + L.Z, *Y = a.scratch + L.y;
  double *pd = a.scratch + L.pd, *pc = a.scratch + L.pc, *pl = a.scratch + L.pl;
  double *partials = a.scratch + L.partials;
  const int r0 = min(n, (int)blockIdx.x * a.rows_per_cta);
  const int r1 = min(n, r0 + a.rows_per_cta);
  int parity = 0;
  // block factors (each 64-row block lies inside one CTA's rows)
  for (int b0 = r0 + threadIdx.x * kBlk; b0 < r1; b0 += kT * kBlk) {
    const int e = min(r1, b0 + kBlk);
    double cprev = 0;
    for (int j = b0; j < e; j++) {
      double d, lo, hi;
      tri(a, j, d, lo, hi);
      const double dd = 1.0 / (d - lo * cprev);
      cprev = hi * dd;
      pd[j] = dd;
      pc[j] = cprev;
      pl[j] = lo;
    }
  }
  double acc[kM + 1];
  acc[0] = acc[1] = 0;
  for (int j = r0 + threadIdx.x; j < r1; j += kT) {
    // ||b|| over coupled rows only: a decoupled row (the reference's identity rows) is
    // solved exactly by the block preconditioner and would otherwise dominate the norm
    bool coupled = false;
    for (int p = a.row_ptr[j]; p < a.row_ptr[j + 1]; p++) coupled |= a.col[p] != j;
    if (coupled) acc[0] += a.b[j] * a.b[j];
    acc[1] += a.b[j] * a.b[j];
  }
  grid_sums(grid, acc, 2, partials, parity, warp_part, red);
  // relative mode: against ||b|| over the coupled rows; over all rows when those are zero;
  // against the first residual when b is zero everywhere (x = 0 is then the solution and
  // an exact zero residual need never come)
  const double bref = red[0] > 0 ? sqrt(red[0]) : sqrt(red[1]);
  double target = a.tol_mode == NRT_TOL_REL ? a.tol * bref : a.tol;
  const bool target_from_r0 = a.tol_mode == NRT_TOL_REL && !(bref > 0);
  const int budget = a.max_iter > 0 ? a.max_iter : n;
  int iters = 0;
  double res = 0;
  int status = 0;  // 1 converged, 2 a non-finite residual or basis norm ended the solve
  for (int cycle = 0;; cycle++) {
    // residual of the current x; W_0 = r, Z_0 = M^-1 r
    acc[0] = 0;
    for (int j = r0 + threadIdx.x; j < r1; j += kT) {
      const double r = a.b[j] - row_mv(a, j, a.x);
      W[j] = r;
      acc[0] += r * r;
    }
    __syncthreads();
    precond(pd, pc, pl, W, Z, r0, r1);
    grid_sums(grid, acc, 1, partials, parity, warp_part, red);  // also publishes Z_0
    res = sqrt(red[0]);
    if (!isfinite(res)) {  // NaN or Inf in the system or in x: no iteration can recover
      status = 2;
      break;
    }
    if (cycle == 0 && target_from_r0) target = a.tol * res;
    if (res <= target) {
      status = 1;
      break;
    }
    if (iters >= budget) break;
    if (threadIdx.x == 0) {
      g[0] = res;
      for (int i = 1; i <= m; i++) g[i] = 0;
      s[0] = 1.0 / res;
    }
    __syncthreads();
    int k = 0;
    for (int j = 0; j < m; j++) {
      for (int i = 0; i <= j; i++) acc[i] = 0;
      const double *Zj = Z + (size_t)j * n;
      for (int r = r0 + threadIdx.x; r < r1; r += kT) {
        const double y = s[j] * row_mv(a, r, Zj);
        Y[r] = y;
        for (int i = 0; i <= j; i++) acc[i] += y * W[(size_t)i * n + r];
      }
      grid_sums(grid, acc, j + 1, partials, parity, warp_part, red);
      if (threadIdx.x <= j) H[threadIdx.x * m + j] = s[threadIdx.x] * red[threadIdx.x];
      __syncthreads();
      double *Wn = W + (size_t)(j + 1) * n;
      acc[0] = 0;
      for (int r = r0 + threadIdx.x; r < r1; r += kT) {
        double v = Y[r];
        for (int i = 0; i <= j; i++) v -= H[i * m + j] * s[i] * W[(size_t)i * n + r];
        Wn[r] = v;
        acc[0] += v * v;
      }
      __syncthreads();
      precond(pd, pc, pl, Wn, Z + (size_t)(j + 1) * n, r0, r1);
      grid_sums(grid, acc, 1, partials, parity, warp_part, red);  // publishes Z_{j+1}
      if (threadIdx.x == 0) {
        const double hn = sqrt(red[0]);
        s[j + 1] = hn > 0 ? 1.0 / hn : 0.0;
        for (int i = 0; i < j; i++) {
          const double p = H[i * m + j], q = H[(i + 1) * m + j];
          H[i * m + j] = cs[i] * p + sn[i] * q;
          H[(i + 1) * m + j] = -sn[i] * p + cs[i] * q;
        }
        const double p = H[j * m + j];
        const double den = sqrt(p * p + hn * hn);
        cs[j] = den == 0 ? 1.0 : p / den;
        sn[j] = den == 0 ? 0.0 : hn / den;
        H[j * m + j] = den;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        flag = !isfinite(hn) ? 2 : ((fabs(g[j + 1]) <= target || hn == 0) ? 1 : 0);
      }
      __syncthreads();
      if (flag == 2) break;  // every CTA read the same sums: a uniform exit
      k = j + 1;
      iters++;
      if (flag || iters >= budget) break;
    }
    if (flag == 2) {  // leave x at the cycle's start, which was finite
      status = 2;
      break;
    }
    if (threadIdx.x == 0) {
      for (int i = k - 1; i >= 0; i--) {
        double v = g[i];
        for (int l = i + 1; l < k; l++) v -= H[i * m + l] * yv[l];
        yv[i] = v / H[i * m + i];
      }
      for (int i = 0; i < k; i++) yv[i] *= s[i];
    }
    __syncthreads();
    for (int r = r0 + threadIdx.x; r < r1; r += kT) {
      double v = a.x[r];
      for (int i = 0; i < k; i++) v += yv[i] * Z[(size_t)i * n + r];
      a.x[r] = v;
    }
    __syncthreads();
    __threadfence();
    grid.sync();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double *out = a.scratch + L.result;
    out[0] = iters;
    out[1] = res;
    out[2] = status;
  }
}

std::mutex g_setup_mu;
constexpr int kMaxDevices = 64;
double *g_scratch_ptr[kMaxDevices] = {nullptr};

}  // namespace
}  // namespace nrt

extern "C" int nrt_solve_csr_static(int32_t n, const int32_t *row_ptr, const int32_t *col,
                                    const double *val, const double *b, double *x,
                                    int32_t restart, double tol, int32_t tol_mode,
                                    int32_t max_iter, void *stream, int32_t *iters_out,
                                    double *residual_out) {
  return nrt::guarded([&]() -> int {
    using namespace nrt;
    if (n < 1 || !row_ptr || !col || !val || !b || !x || !(tol > 0) || max_iter < 0 ||
        (tol_mode != NRT_TOL_ABS && tol_mode != NRT_TOL_REL)) {
      set_error("nrt_solve_csr_static: bad argument");
      return NRT_EINVAL;
    }
    if (restart < 1 || restart > kM) {
      set_error("nrt_solve_csr_static: restart must be in [1, NRT_STATIC_MAX_RESTART]");
      return NRT_EINVAL;
    }
    const Layout L = layout(n, restart);
    if (L.total * sizeof(double) > (size_t)NRT_STATIC_SCRATCH_BYTES) {
      set_error("nrt_solve_csr_static: n * (2 * restart + 6) doubles exceed the static scratch "
                "(NRT_STATIC_SCRATCH_BYTES); use a smaller restart or the handle API");
      return NRT_EBUDGET;
    }
    int dev = 0;
    NRT_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
      set_error("nrt_solve_csr_static: device ordinal out of range");
      return NRT_EDEVICE;
    }
    double *scratch;
    {
      // Once per device, with that device current: the device address of the static array.
      std::lock_guard<std::mutex> lk(g_setup_mu);
      if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        NRT_CUDA(cudaGetSymbolAddress(&p, g_static_scratch));
        g_scratch_ptr[dev] = (double *)p;
      }
      scratch = g_scratch_ptr[dev];
    }
    int sms = 0, per_sm = 0;
    NRT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    NRT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, static_gmres, kT, 0));
    if (per_sm < 1) {
      set_error("nrt_solve_csr_static: kernel does not fit on an SM");
      return NRT_EDEVICE;
    }
    // rows per CTA: whole preconditioner blocks, at least 4 of them per CTA
    int G = (int)std::min<long long>((long long)sms * per_sm, kMaxG);
    int rows = (((n + G - 1) / G + kBlk - 1) / kBlk) * kBlk;
    rows = std::max(rows, 4 * kBlk);
    G = (n + rows - 1) / rows;
    Args a;
    a.n = n;
    a.m = restart;
    a.tol = tol;
    a.tol_mode = tol_mode;
    a.max_iter = max_iter;
    a.rows_per_cta = rows;
    a.row_ptr = row_ptr;
    a.col = col;
    a.val = val;
    a.b = b;
    a.x = x;
    a.scratch = scratch;
    void *args[] = {&a};
    cudaStream_t st = (cudaStream_t)stream;
    NRT_CUDA(cudaLaunchCooperativeKernel((const void *)static_gmres, dim3(G), dim3(kT), args, 0, st));
    count_launch_on(st);
    double res[3];
    NRT_CUDA(cudaMemcpyAsync(res, scratch + L.result, sizeof(res), cudaMemcpyDeviceToHost, st));
    NRT_CUDA(cudaStreamSynchronize(st));
    if (iters_out) *iters_out = (int32_t)res[0];
    if (residual_out) *residual_out = res[1];
    if (res[2] == 2.0) {
      set_error("nrt_solve_csr_static: a residual or Krylov basis norm is not finite (NaN or "
                "Inf in the system, the right-hand side or the initial guess)");
      return NRT_EINVAL;
    }
    if (res[2] == 0.0) {
      set_error("nrt_solve_csr_static: iteration budget reached");
      return NRT_ENOCONV;
    }
    return NRT_OK;
  });
}
