// Time-varying strain for the explicit stepper (nrt_set_strain).
//
// The reference applies strain once, before the run (src/init.cpp:235-254,320-333:
// dX (1+e), d / sqrt(1+e), the damage shifts of E_Na, E_K and the left shifts, g_Na and
// g_K / sqrt(1+e), E_L from the rest equilibrium).  Here a set of elements follows a
// strain that ramps linearly in time, e(t) = e0 + (e1 - e0) (t - t0) / (t1 - t0) clamped
// to [t0, t1], and before every step a small kernel re-evaluates those static formulas
// for them (derive_elem.h, the same code as nrt_derive) at t = i dT.  It rewrites what
// the step reads: dT/(c_m dX), 1/(r_a dX), W dX and K dX of cables, and the parameter
// column of each HH element (each strained HH element gets a column of its own).  The
// gates are state: strain changes their rates, not their values.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "derive_elem.h"
#include "nrt_solver.h"
#include "pdl.cuh"
#include "strain.cuh"

namespace nrt {

struct StrainState {
  void *mem = nullptr;
  StrainView view{};
  ~StrainState() {
    if (mem) cudaFree(mem);
  }
};

namespace {

constexpr int kStrainBlock = 32;          // strained elements (or table entries) per block

// Class c's coefficients for step k of the current loop range into o[kStrainOut]; false
// when the class's instance has finished its run (nothing is written then).
__device__ bool derive_class(const StrainView &s, const PackView &p, int c, int k, double *o) {
  const InstDev in = p.inst[s.inst[c]];
  const int64_t i = in.base + k;
  if (i >= in.iend) return false;
  const double t = (double)i * in.dT;
  const double e =
      t <= s.t0 ? s.eps0
                : (t >= s.t1 ? s.eps1 : s.eps0 + (s.eps1 - s.eps0) * ((t - s.t0) / (s.t1 - s.t0)));
  const int n = s.ncls;
  nrt_param::ElemIn x;
  x.kind = s.kind[c];
  x.dX0 = s.spec[c];
  x.diam0 = s.spec[n + c];
  x.eps = e;
  x.ro_a = s.spec[2 * n + c];
  x.ro_m = s.spec[3 * n + c];
  x.per_m = s.spec[4 * n + c];
  x.th = s.spec[5 * n + c];
  x.rest = s.spec[6 * n + c];
  x.sna = s.spec[7 * n + c];
  x.sk = s.spec[8 * n + c];
  x.sl = s.spec[9 * n + c];
  double ep[6], hp[12];
  nrt_param::derive_element(x, s.myelin, s.e_max, ep, hp);
  const double c_m = ep[0], r_a = ep[1], dx = ep[2];
  o[0] = in.dT / (c_m * dx);  // as the pack builds them
  o[1] = 1.0 / (r_a * dx);
  if (x.kind == 1) {
    double *v = o + 2;
    v[HP_GNA] = hp[3];
    v[HP_GK] = hp[4];
    v[HP_GL] = hp[5];
    v[HP_ENA] = hp[6];
    v[HP_EK] = hp[7];
    v[HP_EL] = hp[8];
    v[HP_LSNA] = hp[9];
    v[HP_LSK] = hp[10];
    v[HP_REST] = hp[11];
    v[HP_DX] = dx;
    v[HP_DTMS] = in.dT * 1000;  // src/solverEx-cpu.cpp:96
  } else {
    o[2] = ep[3] * dx;
    o[3] = ep[4] * dx;
  }
  return true;
}

// Step k, derivation and writes in one launch.  Block b owns elements [32 b, 32 b + 32)
// of the class-sorted list, which span at most 32 consecutive classes.  Thread t derives
// class (first class of the block) + t, if the block has it, into shared memory; then
// every thread writes its own element.
__global__ void __launch_bounds__(kStrainBlock) strain_update(StrainView s, PackView p, int k,
                                                                int mixed) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  __shared__ double out[kStrainBlock][kStrainOut];
  __shared__ int live[kStrainBlock];
  const int q0 = blockIdx.x * kStrainBlock;
  const int qlast = min(q0 + kStrainBlock, s.n) - 1;
  const int c0 = s.cls[q0], c = c0 + (int)threadIdx.x;
  if (c <= s.cls[qlast]) live[threadIdx.x] = derive_class(s, p, c, k, out[threadIdx.x]);
  __syncthreads();
  const int q = q0 + (int)threadIdx.x;
  if (q > qlast) return;
  const int t = s.cls[q] - c0;
  if (live[t]) apply_element(s, p, q, out[t], mixed);
}

// Steps 0 .. nk-1 of a graph chunk, derived ahead in one launch: the coefficients depend
// on time only, so all (step, class) pairs run in parallel instead of one chain of FP64
// work per step.  Entry g is step g / ncls, class g % ncls.
__global__ void __launch_bounds__(kStrainBlock) strain_derive(StrainView s, PackView p, int nk) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  const int64_t g = (int64_t)blockIdx.x * kStrainBlock + threadIdx.x;
  if (g >= (int64_t)nk * s.ncls) return;
  const int k = (int)(g / s.ncls), c = (int)(g % s.ncls);
  s.tlive[g] = derive_class(s, p, c, k, s.tab + g * kStrainOut);
}

// Step k of the chunk: every strained element takes its class's row of the table.
__global__ void __launch_bounds__(256) strain_apply(StrainView s, PackView p, int k, int mixed) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.n) return;
  apply_row(s, p, q, k, mixed);
}

}  // namespace

int launch_strain_update(const Engine &e, int k, cudaStream_t st) {
  const StrainView &v = e.strain->view;
  if (v.n <= 0) return NRT_OK;
  // one warp per block: distinct classes are bound by each SM's FP64 pipe, so they are
  // spread over as many SMs as there are warps of elements
  NRT_CUDA(launch_chained(strain_update, (v.n + kStrainBlock - 1) / kStrainBlock, kStrainBlock, 0,
                          st, v, e.pv, k, (int)(e.opt.precision == NRT_MIXED)));
  return NRT_OK;
}

bool strain_tabled(const Engine &e) { return e.strain && e.strain->view.tab; }

const StrainView *strain_view(const Engine &e) { return e.strain ? &e.strain->view : nullptr; }

int launch_strain_derive(const Engine &e, int nk, cudaStream_t st) {
  const StrainView &v = e.strain->view;
  if (v.n <= 0) return NRT_OK;
  if (!v.tab || nk > kChunk) return NRT_EINVAL;
  const int64_t entries = (int64_t)nk * v.ncls;
  NRT_CUDA(launch_chained(strain_derive, (unsigned)((entries + kStrainBlock - 1) / kStrainBlock),
                          kStrainBlock, 0, st, v, e.pv, nk));
  return NRT_OK;
}

int launch_strain_apply(const Engine &e, int k, cudaStream_t st) {
  const StrainView &v = e.strain->view;
  if (v.n <= 0) return NRT_OK;
  if (!v.tab || k < 0 || k >= kChunk) return NRT_EINVAL;
  NRT_CUDA(launch_chained(strain_apply, (v.n + 255) / 256, 256, 0, st, v, e.pv, k,
                          (int)(e.opt.precision == NRT_MIXED)));
  return NRT_OK;
}

void Engine::strain_release() {
  delete strain;
  strain = nullptr;
}

int Engine::strain_config(const nrt_strain_config *c) {
  if (!c) {
    set_error("null strain configuration");
    return NRT_EINVAL;
  }
  if (opt.mode != NRT_EXPLICIT) {
    set_error("time-varying strain is implemented for the explicit stepper only");
    return NRT_EINVAL;
  }
  const int32_t n = c->num_elem;
  if (n < 0 || (n > 0 && (!c->element || !c->kind || !c->dspec)) || !(c->t1 > c->t0) ||
      !(c->e_max > 0)) {
    set_error("bad strain configuration (sizes, null arrays, t1 <= t0 or e_max <= 0)");
    return NRT_EINVAL;
  }
  std::vector<int64_t> elem(n), col(n, -1);
  std::vector<int32_t> inst(n), kind(n);
  for (int32_t q = 0; q < n; q++) {
    const int32_t in = c->instance ? c->instance[q] : 0;
    if (in < 0 || in >= host.ninst || c->element[q] < 0 || c->element[q] >= host.num_elem[in]) {
      set_error("strained element " + std::to_string(q) + " names no element of its instance");
      return NRT_EINVAL;
    }
    elem[q] = host.off[in] + c->element[q];
    inst[q] = in;
    kind[q] = c->kind[q];
    if ((kind[q] == 1) != ((host.topo[elem[q]].flags & F_HH) != 0)) {
      set_error("strained element " + std::to_string(q) + ": kind differs from the tree's");
      return NRT_EINVAL;
    }
  }
  NRT_CUDA(cudaStreamSynchronize(stream));
  for (int q = 0; q < 2; q++)  // the graphs of the time loop gain (or lose) a launch
    if (graph_exec[q]) {
      cudaGraphExecDestroy(graph_exec[q]);
      graph_exec[q] = nullptr;
    }
  strain_release();
  if (n == 0) return NRT_OK;
  std::unique_ptr<StrainState> S(new (std::nothrow) StrainState());
  if (!S) {
    set_error("host allocation");
    return NRT_ENOMEM;
  }
  // every strained HH element gets a parameter column of its own
  const bool mixed = opt.precision == NRT_MIXED;
  const int64_t N = host.ntot, L0 = host.hp_ld;
  std::vector<int64_t> hh_q;
  for (int32_t q = 0; q < n; q++)
    if (kind[q] == 1) hh_q.push_back(q);
  const bool per_element = !host.hp_inst && host.hp_cls.empty();
  if (per_element) {
    for (int64_t q : hh_q) col[q] = elem[q];
  } else if (!hh_q.empty()) {
    const int64_t L1 = L0 + (int64_t)hh_q.size();
    std::vector<double> hp((size_t)HP_ROWS * L1);
    for (int r = 0; r < HP_ROWS; r++)
      for (int64_t cc = 0; cc < L0; cc++) hp[(size_t)r * L1 + cc] = host.hp[(size_t)r * L0 + cc];
    hvec<uint32_t> cls(N);  // every entry written below
    for (int32_t i = 0; i < host.ninst; i++)
      for (int64_t j = host.off[i]; j < host.off[i + 1]; j++)
        cls[j] = host.hp_cls.empty() ? (uint32_t)i : host.hp_cls[j];
    for (size_t k = 0; k < hh_q.size(); k++) {
      const int64_t q = hh_q[k], j = elem[q], old = cls[j], nc = L0 + (int64_t)k;
      for (int r = 0; r < HP_ROWS; r++) hp[(size_t)r * L1 + nc] = hp[(size_t)r * L1 + old];
      cls[j] = (uint32_t)nc;
      col[q] = nc;
    }
    void *d_tab = nullptr, *d_cls = nullptr;
    const size_t tab_bytes = mixed ? (size_t)12 * 4 * L1 : (size_t)HP_ROWS * 8 * L1;
    if (cudaMalloc(&d_tab, tab_bytes) != cudaSuccess || cudaMalloc(&d_cls, 4 * (size_t)N) != cudaSuccess) {
      cudaGetLastError();
      if (d_tab) cudaFree(d_tab);
      set_error("device allocation for the strained parameter table");
      return NRT_ENOMEM;
    }
    extra_mem.push_back(d_tab);  // the pack reads these from now on: freed with the engine
    extra_mem.push_back(d_cls);
    std::vector<float> q32;
    if (mixed) {
      q32.assign((size_t)12 * L1, 0.0f);
      for (int64_t cc = 0; cc < L1; cc++)
        for (int r = 0; r < HP_ROWS; r++) q32[12 * cc + r] = (float)hp[(size_t)r * L1 + cc];
    }
    NRT_CUDA(cudaMemcpyAsync(d_tab, mixed ? (const void *)q32.data() : (const void *)hp.data(),
                             tab_bytes, cudaMemcpyHostToDevice, stream));
    NRT_CUDA(cudaMemcpyAsync(d_cls, cls.data(), 4 * (size_t)N, cudaMemcpyHostToDevice, stream));
    NRT_CUDA(cudaStreamSynchronize(stream));
    if (mixed)
      pv.hpq = (const float4 *)d_tab;
    else
      pv.hp = (const double *)d_tab;
    pv.hp_cls = (const uint32_t *)d_cls;
    pv.hp_ld = L1;
    pv.hp_inst = 0;
    host.hp.swap(hp);
    host.hp_cls.swap(cls);
    host.hp_ld = L1;
    host.hp_inst = false;
  }
  // classes of identical input columns (instance, kind, the ten description values used:
  // no epsilon, no input), the elements sorted by class
  const int rows[10] = {0, 1, 4, 5, 6, 7, 8, 9, 10, 11};
  constexpr int kKey = 11;
  std::vector<uint64_t> key((size_t)kKey * n);
  for (int32_t q = 0; q < n; q++) {
    key[(size_t)kKey * q] = ((uint64_t)(uint32_t)inst[q] << 1) | (uint64_t)(kind[q] == 1);
    for (int r = 0; r < 10; r++)
      std::memcpy(&key[(size_t)kKey * q + 1 + r], &c->dspec[(size_t)rows[r] * n + q], 8);
  }
  std::vector<int32_t> order(n);
  for (int32_t q = 0; q < n; q++) order[q] = q;
  auto key_less = [&](int32_t x, int32_t y) {
    return std::lexicographical_compare(&key[(size_t)kKey * x], &key[(size_t)kKey * x + kKey],
                                        &key[(size_t)kKey * y], &key[(size_t)kKey * y + kKey]);
  };
  std::stable_sort(order.begin(), order.end(), key_less);
  std::vector<int64_t> s_elem(n), s_col(n);
  std::vector<int32_t> s_cls(n), first;  // first: one member of each class
  for (int32_t r = 0; r < n; r++) {
    const int32_t q = order[r];
    if (r == 0 || key_less(order[r - 1], q)) first.push_back(q);
    s_elem[r] = elem[q];
    s_col[r] = col[q];
    s_cls[r] = (int32_t)first.size() - 1;
  }
  const int32_t ncls = (int32_t)first.size();
  std::vector<int32_t> c_inst(ncls), c_kind(ncls);
  std::vector<double> c_spec((size_t)10 * ncls);
  for (int32_t k = 0; k < ncls; k++) {
    c_inst[k] = inst[first[k]];
    c_kind[k] = kind[first[k]];
    for (int r = 0; r < 10; r++)
      c_spec[(size_t)r * ncls + k] = c->dspec[(size_t)rows[r] * n + first[k]];
  }
  // the table a graph chunk derives ahead, when it stays small (64 MiB); otherwise each
  // step derives its own coefficients
  const size_t tab_entries = (size_t)kChunk * ncls;
  const bool tabled = tab_entries * (8 * kStrainOut + 4) <= ((size_t)64 << 20);
  // mixed, with the table: a second copy of the coefficient rows and of the parameter
  // table, for the steps of a graph chunk that write the next step's rows (StrainFold)
  const bool alt = tabled && mixed;
  auto rnd = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t fold_bytes = alt ? 4 * rnd(4 * (size_t)N) + rnd(48 * (size_t)pv.hp_ld) : 0;
  const size_t bytes = 8 * (size_t)n * 2 + 4 * (size_t)n + 4 * (size_t)ncls * 2 +
                       8 * c_spec.size() +
                       (tabled ? tab_entries * (8 * kStrainOut + 4) : 0) + fold_bytes + 256 * 8;
  if (cudaMalloc(&S->mem, bytes) != cudaSuccess) {
    cudaGetLastError();
    set_error("device allocation for the strain");
    return NRT_ENOMEM;
  }
  char *m = (char *)S->mem;
  auto take = [&](size_t b) {
    char *r = m;
    m += (b + 255) & ~(size_t)255;
    return (void *)r;
  };
  StrainView &v = S->view;
  int64_t *d_elem = (int64_t *)take(8 * (size_t)n), *d_col = (int64_t *)take(8 * (size_t)n);
  int32_t *d_cls = (int32_t *)take(4 * (size_t)n);
  int32_t *d_inst = (int32_t *)take(4 * (size_t)ncls), *d_kind = (int32_t *)take(4 * (size_t)ncls);
  double *d_spec = (double *)take(8 * c_spec.size());
  v.tab = tabled ? (double *)take(8 * kStrainOut * tab_entries) : nullptr;
  v.tlive = tabled ? (int32_t *)take(4 * tab_entries) : nullptr;
  v.alt_cdtf = alt ? (float *)take(4 * (size_t)N) : nullptr;
  v.alt_gaxf = alt ? (float *)take(4 * (size_t)N) : nullptr;
  v.alt_wdxf = alt ? (float *)take(4 * (size_t)N) : nullptr;
  v.alt_kdxf = alt ? (float *)take(4 * (size_t)N) : nullptr;
  v.alt_hpq = alt ? (float4 *)take(48 * (size_t)pv.hp_ld) : nullptr;
  NRT_CUDA(cudaMemcpyAsync(d_elem, s_elem.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaMemcpyAsync(d_col, s_col.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaMemcpyAsync(d_cls, s_cls.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaMemcpyAsync(d_inst, c_inst.data(), 4 * (size_t)ncls, cudaMemcpyHostToDevice,
                           stream));
  NRT_CUDA(cudaMemcpyAsync(d_kind, c_kind.data(), 4 * (size_t)ncls, cudaMemcpyHostToDevice,
                           stream));
  NRT_CUDA(cudaMemcpyAsync(d_spec, c_spec.data(), 8 * c_spec.size(), cudaMemcpyHostToDevice,
                           stream));
  NRT_CUDA(cudaStreamSynchronize(stream));
  v.n = n;
  v.ncls = ncls;
  v.elem = d_elem;
  v.col = d_col;
  v.cls = d_cls;
  v.inst = d_inst;
  v.kind = d_kind;
  v.spec = d_spec;
  v.myelin = c->myelin;
  v.e_max = c->e_max;
  v.eps0 = c->eps0;
  v.eps1 = c->eps1;
  v.t0 = c->t0;
  v.t1 = c->t1;
  if (alt) {  // unstrained elements keep the same coefficients in both copies for good
    const auto d2d = cudaMemcpyDeviceToDevice;
    NRT_CUDA(cudaMemcpyAsync(v.alt_cdtf, pv.cdtf, 4 * (size_t)N, d2d, stream));
    NRT_CUDA(cudaMemcpyAsync(v.alt_gaxf, pv.gaxf, 4 * (size_t)N, d2d, stream));
    NRT_CUDA(cudaMemcpyAsync(v.alt_wdxf, pv.wdxf, 4 * (size_t)N, d2d, stream));
    NRT_CUDA(cudaMemcpyAsync(v.alt_kdxf, pv.kdxf, 4 * (size_t)N, d2d, stream));
    NRT_CUDA(cudaMemcpyAsync(v.alt_hpq, pv.hpq, 48 * (size_t)pv.hp_ld, d2d, stream));
  }
  NRT_CUDA(cudaStreamSynchronize(stream));
  strain = S.release();
  return NRT_OK;
}

}  // namespace nrt
