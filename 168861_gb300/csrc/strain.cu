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
#include <vector>

#include "derive_elem.h"
#include "nrt_solver.h"

namespace nrt {

struct StrainView {
  int32_t n;
  const int64_t *elem;   // global element index
  const int32_t *inst;   // instance (time and dT)
  const int32_t *kind;   // 1 HH / 0 cable
  const int64_t *col;    // parameter column of an HH element
  const double *spec;    // [10][n]: dX, diameter, ro_a, ro_m, per_m, thickness, rest, sigma_Na, sigma_K, sigma_L
  int32_t myelin;
  double e_max, eps0, eps1, t0, t1;
};

struct StrainState {
  void *mem = nullptr;
  StrainView view{};
  ~StrainState() {
    if (mem) cudaFree(mem);
  }
};

namespace {

__global__ void strain_update(StrainView s, PackView p, int k, int mixed) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.n) return;
  const InstDev in = p.inst[s.inst[q]];
  const int64_t i = in.base + k;
  if (i >= in.iend) return;
  const double t = (double)i * in.dT;
  const double e = t <= s.t0 ? s.eps0
                             : (t >= s.t1 ? s.eps1
                                          : s.eps0 + (s.eps1 - s.eps0) * ((t - s.t0) / (s.t1 - s.t0)));
  nrt_param::ElemIn x;
  x.kind = s.kind[q];
  x.dX0 = s.spec[q];
  x.diam0 = s.spec[s.n + q];
  x.eps = e;
  x.ro_a = s.spec[2 * s.n + q];
  x.ro_m = s.spec[3 * s.n + q];
  x.per_m = s.spec[4 * s.n + q];
  x.th = s.spec[5 * s.n + q];
  x.rest = s.spec[6 * s.n + q];
  x.sna = s.spec[7 * s.n + q];
  x.sk = s.spec[8 * s.n + q];
  x.sl = s.spec[9 * s.n + q];
  double ep[6], hp[12];
  nrt_param::derive_element(x, s.myelin, s.e_max, ep, hp);
  const int64_t j = s.elem[q];
  const double c_m = ep[0], r_a = ep[1], dx = ep[2];
  const double cdt = in.dT / (c_m * dx), gax = 1.0 / (r_a * dx);  // as the pack builds them
  if (mixed) {
    ((float *)p.cdtf)[j] = (float)cdt;
    ((float *)p.gaxf)[j] = (float)gax;
  } else {
    ((double *)p.cdt)[j] = cdt;
    ((double *)p.gax)[j] = gax;
  }
  if (x.kind == 1) {
    double v[HP_ROWS];
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
    const int64_t c = s.col[q];
    if (mixed) {
      float *col = (float *)(p.hpq + 3 * c);
      for (int r = 0; r < HP_ROWS; r++) col[r] = (float)v[r];
    } else {
      for (int r = 0; r < HP_ROWS; r++) ((double *)p.hp)[r * p.hp_ld + c] = v[r];
    }
  } else if (mixed) {
    ((float *)p.wdxf)[j] = (float)(ep[3] * dx);
    ((float *)p.kdxf)[j] = (float)(ep[4] * dx);
  } else {
    ((double *)p.wdx)[j] = ep[3] * dx;
    ((double *)p.kdx)[j] = ep[4] * dx;
  }
}

}  // namespace

int launch_strain_update(const Engine &e, int k, cudaStream_t st) {
  const StrainView &v = e.strain->view;
  if (v.n <= 0) return NRT_OK;
  // one warp per block: the FP64 re-derivation is bound by each SM's FP64 pipe, so the
  // elements are spread over as many SMs as there are warps of them
  strain_update<<<(v.n + 31) / 32, 32, 0, st>>>(v, e.pv, k, e.opt.precision == NRT_MIXED);
  NRT_CUDA(cudaGetLastError());
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
  StrainState *S = new (std::nothrow) StrainState();
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
    std::vector<uint32_t> cls(N);
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
      delete S;
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
  // the strained elements' description, unstrained
  std::vector<double> spec((size_t)10 * n);
  const int rows[10] = {0, 1, 4, 5, 6, 7, 8, 9, 10, 11};  // dspec rows used (no epsilon, input)
  for (int r = 0; r < 10; r++)
    for (int32_t q = 0; q < n; q++) spec[(size_t)r * n + q] = c->dspec[(size_t)rows[r] * n + q];
  const size_t bytes = 8 * (size_t)n * 2 + 4 * (size_t)n * 2 + 8 * spec.size() + 256 * 4;
  if (cudaMalloc(&S->mem, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete S;
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
  int32_t *d_inst = (int32_t *)take(4 * (size_t)n), *d_kind = (int32_t *)take(4 * (size_t)n);
  double *d_spec = (double *)take(8 * spec.size());
  NRT_CUDA(cudaMemcpyAsync(d_elem, elem.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaMemcpyAsync(d_col, col.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaMemcpyAsync(d_inst, inst.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaMemcpyAsync(d_kind, kind.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaMemcpyAsync(d_spec, spec.data(), 8 * spec.size(), cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaStreamSynchronize(stream));
  v.n = n;
  v.elem = d_elem;
  v.inst = d_inst;
  v.kind = d_kind;
  v.col = d_col;
  v.spec = d_spec;
  v.myelin = c->myelin;
  v.e_max = c->e_max;
  v.eps0 = c->eps0;
  v.eps1 = c->eps1;
  v.t0 = c->t0;
  v.t1 = c->t1;
  strain = S;
  return NRT_OK;
}

}  // namespace nrt
