// C ABI of the solver hot path: validation, packing into device-resident SoA, handles,
// CUDA-graph time loops, batches.  Declared in include/neurite_gb300.h.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <atomic>
#include <memory>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "nrt_internal.h"
#include "nrt_solver.h"
#include "strain.cuh"

namespace nrt {

namespace {
thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};  // kernels launched by this library (all threads)
}

void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_total() { return g_launches.load(std::memory_order_relaxed); }

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? NRT_ENOMEM : NRT_EDEVICE;
}

static int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

// ------------------------------------------------------------------ validation

// Checks one tree.  strict = the numbering convention that the reference's implicit
// assembly relies on (src/solverIm-cpu.cpp:86-145 detects terminals through
// element[j+1].DR == j+1 and takes mother as the only lower column).
static int validate_problem(const nrt_problem *p, bool strict, std::string &why) {
  if (!p) return (why = "null problem", NRT_EINVAL);
  const int32_t n = p->num_elem;
  if (n < 4) return (why = "num_elem must be >= 4", NRT_EINVAL);
  if (!p->mother || !p->dr || !p->dl || !p->branching || !p->terminals || !p->dx || !p->c_m ||
      !p->r_a || !p->W || !p->K || !p->input || !p->V0)
    return (why = "null element array", NRT_EINVAL);
  if (p->num_term < 1) return (why = "num_term must be >= 1", NRT_EINVAL);
  if (!(p->dT > 0)) return (why = "dT must be > 0", NRT_EINVAL);
  if (p->num_hh < 0 || p->num_hh > n) return (why = "bad num_hh", NRT_EINVAL);
  if (p->num_hh > 0 && (!p->hh_elem || !p->m || !p->h || !p->n || !p->g_Na || !p->g_K ||
                        !p->G_L || !p->E_Na || !p->E_K || !p->E_L || !p->ls_Na || !p->ls_K ||
                        !p->rest))
    return (why = "null HH array", NRT_EINVAL);
  std::vector<char> is_term(n, 0);
  for (int32_t q = 0; q < p->num_term; q++) {
    int32_t t = p->terminals[q];
    if (t < 0 || t >= n) return (why = "terminal index out of range", NRT_ETOPOLOGY);
    is_term[t] = 1;
  }
  if (p->terminals[0] + 1 >= n) return (why = "terminals[0] + 1 out of range", NRT_ETOPOLOGY);
  for (int32_t j = 0; j < n; j++) {
    const int32_t m = p->mother[j], r = p->dr[j], l = p->dl[j];
    if (r < 0 || r >= n || l < 0 || l >= n) return (why = "DR/DL out of range", NRT_ETOPOLOGY);
    if (j > 0 && (m < 0 || m >= n)) return (why = "mother out of range", NRT_ETOPOLOGY);
    if (j == 0 && m != -1 && (m < 0 || m >= n)) return (why = "mother out of range", NRT_ETOPOLOGY);
    if (p->branching[j] != 0 && p->branching[j] != 1) return (why = "branching must be 0/1", NRT_EINVAL);
  }
  for (int32_t q = 1; q < p->num_term; q++) {
    const int32_t t = p->terminals[q];
    if (t == 0 || p->mother[t] < 0) return (why = "terminal without a mother", NRT_ETOPOLOGY);
    if (is_term[p->mother[t]]) return (why = "terminal whose mother is a terminal", NRT_ETOPOLOGY);
  }
  if (is_term[p->terminals[0] + 1]) return (why = "terminals[0] + 1 is a terminal", NRT_ETOPOLOGY);
  int32_t prev = -1;
  for (int32_t k = 0; k < p->num_hh; k++) {
    const int32_t e = p->hh_elem[k];
    if (e < 0 || e >= n || e <= prev) return (why = "hh_elem must be ascending and in range", NRT_EINVAL);
    prev = e;
  }
  if (strict) {
    if (p->terminals[0] != 0 || p->mother[0] != -1) return (why = "element 0 must be the fictitious root", NRT_ETOPOLOGY);
    if (!is_term[n - 1]) return (why = "the last element must be a terminal", NRT_ETOPOLOGY);
    for (int32_t j = 1; j < n; j++) {
      const int32_t m = p->mother[j];
      if (m >= j) return (why = "a mother must precede its child", NRT_ETOPOLOGY);
      if (is_term[j]) {
        if (p->dr[j] != j) return (why = "a terminal must have DR == itself", NRT_ETOPOLOGY);
        // the reference's assembly turns the row after a terminal's mother into the
        // identity row, so a terminal must directly follow its mother
        if (m != j - 1) return (why = "a terminal's mother must be the previous element", NRT_ETOPOLOGY);
      } else {
        if (p->dr[j] != j + 1 || p->mother[j + 1] != j)
          return (why = "non-terminal elements need DR == j + 1 with mother j", NRT_ETOPOLOGY);
      }
      if (p->branching[j]) {
        const int32_t l = p->dl[j];
        if (l <= j || p->mother[l] != j) return (why = "DL must be a later element whose mother is the branch point", NRT_ETOPOLOGY);
        if (is_term[j + 1] || is_term[l])
          return (why = "a branch point's children must not be terminals", NRT_ETOPOLOGY);
      } else if (p->dl[j] != 0) {
        return (why = "DL must be 0 off branch points", NRT_ETOPOLOGY);
      }
      if (m != j - 1 && !(p->branching[m] && p->dl[m] == j))
        return (why = "an element's mother must be j-1 unless it is a DL child", NRT_ETOPOLOGY);
    }
    if (is_term[1] || is_term[2] || p->branching[1])
      return (why = "the root branch needs at least two plain compartments", NRT_ETOPOLOGY);
  }
  return NRT_OK;
}

// ------------------------------------------------------------------ packing

namespace {

// One HH parameter set in HP_* row order.
struct HHKey {
  double v[HP_ROWS];
  bool operator==(const HHKey &o) const { return memcmp(v, o.v, sizeof(v)) == 0; }
};
struct HHKeyHash {
  size_t operator()(const HHKey &k) const {
    uint64_t h = 1469598103934665603ull;  // FNV-1a over the bytes
    const unsigned char *b = (const unsigned char *)k.v;
    for (size_t q = 0; q < sizeof(k.v); q++) h = (h ^ b[q]) * 1099511628211ull;
    return (size_t)h;
  }
};

HHKey hh_key(const nrt_problem &p, int32_t k) {
  HHKey key;
  key.v[HP_GNA] = p.g_Na[k];
  key.v[HP_GK] = p.g_K[k];
  key.v[HP_GL] = p.G_L[k];
  key.v[HP_ENA] = p.E_Na[k];
  key.v[HP_EK] = p.E_K[k];
  key.v[HP_EL] = p.E_L[k];
  key.v[HP_LSNA] = p.ls_Na[k];
  key.v[HP_LSK] = p.ls_K[k];
  key.v[HP_REST] = p.rest[k];
  key.v[HP_DX] = p.dx[p.hh_elem[k]];
  key.v[HP_DTMS] = p.dT * 1000;  // src/solverEx-cpu.cpp:96
  return key;
}

}  // namespace

int build_host_pack(const nrt_problem *probs, int32_t count, HostPack &hp) {
  hp.ninst = count;
  hp.off.assign(count + 1, 0);
  hp.hh_off.assign(count + 1, 0);
  std::vector<int64_t> term_off(count + 1, 0);
  for (int32_t i = 0; i < count; i++) {
    hp.off[i + 1] = hp.off[i] + probs[i].num_elem;
    hp.hh_off[i + 1] = hp.hh_off[i] + probs[i].num_hh;
    term_off[i + 1] = term_off[i] + probs[i].num_term;
  }
  const int64_t N = hp.ntot = hp.off[count];
  if (N >= ((int64_t)1 << 31)) return fail(NRT_EINVAL, "total elements exceed 2^31");
  if (count >= (1 << (32 - INST_SHIFT))) return fail(NRT_EINVAL, "too many instances");
  hp.topo.resize(N);
  hp.cdt.resize(N); hp.gax.resize(N); hp.wdx.resize(N); hp.kdx.resize(N); hp.inp.resize(N);
  hp.V0.resize(N); hp.V1.resize(N);
  hp.c_m_dx.resize(N); hp.radx.resize(N); hp.Wfull.resize(N); hp.Kfull.resize(N);
  hp.gate.resize(3 * N);  // zeroed per instance below, HH entries then set
  hp.inst.resize(count);
  hp.num_elem.resize(count);
  hp.hh_local.resize(hp.hh_off[count]);
  hp.terms.resize(term_off[count]);
  // Per instance: everything element-indexed, plus the instance's distinct HH parameter
  // sets in order of first appearance and each HH element's index among them.
  std::vector<char> fusable(count, 1), invariant(count, 1);
  std::vector<std::vector<HHKey>> local_keys(count);
  hvec<uint32_t> cls(N);  // written per instance below (no serial zero fill)
  parallel_for(count, [&](int32_t i) {
    const nrt_problem &p = probs[i];
    const int64_t o = hp.off[i];
    const int32_t n = p.num_elem;
    hp.num_elem[i] = n;
    std::vector<char> is_term(n, 0);
    for (int32_t q = 0; q < p.num_term; q++) is_term[p.terminals[q]] = 1;
    std::vector<char> is_hh(n, 0);
    for (int32_t k = 0; k < p.num_hh; k++) is_hh[p.hh_elem[k]] = 1;
    auto src_of = [&](int32_t t_) { return t_ == p.terminals[0] ? t_ + 1 : p.mother[t_]; };
    for (int32_t j = 0; j < n; j++) {
      Topo t;
      t.mother = (int32_t)(o + (p.mother[j] >= 0 ? p.mother[j] : j));
      t.dr = (int32_t)(o + p.dr[j]);
      t.dl = (int32_t)(o + (p.branching[j] ? p.dl[j] : j));
      uint32_t f = 0;
      if (is_hh[j]) f |= F_HH;
      if (p.branching[j]) f |= F_BRANCH;
      if (is_term[j]) f |= F_TERM;
      if (j == p.terminals[0]) f |= F_ROOT;
      if (p.input[j] != 0.0) f |= F_INP;
      if (p.branching[j] || is_term[j] || j == p.terminals[0] || p.mother[j] != j - 1 ||
          p.dr[j] != j + 1)
        f |= F_XTOPO;
      // Flux through a terminal neighbour is zero when that terminal copies this element.
      if (!is_term[j]) {
        if (p.branching[j] && is_term[p.dl[j]]) {
          if (src_of(p.dl[j]) == j) f |= F_DL_TERM; else fusable[i] = 0;
        }
        if (is_term[p.dr[j]]) {
          if (src_of(p.dr[j]) == j) f |= F_DR_TERM; else fusable[i] = 0;
        }
        if (p.mother[j] >= 0 && is_term[p.mother[j]]) {
          if (src_of(p.mother[j]) == j) f |= F_MO_TERM; else fusable[i] = 0;
        }
      }
      t.flags = f | ((uint32_t)i << INST_SHIFT);
      hp.topo[o + j] = t;
      cls[o + j] = 0;  // HH elements get their class below
      const double dx = p.dx[j], c_m = p.c_m[j], r_a = p.r_a[j];
      hp.cdt[o + j] = p.dT / (c_m * dx);     // dT/(c_m dX), src/solverEx-cpu.cpp:141
      hp.gax[o + j] = 1.0 / (r_a * dx);      // 1/(r_a dX)
      hp.wdx[o + j] = p.W[j] * dx;
      hp.kdx[o + j] = p.K[j] * dx;
      hp.inp[o + j] = p.input[j];
      hp.V0[o + j] = p.V0[j];
      hp.V1[o + j] = p.V1 ? p.V1[j] : p.V0[j];
      hp.c_m_dx[o + j] = c_m * dx;
      hp.radx[o + j] = r_a * dx;
      hp.Wfull[o + j] = p.W[j];
      hp.Kfull[o + j] = p.K[j];
      hp.gate[o + j] = hp.gate[N + o + j] = hp.gate[2 * N + o + j] = 0.0;
    }
    for (int32_t q = 0; q < p.num_term; q++) {
      const int32_t t = p.terminals[q];
      hp.terms[term_off[i] + q] = o + t;
      const int32_t src = (q == 0 || t == p.terminals[0]) ? t + 1 : p.mother[t];
      if (p.V0[t] != p.V0[src]) invariant[i] = 0;
    }
    std::vector<HHKey> &keys = local_keys[i];
    uint32_t prev = UINT32_MAX;
    for (int32_t k = 0; k < p.num_hh; k++) {
      const int64_t e = o + p.hh_elem[k];
      hp.hh_local[hp.hh_off[i] + k] = p.hh_elem[k];
      hp.gate[e] = p.m[k];
      hp.gate[N + e] = p.h[k];
      hp.gate[2 * N + e] = p.n[k];
      const HHKey key = hh_key(p, k);
      if (prev == UINT32_MAX || !(key == keys[prev])) {
        prev = UINT32_MAX;
        for (size_t c = 0; c < keys.size() && c < 64; c++)
          if (keys[c] == key) {
            prev = (uint32_t)c;
            break;
          }
        if (prev == UINT32_MAX) {
          prev = (uint32_t)keys.size();
          keys.push_back(key);
        }
      }
      cls[e] = prev;
    }
    InstDev in;
    in.base = 0;
    in.iend = INT64_MAX;
    in.dT = p.dT;
    in.t0 = 0;
    in.t1 = -1;
    set_window(in);
    hp.inst[i] = in;
  });
  hp.fusable = std::all_of(fusable.begin(), fusable.end(), [](char c) { return c != 0; });
  hp.invariant = std::all_of(invariant.begin(), invariant.end(), [](char c) { return c != 0; });
  // HH parameter columns.  One per instance when every HH element of each instance
  // carries the same parameters; else one per distinct set (class), merged across
  // instances in instance order, while there are at most N/4 sets; else one per element.
  hp.hp_inst = true;
  for (int32_t i = 0; i < count; i++)
    if (local_keys[i].size() > 1) hp.hp_inst = false;
  if (hp.hp_inst) {
    hp.hp.assign((size_t)HP_ROWS * count, 0.0);
    for (int32_t i = 0; i < count; i++)
      if (!local_keys[i].empty())
        for (int r = 0; r < HP_ROWS; r++) hp.hp[(size_t)r * count + i] = local_keys[i][0].v[r];
    hp.hp_ld = count;
    return NRT_OK;
  }
  std::unordered_map<HHKey, uint32_t, HHKeyHash> ids;
  std::vector<HHKey> keys;
  std::vector<std::vector<uint32_t>> remap(count);
  bool few = true;
  for (int32_t i = 0; i < count && few; i++) {
    for (const HHKey &k : local_keys[i]) {
      auto it = ids.find(k);
      if (it == ids.end()) {
        it = ids.emplace(k, (uint32_t)keys.size()).first;
        keys.push_back(k);
      }
      remap[i].push_back(it->second);
    }
    few = (int64_t)keys.size() * 4 <= N;
  }
  if (few) {
    parallel_for(count, [&](int32_t i) {
      for (int64_t k = hp.hh_off[i]; k < hp.hh_off[i + 1]; k++) {
        const int64_t e = hp.off[i] + hp.hh_local[k];
        cls[e] = remap[i][cls[e]];
      }
    });
    const size_t nc = keys.size();
    hp.hp.assign((size_t)HP_ROWS * nc, 0.0);
    for (size_t c = 0; c < nc; c++)
      for (int r = 0; r < HP_ROWS; r++) hp.hp[(size_t)r * nc + c] = keys[c].v[r];
    hp.hp_cls.swap(cls);
    hp.hp_ld = (int64_t)nc;
    return NRT_OK;
  }
  hp.hp.assign((size_t)HP_ROWS * N, 0.0);
  parallel_for(count, [&](int32_t i) {
    const nrt_problem &p = probs[i];
    for (int32_t k = 0; k < p.num_hh; k++) {
      const int64_t e = hp.off[i] + p.hh_elem[k];
      const HHKey key = hh_key(p, k);
      for (int r = 0; r < HP_ROWS; r++) hp.hp[(size_t)r * N + e] = key.v[r];
    }
  });
  hp.hp_ld = N;
  return NRT_OK;
}

// ------------------------------------------------------------------ device arena

int Arena::reserve(size_t bytes) {
  if (base) return NRT_EINVAL;
  NRT_CUDA(cudaMalloc(&base, bytes));
  cap = bytes;
  used = 0;
  return NRT_OK;
}

void *Arena::take(size_t bytes) {
  size_t o = (used + 255) & ~(size_t)255;
  if (o + bytes > cap) return nullptr;
  used = o + bytes;
  return (char *)base + o;
}

void Arena::release() {
  if (base) cudaFree(base);
  base = nullptr;
  cap = used = 0;
}

static size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

template <typename T>
static int upload(Arena &a, T *&dst, const T *src, size_t count, cudaStream_t st) {
  dst = (T *)a.take(sizeof(T) * count);
  if (!dst) return fail(NRT_ENOMEM, "arena exhausted");
  if (src) NRT_CUDA(cudaMemcpyAsync(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice, st));
  return NRT_OK;
}

#define TRY(x)                 \
  do {                         \
    int _rc = (x);             \
    if (_rc != NRT_OK) return _rc; \
  } while (0)

int Engine::init(const nrt_problem *probs, int32_t count, const nrt_options *o) {
  opt = *o;
  if (opt.device >= 0) NRT_CUDA(cudaSetDevice(opt.device));
  NRT_CUDA(cudaGetDevice(&device));
  NRT_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  TRY(build_host_pack(probs, count, host));
  const int64_t N = host.ntot;
  const bool mixed = opt.precision == NRT_MIXED;
  // Sizes: V x2, topo, coefficient rows, gates, HH rows, instances, terminals, implicit.
  size_t bytes = 2 * al(8 * N) + al(sizeof(Topo) * N) + al(sizeof(InstDev) * count) +
                 al(8 * host.terms.size() + 8) + al(16);
  const size_t hpn = (size_t)HP_ROWS * host.hp_ld;
  // the explicit step's coefficient rows (the implicit kernel reads its own FP64 rows)
  const bool explicit_rows = opt.mode == NRT_EXPLICIT;
  if (!host.hp_cls.empty()) bytes += al(4 * N);
  if (mixed && explicit_rows) bytes += al(4 * N);  // flags of the compact step
  if (mixed)
    bytes += (explicit_rows ? 7 * al(4 * N) : 0) + al(4 * 3 * N) + al(4 * 12 * (size_t)host.hp_ld);
  else
    bytes += (explicit_rows ? 5 * al(8 * N) : 0) + al(8 * 3 * N) + al(8 * hpn);
  if (opt.mode == NRT_IMPLICIT_BE) {
    size_t ib = 0;
    TRY(implicit_plan(ib));
    bytes += ib;
  }
  TRY(arena.reserve(bytes + 4096));
  cudaStream_t st = stream;
  TRY(upload(arena, V[0], host.V0.data(), N, st));
  TRY(upload(arena, V[1], host.V1.data(), N, st));
  if (mixed && opt.mode == NRT_EXPLICIT) {
    hostf.reserve(10);
    hostf.emplace_back(host.V0.begin(), host.V0.end());
    TRY(upload(arena, Vf[0], hostf.back().data(), N, st));
    hostf.emplace_back(host.V1.begin(), host.V1.end());
    TRY(upload(arena, Vf[1], hostf.back().data(), N, st));
  }
  Topo *topo = nullptr;  // the implicit set-up uploads it once it has set the row flags
  TRY(upload(arena, topo, explicit_rows ? host.topo.data() : nullptr, N, st));
  InstDev *inst = nullptr;
  TRY(upload(arena, inst, host.inst.data(), count, st));
  TRY(upload(arena, terms, host.terms.data(), host.terms.size(), st));
  pv.ntot = N;
  pv.ninst = count;
  pv.hp_ld = host.hp_ld;
  pv.hp_inst = host.hp_inst ? 1 : 0;
  pv.hp_cls = nullptr;
  pv.hh_dense = 2 * (int64_t)host.hh_local.size() >= N ? 1 : 0;
  pv.eflags = nullptr;
  if (mixed && opt.mode == NRT_EXPLICIT) {
    hvec<uint32_t> fl(N);  // every entry written below
    parallel_ranges(N, [&](int64_t a, int64_t b) {
      for (int64_t j = a; j < b; j++) fl[j] = host.topo[j].flags;
    });
    uint32_t *pf = nullptr;
    TRY(upload(arena, pf, fl.data(), N, st));
    pv.eflags = pf;
    NRT_CUDA(cudaStreamSynchronize(st));  // fl is a local buffer
  }
  if (!host.hp_cls.empty()) {
    uint32_t *pc = nullptr;
    TRY(upload(arena, pc, host.hp_cls.data(), N, st));
    pv.hp_cls = pc;
  }
  pv.topo = topo;
  pv.inst = inst;
  // [0] the device error word; [4..7] the explicit chunk kernel's barrier words
  int *err = nullptr;
  TRY(upload(arena, err, (const int *)nullptr, 8, st));
  NRT_CUDA(cudaMemsetAsync(err, 0, 32, st));
  pv.err = err;
  gbar = (GridBar *)(err + 4);
  pv.tile_blocks = (mixed && opt.mode == NRT_EXPLICIT && opt.tiled != 0)
                       ? explicit_tile_blocks(device, N, opt.tile_ctas_per_sm) : 0;
  pv.step_threads = opt.step_threads;
  NRT_CUDA(cudaDeviceGetAttribute(&pv.sms, cudaDevAttrMultiProcessorCount, device));
  if (mixed) {
    auto f32 = [&](const auto &v) {
      hostf.emplace_back(v.size());
      float *d = hostf.back().data();
      const double *src = v.data();
      parallel_ranges((int64_t)v.size(), [&](int64_t a, int64_t b) {
        for (int64_t q = a; q < b; q++) d[q] = (float)src[q];
      });
      return d;
    };
    hostf.reserve(8);
    float *p;
    if (explicit_rows) {
      TRY(upload(arena, p, f32(host.cdt), N, st)); pv.cdtf = p;
      TRY(upload(arena, p, f32(host.gax), N, st)); pv.gaxf = p;
      TRY(upload(arena, p, f32(host.wdx), N, st)); pv.wdxf = p;
      TRY(upload(arena, p, f32(host.kdx), N, st)); pv.kdxf = p;
      TRY(upload(arena, p, f32(host.inp), N, st)); pv.inpf = p;
    }
    TRY(upload(arena, p, f32(host.gate), 3 * N, st)); pv.gatef = p;
    {  // the parameter table by column: 12 floats (HP_* rows and a pad) per column
      const int64_t L = host.hp_ld;
      hostf.emplace_back((size_t)12 * L, 0.0f);
      float *q = hostf.back().data();
      for (int64_t c = 0; c < L; c++)
        for (int r = 0; r < HP_ROWS; r++) q[12 * c + r] = (float)host.hp[(size_t)r * L + c];
      float4 *dq = nullptr;
      TRY(upload(arena, dq, (const float4 *)q, 3 * (size_t)L, st));
      pv.hpq = dq;
    }
  } else {
    double *p;
    if (explicit_rows) {
      TRY(upload(arena, p, host.cdt.data(), N, st)); pv.cdt = p;
      TRY(upload(arena, p, host.gax.data(), N, st)); pv.gax = p;
      TRY(upload(arena, p, host.wdx.data(), N, st)); pv.wdx = p;
      TRY(upload(arena, p, host.kdx.data(), N, st)); pv.kdx = p;
      TRY(upload(arena, p, host.inp.data(), N, st)); pv.inp = p;
    }
    TRY(upload(arena, p, host.gate.data(), 3 * N, st)); pv.gate = p;
    TRY(upload(arena, p, host.hp.data(), hpn, st)); pv.hp = p;
  }
  if (opt.mode == NRT_IMPLICIT_BE) TRY(implicit_init());
  NRT_CUDA(cudaStreamSynchronize(st));
  hostf.clear();
  hostf.shrink_to_fit();
  return NRT_OK;
}

Engine::~Engine() {
  if (device >= 0) cudaSetDevice(device);
  for (int q = 0; q < 2; q++)
    if (graph_exec[q]) cudaGraphExecDestroy(graph_exec[q]);
  if (stream) cudaStreamSynchronize(stream);
  implicit_release();
  record_release();
  strain_release();
  for (void *p : extra_mem) cudaFree(p);
  arena.release();
  if (stream) cudaStreamDestroy(stream);
}

// One loop iteration (update + calculate) for every instance, reading V[cur].
int Engine::step(int k, int force) {
  const bool general = needs_general();
  if (opt.mode == NRT_IMPLICIT_BE) {
    TRY(implicit_step(k, force));
  } else {
    TRY(launch_explicit_step(pv, opt.precision, general || !host.fusable, k, force, V[cur],
                             V[cur ^ 1], Vf[cur], Vf[cur ^ 1], stream));
    if (general || !host.fusable)
      TRY(launch_terminal_fixup(pv.topo, terms, (int64_t)host.terms.size(), V[cur ^ 1],
                                Vf[cur ^ 1], stream));
  }
  cur ^= 1;
  steps_done++;
  general_next = false;
  terminals_dirty = opt.mode == NRT_EXPLICIT;
  return NRT_OK;
}

// State of one instance: V (current buffer), the other buffer (the implicit step's
// V^{n-1}, used for its initial guess), and the gates of its HH elements in HH order.
int Engine::get_state(int32_t q, double *Vc, double *Vo, double *m, double *h, double *n) {
  TRY(fixup());
  const int64_t o = host.off[q], ne = host.num_elem[q], N = host.ntot;
  if (Vc) NRT_CUDA(cudaMemcpyAsync(Vc, V[cur] + o, 8 * ne, cudaMemcpyDeviceToHost, stream));
  if (Vo) NRT_CUDA(cudaMemcpyAsync(Vo, V[cur ^ 1] + o, 8 * ne, cudaMemcpyDeviceToHost, stream));
  const int64_t h0 = host.hh_off[q], nh = host.hh_off[q + 1] - h0;
  if ((m || h || n) && nh > 0) {
    std::vector<double> g(3 * ne);
    if (opt.precision == NRT_MIXED) {
      std::vector<float> gf(3 * ne);
      for (int c = 0; c < 3; c++)
        NRT_CUDA(cudaMemcpyAsync(gf.data() + c * ne, pv.gatef + c * N + o, 4 * ne,
                                 cudaMemcpyDeviceToHost, stream));
      NRT_CUDA(cudaStreamSynchronize(stream));
      for (int64_t k = 0; k < 3 * ne; k++) g[k] = gf[k];
    } else {
      for (int c = 0; c < 3; c++)
        NRT_CUDA(cudaMemcpyAsync(g.data() + c * ne, pv.gate + c * N + o, 8 * ne,
                                 cudaMemcpyDeviceToHost, stream));
    }
    NRT_CUDA(cudaStreamSynchronize(stream));
    for (int64_t k = 0; k < nh; k++) {
      const int64_t el = host.hh_local[h0 + k];
      if (m) m[k] = g[el];
      if (h) h[k] = g[ne + el];
      if (n) n[k] = g[2 * ne + el];
    }
  }
  NRT_CUDA(cudaStreamSynchronize(stream));
  return NRT_OK;
}

int Engine::set_state(int32_t q, const double *Vc, const double *Vo, const double *m,
                      const double *h, const double *n) {
  NRT_CUDA(cudaStreamSynchronize(stream));
  TRY(fixup());
  const int64_t o = host.off[q], ne = host.num_elem[q], N = host.ntot;
  const bool mixed_ex = opt.precision == NRT_MIXED && opt.mode == NRT_EXPLICIT;
  std::vector<float> f(ne);
  auto put_v = [&](int buf, const double *src) -> int {
    NRT_CUDA(cudaMemcpyAsync(V[buf] + o, src, 8 * ne, cudaMemcpyHostToDevice, stream));
    if (mixed_ex && Vf[buf]) {  // the FP32 shadow the explicit stencil reads
      for (int64_t k = 0; k < ne; k++) f[k] = (float)src[k];
      NRT_CUDA(cudaMemcpyAsync(Vf[buf] + o, f.data(), 4 * ne, cudaMemcpyHostToDevice, stream));
      NRT_CUDA(cudaStreamSynchronize(stream));
    }
    return NRT_OK;
  };
  if (Vc) TRY(put_v(cur, Vc));
  if (Vo) TRY(put_v(cur ^ 1, Vo));
  const int64_t h0 = host.hh_off[q], nh = host.hh_off[q + 1] - h0;
  const double *src[3] = {m, h, n};
  for (int c = 0; c < 3; c++) {
    if (!src[c] || nh == 0) continue;
    // read-modify-write of the instance's column: passive elements keep their entries
    if (opt.precision == NRT_MIXED) {
      std::vector<float> g(ne);
      NRT_CUDA(cudaMemcpyAsync(g.data(), pv.gatef + c * N + o, 4 * ne, cudaMemcpyDeviceToHost, stream));
      NRT_CUDA(cudaStreamSynchronize(stream));
      for (int64_t k = 0; k < nh; k++) g[host.hh_local[h0 + k]] = (float)src[c][k];
      NRT_CUDA(cudaMemcpyAsync(pv.gatef + c * N + o, g.data(), 4 * ne, cudaMemcpyHostToDevice, stream));
    } else {
      std::vector<double> g(ne);
      NRT_CUDA(cudaMemcpyAsync(g.data(), pv.gate + c * N + o, 8 * ne, cudaMemcpyDeviceToHost, stream));
      NRT_CUDA(cudaStreamSynchronize(stream));
      for (int64_t k = 0; k < nh; k++) g[host.hh_local[h0 + k]] = src[c][k];
      NRT_CUDA(cudaMemcpyAsync(pv.gate + c * N + o, g.data(), 8 * ne, cudaMemcpyHostToDevice, stream));
    }
    NRT_CUDA(cudaStreamSynchronize(stream));
  }
  // explicit: a terminal that does not copy its source breaks the fused step's invariant;
  // the next step then runs in the general form, as a first step from such a state does
  if (Vc && opt.mode == NRT_EXPLICIT) {
    for (int64_t t : host.terms) {
      if (t < o || t >= o + ne) continue;
      const Topo &tp = host.topo[t];
      const int64_t s = (tp.flags & F_ROOT) ? t + 1 : (int64_t)tp.mother;
      if (Vc[t - o] != Vc[s - o]) general_next = true;
    }
  }
  return NRT_OK;
}

int Engine::fixup() {
  if (!terminals_dirty) return NRT_OK;
  TRY(launch_terminal_fixup(pv.topo, terms, (int64_t)host.terms.size(), V[cur], Vf[cur], stream));
  terminals_dirty = false;
  return NRT_OK;
}

// The explicit time loop runs a chunk of steps per cooperative launch (nrt_options.
// step_launch), in the fused form, with the strain (if any) derived ahead per chunk.
bool Engine::chunk_kernel() const {
  if (opt.mode != NRT_EXPLICIT || !host.fusable || !gbar || opt.step_launch != 1) return false;
  return !strain || strain_tabled(*this);
}

// Runs `steps` loop iterations from every instance's current base (device-side loop
// indices): chunks of up to kChunk steps per launch when asked for, otherwise a captured
// graph of kChunk steps where possible.
int Engine::advance(int64_t steps) {
  if (opt.mode == NRT_IMPLICIT_BE) return implicit_advance(*this, steps);
  int64_t left = steps;
  while (left > 0 && needs_general()) {  // exact first step
    if (strain) TRY(launch_strain_update(*this, 0, stream));
    TRY(step(0, -1));
    if (rec) TRY(launch_record_step(rec_view_host(), pv.inst, 0, V[cur], stream));
    TRY(launch_advance_base(pv.inst, pv.ninst, 1, stream));
    left--;
  }
  if (left > 0 && chunk_kernel()) {
    const RecView none_r{};
    const StrainView none_s{};
    const StrainView *sv = strain_view(*this);
    while (left > 0) {
      const int nk = (int)std::min<int64_t>(left, kChunk);
      if (sv) TRY(launch_strain_derive(*this, nk, stream));
      TRY(launch_explicit_chunk(pv, opt.precision, nk, V[cur], V[cur ^ 1], Vf[cur], Vf[cur ^ 1],
                                rec ? rec_view_host() : none_r, sv ? *sv : none_s, gbar,
                                opt.tile_ctas_per_sm, stream));
      TRY(launch_advance_base(pv.inst, pv.ninst, nk, stream));
      cur ^= nk & 1;
      steps_done += nk;
      left -= nk;
      terminals_dirty = true;
    }
    return NRT_OK;
  }
  const bool graphs = opt.use_graphs != 0 && opt.mode == NRT_EXPLICIT && host.fusable;
  if (graphs && left >= kChunk) {
    if (!graph_exec[cur]) {
      cudaGraph_t g;
      NRT_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      int rc = NRT_OK;
      const bool tabled = strain_tabled(*this);
      // mixed steps write the strained rows of the step after them (StrainFold): one row
      // write per chunk instead of one launch per step; the coefficient rows and the
      // parameter table alternate between two copies by the step's parity
      const StrainView *sv = strain_view(*this);
      const bool fold = tabled && opt.precision == NRT_MIXED && sv && sv->alt_gaxf;
      PackView alt = pv;
      if (fold) {
        alt.cdtf = sv->alt_cdtf;
        alt.gaxf = sv->alt_gaxf;
        alt.wdxf = sv->alt_wdxf;
        alt.kdxf = sv->alt_kdxf;
        alt.hpq = sv->alt_hpq;
      }
      if (tabled) rc = launch_strain_derive(*this, kChunk, stream);
      for (int k = 0; k < kChunk && rc == NRT_OK; k++) {
        if (strain && (!fold || k == 0))
          rc = tabled ? launch_strain_apply(*this, k, stream) : launch_strain_update(*this, k, stream);
        if (rc != NRT_OK) break;
        const PackView &pk = fold && (k & 1) ? alt : pv;
        StrainFold f{};
        f.row = -1;
        if (fold && k + 1 < kChunk) {
          f.s = *sv;
          f.next = (k + 1) & 1 ? alt : pv;
          f.row = k + 1;
        }
        rc = launch_explicit_step(pk, opt.precision, false, k, -1, V[(cur + k) & 1],
                                  V[(cur + k + 1) & 1], Vf[(cur + k) & 1], Vf[(cur + k + 1) & 1],
                                  stream, fold ? &f : nullptr);
        if (rc == NRT_OK && rec)
          rc = launch_record_step(rec_view_host(), pv.inst, k, V[(cur + k + 1) & 1], stream);
      }
      if (rc == NRT_OK) rc = launch_advance_base(pv.inst, pv.ninst, kChunk, stream);
      cudaError_t e = cudaStreamEndCapture(stream, &g);
      if (rc != NRT_OK) return rc;
      NRT_CUDA(e);
      size_t nodes = 0;  // every node of the captured chunk is a kernel of this library
      if (cudaGraphGetNodes(g, nullptr, &nodes) == cudaSuccess) graph_nodes[cur] = (int64_t)nodes;
      e = cudaGraphInstantiate(&graph_exec[cur], g, 0);
      cudaGraphDestroy(g);
      NRT_CUDA(e);
    }
    while (left >= kChunk) {
      NRT_CUDA(cudaGraphLaunch(graph_exec[cur], stream));
      count_launches(graph_nodes[cur]);
      steps_done += kChunk;  // kChunk is even: cur is unchanged
      left -= kChunk;
      terminals_dirty = true;
    }
  }
  while (left > 0) {
    if (strain) TRY(launch_strain_update(*this, 0, stream));
    TRY(step(0, -1));
    if (rec) TRY(launch_record_step(rec_view_host(), pv.inst, 0, V[cur], stream));
    TRY(launch_advance_base(pv.inst, pv.ninst, 1, stream));
    left--;
  }
  return NRT_OK;
}

}  // namespace nrt

using nrt::Engine;

struct nrt_solver {
  Engine eng;
  int pending_input = 0;
  bool have_update = false;
};

struct nrt_batch {
  Engine eng;
  std::vector<nrt_instance_run> runs;
};

extern "C" {

const char *nrt_status_string(int s) {
  switch (s) {
    case NRT_OK: return "ok";
    case NRT_EINVAL: return "invalid argument";
    case NRT_ETOPOLOGY: return "invalid tree topology";
    case NRT_ENOMEM: return "out of memory";
    case NRT_ENOCONV: return "Krylov solve did not converge within its iteration budget";
    case NRT_EDEVICE: return "CUDA device error";
    case NRT_EBUDGET: return "request exceeds the memory budget";
    case NRT_ESTATE: return "call out of order";
    case NRT_ENOTREADY: return "result not ready";
    default: return "unknown status";
  }
}

const char *nrt_last_error(void) { return nrt::g_last_error.c_str(); }

int64_t nrt_kernel_launches(void) { return (int64_t)nrt::launches_total(); }

int nrt_options_default(nrt_options *o) {
  return nrt::guarded([&]() -> int {
    if (!o) return NRT_EINVAL;
    memset(o, 0, sizeof(*o));
    o->mode = NRT_EXPLICIT;
    o->precision = NRT_FP64;
    o->krylov = NRT_GMRES;
    o->precond = NRT_PRECOND_TREE;
    o->restart = 30;
    o->tol_mode = NRT_TOL_ABS;
    o->tol = 1e-14;  // RANGE_ERROR, inc/configuration.h:16
    o->max_iter = 0;
    o->device = -1;
    o->use_graphs = 1;
    o->tiled = 1;
    return NRT_OK;
  });
}

static int check_options(const nrt_options *o, std::string &why) {
  if (o->mode != NRT_EXPLICIT && o->mode != NRT_IMPLICIT_BE) return (why = "bad mode", NRT_EINVAL);
  if (o->precision != NRT_FP64 && o->precision != NRT_MIXED) return (why = "bad precision", NRT_EINVAL);
  if (o->krylov != NRT_GMRES && o->krylov != NRT_BICGSTAB) return (why = "bad krylov", NRT_EINVAL);
  if (o->mode == NRT_IMPLICIT_BE && o->krylov == NRT_BICGSTAB && o->restart < 3)
    return (why = "BiCGSTAB needs restart >= 3 (its eight work vectors share the GMRES basis)", NRT_EINVAL);
  if (o->precond < NRT_PRECOND_NONE || o->precond > NRT_PRECOND_TREE) return (why = "bad precond", NRT_EINVAL);
  if (o->restart < 1 || o->restart > nrt::kMaxRestart) return (why = "restart must be in [1, 32]", NRT_EINVAL);
  if (!(o->tol > 0)) return (why = "tol must be > 0", NRT_EINVAL);
  if (o->max_iter < 0) return (why = "max_iter must be >= 0", NRT_EINVAL);
  if (!(o->inner_tol >= 0 && o->inner_tol < 1)) return (why = "inner_tol must be in [0, 1)", NRT_EINVAL);
  if (o->refinement != 0 && o->refinement != 1) return (why = "refinement must be 0 or 1", NRT_EINVAL);
  if (o->scheme != NRT_BACKWARD_EULER && o->scheme != NRT_CRANK_NICOLSON)
    return (why = "bad scheme", NRT_EINVAL);
  if (o->tile_ctas_per_sm < 0 || o->tile_ctas_per_sm > 64)
    return (why = "tile_ctas_per_sm must be in [0, 64]", NRT_EINVAL);
  if (o->step_threads != 0 && (o->step_threads < 32 || o->step_threads > 256 || o->step_threads % 32))
    return (why = "step_threads must be 0 or a multiple of 32 in [32, 256]", NRT_EINVAL);
  if (o->step_launch != 0 && o->step_launch != 1) return (why = "step_launch must be 0 or 1", NRT_EINVAL);
  return NRT_OK;
}

int nrt_create(const nrt_problem *p, const nrt_options *opt, nrt_solver **out) {
  return nrt::guarded([&]() -> int {
    if (!p || !out) return nrt::fail(NRT_EINVAL, "null argument");
    *out = nullptr;
    nrt_options o;
    if (opt) o = *opt; else nrt_options_default(&o);
    std::string why;
    int rc = check_options(&o, why);
    if (rc) return nrt::fail(rc, why);
    rc = nrt::validate_problem(p, o.mode == NRT_IMPLICIT_BE, why);
    if (rc) return nrt::fail(rc, why);
    std::unique_ptr<nrt_solver> s(new (std::nothrow) nrt_solver());
    if (!s) return nrt::fail(NRT_ENOMEM, "host allocation");
    rc = s->eng.init(p, 1, &o);
    if (rc) return rc;
    *out = s.release();
    return NRT_OK;
  });
}

int nrt_update(nrt_solver *s, int input_active) {
  return nrt::guarded([&]() -> int {
    if (!s) return nrt::fail(NRT_EINVAL, "null solver");
    s->pending_input = input_active ? 1 : 0;
    s->have_update = true;
    return NRT_OK;
  });
}

int nrt_calculate(nrt_solver *s) {
  return nrt::guarded([&]() -> int {
    if (!s) return nrt::fail(NRT_EINVAL, "null solver");
    if (!s->have_update) return nrt::fail(NRT_ESTATE, "calculate() without a preceding update()");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    const int64_t before = s->eng.opt.mode == NRT_IMPLICIT_BE ? nrt::nonconverged_total(s->eng) : 0;
    int rc = s->eng.step(0, s->pending_input);
    s->have_update = false;
    if (rc == NRT_OK && s->eng.opt.mode == NRT_IMPLICIT_BE) {
      const int64_t after = nrt::nonconverged_total(s->eng);
      if (after < 0) return NRT_EDEVICE;
      if (after > before)
        return nrt::fail(NRT_ENOCONV, "implicit step hit its Krylov iteration budget");
    }
    return rc;
  });
}

int nrt_export_system(nrt_solver *s, int input_active, int32_t *row_ptr, int32_t *col, double *val,
                      double *rhs, int32_t *nnz_out) {
  return nrt::guarded([&]() -> int {
    if (!s || !row_ptr || !col || !val || !rhs || !nnz_out) return nrt::fail(NRT_EINVAL, "null argument");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    return nrt::export_system(s->eng, input_active, row_ptr, col, val, rhs, nnz_out);
  });
}

int nrt_snapshot(nrt_solver *s, double *potential) {
  return nrt::guarded([&]() -> int {
    if (!s || !potential) return nrt::fail(NRT_EINVAL, "null argument");
    nrt::Engine &e = s->eng;
    NRT_CUDA(cudaSetDevice(e.device));
    int rc = e.fixup();
    if (rc) return rc;
    NRT_CUDA(cudaMemcpyAsync(potential, e.V[e.cur], sizeof(double) * e.host.ntot,
                             cudaMemcpyDeviceToHost, e.stream));
    NRT_CUDA(cudaStreamSynchronize(e.stream));
    return nrt::implicit_check(e);
  });
}

int nrt_run(nrt_solver *s, int64_t i_begin, int64_t i_end, double init_time, double end_input) {
  return nrt::guarded([&]() -> int {
    if (!s) return nrt::fail(NRT_EINVAL, "null solver");
    if (i_end < i_begin) return nrt::fail(NRT_EINVAL, "i_end < i_begin");
    nrt::Engine &e = s->eng;
    NRT_CUDA(cudaSetDevice(e.device));
    nrt::InstDev in = e.host.inst[0];
    in.base = i_begin;
    in.iend = i_end;
    in.t0 = init_time;
    in.t1 = end_input;
    nrt::set_window(in);
    e.host.inst[0] = in;
    NRT_CUDA(cudaMemcpyAsync(e.pv.inst, &e.host.inst[0], sizeof(in), cudaMemcpyHostToDevice, e.stream));
    const bool implicit = e.opt.mode == NRT_IMPLICIT_BE;
    const int64_t before = implicit ? nrt::nonconverged_total(e) : 0;
    int rc = e.advance(i_end - i_begin);
    if (rc) return rc;
    if (implicit && nrt::nonconverged_total(e) > before)
      rc = nrt::fail(NRT_ENOCONV, "an implicit step hit its Krylov iteration budget");
    // leave the drop-in path's device loop range open again
    e.host.inst[0].base = 0;
    e.host.inst[0].iend = INT64_MAX;
    NRT_CUDA(cudaMemcpyAsync(e.pv.inst, &e.host.inst[0], sizeof(in), cudaMemcpyHostToDevice, e.stream));
    NRT_CUDA(cudaStreamSynchronize(e.stream));
    return rc;
  });
}

int nrt_synchronize(nrt_solver *s) {
  return nrt::guarded([&]() -> int {
    if (!s) return nrt::fail(NRT_EINVAL, "null solver");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    NRT_CUDA(cudaStreamSynchronize(s->eng.stream));
    return nrt::implicit_check(s->eng);
  });
}

int nrt_get_stream(nrt_solver *s, void **stream) {
  return nrt::guarded([&]() -> int {
    if (!s || !stream) return nrt::fail(NRT_EINVAL, "null argument");
    *stream = (void *)s->eng.stream;
    return NRT_OK;
  });
}

int nrt_batch_get_stream(nrt_batch *b, void **stream) {
  return nrt::guarded([&]() -> int {
    if (!b || !stream) return nrt::fail(NRT_EINVAL, "null argument");
    *stream = (void *)b->eng.stream;
    return NRT_OK;
  });
}

int nrt_potential_device(nrt_solver *s, const double **dev_ptr) {
  return nrt::guarded([&]() -> int {
    if (!s || !dev_ptr) return nrt::fail(NRT_EINVAL, "null argument");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    int rc = s->eng.fixup();
    if (rc) return rc;
    *dev_ptr = s->eng.V[s->eng.cur];
    return NRT_OK;
  });
}

int nrt_get_gates(nrt_solver *s, double *m, double *h, double *n) {
  return nrt::guarded([&]() -> int {
    if (!s || !m || !h || !n) return nrt::fail(NRT_EINVAL, "null argument");
    nrt::Engine &e = s->eng;
    NRT_CUDA(cudaSetDevice(e.device));
    const int64_t N = e.host.ntot;
    std::vector<double> g(3 * N);
    if (e.opt.precision == NRT_MIXED) {
      std::vector<float> gf(3 * N);
      NRT_CUDA(cudaMemcpyAsync(gf.data(), e.pv.gatef, sizeof(float) * 3 * N, cudaMemcpyDeviceToHost, e.stream));
      NRT_CUDA(cudaStreamSynchronize(e.stream));
      for (int64_t q = 0; q < 3 * N; q++) g[q] = gf[q];
    } else {
      NRT_CUDA(cudaMemcpyAsync(g.data(), e.pv.gate, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, e.stream));
      NRT_CUDA(cudaStreamSynchronize(e.stream));
    }
    const int64_t nh = e.host.hh_off[1];
    for (int64_t k = 0; k < nh; k++) {
      const int64_t el = e.host.hh_local[k];
      m[k] = g[el];
      h[k] = g[N + el];
      n[k] = g[2 * N + el];
    }
    return NRT_OK;
  });
}

int nrt_get_stats(nrt_solver *s, nrt_stats *st) {
  return nrt::guarded([&]() -> int {
    if (!s || !st) return nrt::fail(NRT_EINVAL, "null argument");
    return s->eng.get_stats(st);
  });
}

int nrt_destroy(nrt_solver *s) {
  return nrt::guarded([&]() -> int {
    delete s;
    return NRT_OK;
  });
}

// ------------------------------------------------------------------ batches

int nrt_batch_create(const nrt_problem *problems, int32_t count, const nrt_options *opt,
                     nrt_batch **out) {
  return nrt::guarded([&]() -> int {
    if (!problems || count < 1 || !out) return nrt::fail(NRT_EINVAL, "bad arguments");
    *out = nullptr;
    nrt_options o;
    if (opt) o = *opt; else nrt_options_default(&o);
    std::string why;
    int rc = check_options(&o, why);
    if (rc) return nrt::fail(rc, why);
    // every instance checked on the host's cores; the first failing one is reported
    std::vector<int> vrc(count, NRT_OK);
    std::vector<std::string> vwhy(count);
    nrt::parallel_for(count, [&](int64_t i) {
      vrc[i] = nrt::validate_problem(&problems[i], o.mode == NRT_IMPLICIT_BE, vwhy[i]);
    });
    for (int32_t i = 0; i < count; i++)
      if (vrc[i]) return nrt::fail(vrc[i], "instance " + std::to_string(i) + ": " + vwhy[i]);
    std::unique_ptr<nrt_batch> b(new (std::nothrow) nrt_batch());
    if (!b) return nrt::fail(NRT_ENOMEM, "host allocation");
    rc = b->eng.init(problems, count, &o);
    if (rc) return rc;
    b->runs.assign(count, nrt_instance_run{0, 0, 0.0, -1.0});
    *out = b.release();
    return NRT_OK;
  });
}

int nrt_batch_set_runs(nrt_batch *b, const nrt_instance_run *runs) {
  return nrt::guarded([&]() -> int {
    if (!b || !runs) return nrt::fail(NRT_EINVAL, "null argument");
    nrt::Engine &e = b->eng;
    NRT_CUDA(cudaSetDevice(e.device));
    for (int32_t i = 0; i < e.pv.ninst; i++) {
      if (runs[i].i_end < runs[i].i_begin) return nrt::fail(NRT_EINVAL, "i_end < i_begin");
      b->runs[i] = runs[i];
      e.host.inst[i].base = runs[i].i_begin;
      e.host.inst[i].iend = runs[i].i_end;
      e.host.inst[i].t0 = runs[i].init_time;
      e.host.inst[i].t1 = runs[i].end_input;
      nrt::set_window(e.host.inst[i]);
    }
    NRT_CUDA(cudaMemcpyAsync(e.pv.inst, e.host.inst.data(), sizeof(nrt::InstDev) * e.pv.ninst,
                             cudaMemcpyHostToDevice, e.stream));
    NRT_CUDA(cudaStreamSynchronize(e.stream));
    return NRT_OK;
  });
}

int nrt_batch_advance(nrt_batch *b, int64_t steps) {
  return nrt::guarded([&]() -> int {
    if (!b || steps < 0) return nrt::fail(NRT_EINVAL, "bad arguments");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    return b->eng.advance(steps);
  });
}

int nrt_batch_synchronize(nrt_batch *b) {
  return nrt::guarded([&]() -> int {
    if (!b) return nrt::fail(NRT_EINVAL, "null batch");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    NRT_CUDA(cudaStreamSynchronize(b->eng.stream));
    return nrt::implicit_check(b->eng);
  });
}

int nrt_batch_snapshot(nrt_batch *b, int32_t instance, double *potential) {
  return nrt::guarded([&]() -> int {
    if (!b || !potential) return nrt::fail(NRT_EINVAL, "null argument");
    nrt::Engine &e = b->eng;
    if (instance < 0 || instance >= e.pv.ninst) return nrt::fail(NRT_EINVAL, "instance out of range");
    NRT_CUDA(cudaSetDevice(e.device));
    int rc = e.fixup();
    if (rc) return rc;
    const int64_t o = e.host.off[instance];
    NRT_CUDA(cudaMemcpyAsync(potential, e.V[e.cur] + o, sizeof(double) * e.host.num_elem[instance],
                             cudaMemcpyDeviceToHost, e.stream));
    NRT_CUDA(cudaStreamSynchronize(e.stream));
    return nrt::implicit_check(e);
  });
}

int nrt_batch_snapshot_all(nrt_batch *b, double *potential) {
  return nrt::guarded([&]() -> int {
    if (!b || !potential) return nrt::fail(NRT_EINVAL, "null argument");
    nrt::Engine &e = b->eng;
    NRT_CUDA(cudaSetDevice(e.device));
    int rc = e.fixup();
    if (rc) return rc;
    NRT_CUDA(cudaMemcpyAsync(potential, e.V[e.cur], sizeof(double) * e.host.ntot,
                             cudaMemcpyDeviceToHost, e.stream));
    NRT_CUDA(cudaStreamSynchronize(e.stream));
    return nrt::implicit_check(e);
  });
}

int nrt_batch_remaining(nrt_batch *b, int64_t *remaining) {
  return nrt::guarded([&]() -> int {
    if (!b || !remaining) return nrt::fail(NRT_EINVAL, "null argument");
    nrt::Engine &e = b->eng;
    NRT_CUDA(cudaSetDevice(e.device));
    std::vector<nrt::InstDev> in(e.pv.ninst);
    NRT_CUDA(cudaMemcpyAsync(in.data(), e.pv.inst, sizeof(nrt::InstDev) * e.pv.ninst,
                             cudaMemcpyDeviceToHost, e.stream));
    NRT_CUDA(cudaStreamSynchronize(e.stream));
    for (int32_t i = 0; i < e.pv.ninst; i++) remaining[i] = in[i].iend - in[i].base;
    return NRT_OK;
  });
}

int nrt_batch_get_stats(nrt_batch *b, nrt_stats *st) {
  return nrt::guarded([&]() -> int {
    if (!b || !st) return nrt::fail(NRT_EINVAL, "null argument");
    return b->eng.get_stats(st);
  });
}

int nrt_batch_instance_stats(nrt_batch *b, int64_t *iters, int32_t *last_iters,
                             int32_t *nonconverged, double *last_residual) {
  return nrt::guarded([&]() -> int {
    if (!b) return nrt::fail(NRT_EINVAL, "null batch");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    return nrt::instance_stats(b->eng, iters, last_iters, nonconverged, last_residual);
  });
}

int nrt_batch_pass_counts(nrt_batch *b, int64_t *residuals, int64_t *precond_applies,
                          int64_t *xupdates, int64_t *basis_reads, int64_t *richardson_steps) {
  return nrt::guarded([&]() -> int {
    if (!b) return nrt::fail(NRT_EINVAL, "null batch");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    return nrt::pass_counts(b->eng, residuals, precond_applies, xupdates, basis_reads,
                            richardson_steps);
  });
}

int nrt_batch_destroy(nrt_batch *b) {
  return nrt::guarded([&]() -> int {
    delete b;
    return NRT_OK;
  });
}

int nrt_get_state(nrt_solver *s, double *V, double *V_other, double *m, double *h, double *n) {
  return nrt::guarded([&]() -> int {
    if (!s) return nrt::fail(NRT_EINVAL, "null solver");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    int rc = s->eng.get_state(0, V, V_other, m, h, n);
    return rc ? rc : nrt::implicit_check(s->eng);
  });
}

int nrt_set_state(nrt_solver *s, const double *V, const double *V_other, const double *m,
                  const double *h, const double *n) {
  return nrt::guarded([&]() -> int {
    if (!s) return nrt::fail(NRT_EINVAL, "null solver");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    return s->eng.set_state(0, V, V_other, m, h, n);
  });
}

int nrt_batch_get_state(nrt_batch *b, int32_t instance, double *V, double *V_other, double *m,
                        double *h, double *n) {
  return nrt::guarded([&]() -> int {
    if (!b) return nrt::fail(NRT_EINVAL, "null batch");
    if (instance < 0 || instance >= b->eng.pv.ninst) return nrt::fail(NRT_EINVAL, "instance out of range");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    int rc = b->eng.get_state(instance, V, V_other, m, h, n);
    return rc ? rc : nrt::implicit_check(b->eng);
  });
}

int nrt_batch_set_state(nrt_batch *b, int32_t instance, const double *V, const double *V_other,
                        const double *m, const double *h, const double *n) {
  return nrt::guarded([&]() -> int {
    if (!b) return nrt::fail(NRT_EINVAL, "null batch");
    if (instance < 0 || instance >= b->eng.pv.ninst) return nrt::fail(NRT_EINVAL, "instance out of range");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    return b->eng.set_state(instance, V, V_other, m, h, n);
  });
}

int nrt_set_strain(nrt_solver *s, const nrt_strain_config *cfg) {
  return nrt::guarded([&]() -> int {
    if (!s || !cfg) return nrt::fail(NRT_EINVAL, "null argument");
    if (cfg->instance)
      for (int32_t q = 0; q < cfg->num_elem; q++)
        if (cfg->instance[q] != 0) return nrt::fail(NRT_EINVAL, "a solver has only instance 0");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    return s->eng.strain_config(cfg);
  });
}

int nrt_batch_set_strain(nrt_batch *b, const nrt_strain_config *cfg) {
  return nrt::guarded([&]() -> int {
    if (!b || !cfg) return nrt::fail(NRT_EINVAL, "null argument");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    return b->eng.strain_config(cfg);
  });
}

int nrt_record(nrt_solver *s, const nrt_record_config *cfg) {
  return nrt::guarded([&]() -> int {
    if (!s || !cfg) return nrt::fail(NRT_EINVAL, "null argument");
    if (cfg->instance)
      for (int32_t p = 0; p < cfg->num_probes; p++)
        if (cfg->instance[p] != 0) return nrt::fail(NRT_EINVAL, "a solver has only instance 0");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    return s->eng.record_config(cfg);
  });
}

int nrt_batch_record(nrt_batch *b, const nrt_record_config *cfg) {
  return nrt::guarded([&]() -> int {
    if (!b || !cfg) return nrt::fail(NRT_EINVAL, "null argument");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    return b->eng.record_config(cfg);
  });
}

int nrt_record_read(nrt_solver *s, int64_t *num_samples, double *times, double *values,
                    int32_t *num_spikes, double *spike_times) {
  return nrt::guarded([&]() -> int {
    if (!s) return nrt::fail(NRT_EINVAL, "null solver");
    NRT_CUDA(cudaSetDevice(s->eng.device));
    int rc = s->eng.record_read(num_samples, times, values, num_spikes, spike_times);
    return rc ? rc : nrt::implicit_check(s->eng);
  });
}

int nrt_batch_record_read(nrt_batch *b, int64_t *num_samples, double *times, double *values,
                          int32_t *num_spikes, double *spike_times) {
  return nrt::guarded([&]() -> int {
    if (!b) return nrt::fail(NRT_EINVAL, "null batch");
    NRT_CUDA(cudaSetDevice(b->eng.device));
    int rc = b->eng.record_read(num_samples, times, values, num_spikes, spike_times);
    return rc ? rc : nrt::implicit_check(b->eng);
  });
}

}  // extern "C"
