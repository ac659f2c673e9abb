// Internal definitions shared by the host runtime (api.cu, pack.cu) and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <utility>
#include <string>
#include <thread>
#include <vector>

#include "guard.h"
#include "neurite_gb300.h"

namespace nrt {

// Per-element flag bits (low 13 bits of Topo::flags; the instance id sits above).
enum : uint32_t {
  F_HH = 1u,        // Hodgkin_Huxley element (gates evolve)
  F_BRANCH = 2u,    // branching point: has a DL child
  F_TERM = 4u,      // terminal: copies a neighbour after the step (explicit)
  F_ROOT = 8u,      // terminals[0]: copies element root+1 (src/solverEx-cpu.cpp:157)
  F_UP = 16u,       // implicit row has a column at its mother
  F_DOWNR = 32u,    // implicit row has a column at DR (== j + 1)
  F_IDENT = 64u,    // implicit identity row (left untouched by the reference)
  F_DL_TERM = 128u, // explicit: the DL neighbour is a terminal (zero flux)
  F_MO_TERM = 256u, // explicit: the mother is a terminal (element 1 next to the root)
  F_DR_TERM = 512u, // explicit: the DR neighbour is a terminal (zero flux)
  F_DOWNL = 1024u,  // implicit row has a column at DL
  F_INP = 2048u,    // nonzero injected current
  F_XTOPO = 4096u,  // a neighbour is not j-1 / j+1 (or the element is a branch point,
                    // terminal or the root): the step needs the full topology record
};
constexpr int INST_SHIFT = 13;

// Topology of one element, global (packed) indices.  16 bytes, loaded as one int4.
struct __align__(16) Topo {
  int32_t mother;   // explicit: neighbour for the mother term; -1 at the root
  int32_t dr;       // DR (== self for terminals)
  int32_t dl;       // DL (branch points only; else the element itself)
  uint32_t flags;   // F_* | instance << INST_SHIFT
};

// HH parameters, SoA rows of Pack::hp (FP64); the mixed path keeps each column's rows
// together as 12 floats (three 16-byte loads, PackView::hpq).  Columns: one per
// instance when every HH element of an instance has the same parameters; else one per
// distinct parameter set ("class", indexed through hp_cls) when there are few of them;
// else one per element.
enum { HP_GNA, HP_GK, HP_GL, HP_ENA, HP_EK, HP_EL, HP_LSNA, HP_LSK, HP_REST, HP_DX, HP_DTMS, HP_ROWS };

// Per-instance run state kept on the device.
struct InstDev {
  int64_t base;     // loop index of the next step
  int64_t iend;     // one past the last loop index
  double dT;
  double t0, t1;    // stimulus window
  int64_t ion, ioff;  // loop indices i with t0 <= i*dT <= t1 (the window as integers)
};

// Fills ion/ioff so that (ion <= i && i <= ioff) == (t0 <= i*dT && i*dT <= t1) for every
// loop index i, evaluating the reference's own test (src/neurite.cpp:227-230) at the bounds.
inline void set_window(InstDev &in) {
  auto on = [&](int64_t i) { const double t = (double)i * in.dT; return t >= in.t0; };
  auto below = [&](int64_t i) { const double t = (double)i * in.dT; return t <= in.t1; };
  const double lim = 9.0e15;
  double a = in.t0 / in.dT, b = in.t1 / in.dT;
  if (!(a == a) || !(b == b) || in.t1 < in.t0) {
    in.ion = 1;
    in.ioff = 0;
    return;
  }
  a = a < -lim ? -lim : (a > lim ? lim : a);
  b = b < -lim ? -lim : (b > lim ? lim : b);
  int64_t i0 = (int64_t)a, i1 = (int64_t)b;
  while (on(i0 - 1)) i0--;
  while (!on(i0)) i0++;
  while (!below(i1) && i1 > i0 - 1) i1--;
  while (below(i1 + 1)) i1++;
  in.ion = i0;
  in.ioff = i1;
}

// Runs f(i) for every i in [0, n) on the host's cores, handing out indices one at a time
// (instances differ in size by orders of magnitude).
template <class F>
void parallel_for(int64_t n, F f) {
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 64u));
  nt = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)nt, n));
  std::atomic<int64_t> next(0);
  auto work = [&]() {
    for (;;) {
      const int64_t i = next.fetch_add(1);
      if (i >= n) break;
      f(i);
    }
  };
  std::vector<std::thread> th;
  for (unsigned t = 1; t < nt; t++) th.emplace_back(work);
  work();
  for (std::thread &t : th) t.join();
}

// f(a, b) over [0, n) in chunks of about 1M.
template <class F>
void parallel_ranges(int64_t n, F f) {
  const int64_t chunk = 1 << 20, nc = (n + chunk - 1) / chunk;
  parallel_for(nc, [&](int64_t c) { f(c * chunk, std::min(n, (c + 1) * chunk)); });
}

// Device-side view passed by value to the kernels.
struct PackView {
  int64_t ntot;
  int32_t ninst;
  const Topo *topo;
  const double *cdt;   // dT / (c_m dX)
  const double *gax;   // 1 / (r_a dX): conductance to the mother
  const double *wdx;   // W dX (cables)
  const double *kdx;   // K dX (cables)
  const double *inp;   // injected current
  double *gate;        // [3][ntot] m, h, n (FP64 path)
  float *gatef;        // [3][ntot] (mixed path)
  const double *hp;    // [HP_ROWS][hp_ld]
  const float4 *hpq;   // mixed: [hp_ld][3], one column's HP_* rows as 12 floats (11 + pad)
  int64_t hp_ld;       // number of columns
  int hp_inst;         // 1: column = instance
  const uint32_t *hp_cls;  // column per element (class tables), or null
  const uint32_t *eflags;  // Topo::flags alone (mixed explicit step), or null
  int hh_dense;        // most elements are HH: the step loads gates before the topology
  const float *cdtf, *gaxf, *wdxf, *kdxf, *inpf;  // FP32 copies (mixed path)
  InstDev *inst;
  int *err;            // device error word (a bounded wait gave up), or null
  int tile_blocks;     // mixed explicit: persistent CTAs of the tiled step (0: untiled)
  int step_threads;    // explicit, one thread per element: threads per block (0: by size)
  int sms;             // multiprocessors of the handle's device
};

// Device-side recording at probes (record.cu, record.cuh).  Probes are sorted by
// instance: those of instance q are [p0[q], p0[q+1]).
struct RecView {
  int32_t nprobe;
  int32_t max_spikes;
  int64_t origin;      // loop index at which the sample counter starts
  int64_t interval;    // sample when (i - origin + 1) % (interval + 1) == 0
  int64_t cap;         // samples kept per probe
  double thresh;       // spike threshold
  const int64_t *src;  // global element read for each probe
  const int32_t *inst; // instance of each probe
  const int32_t *p0;   // [ninst + 1]
  int64_t *nsamp;      // samples taken per probe
  int32_t *nspike;     // crossings found per probe
  int64_t *prev_i;     // loop index of the last value seen
  double *prev_v;      // the last value seen
  double *val;         // [nprobe][cap]
  double *spk;         // [nprobe][max_spikes]
};

// The words of the explicit chunk kernel's grid barrier (explicit.cu), 0 between launches.
struct GridBar {
  unsigned long long count;  // arrivals in the current launch
  unsigned int exits;        // CTAs that have left it
  unsigned int pad;
};

struct DeviceBuffer {
  void *ptr = nullptr;
  size_t bytes = 0;
};

// Host-side error helper: records the message in a thread-local slot.
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
#define NRT_CUDA(call)                                        \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return ::nrt::cuda_fail(_e, #call); \
  } while (0)

// An allocator whose construct() leaves trivially constructible elements uninitialised, so
// that resize() does not zero-fill (on one thread) arrays that a parallel pass then writes
// in full: the writers touch the pages first.
template <class T>
struct NoInitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <class U>
  NoInitAlloc(const NoInitAlloc<U> &) {}
  template <class U>
  void construct(U *) noexcept {}
  template <class U, class... A>
  void construct(U *p, A &&...a) {
    ::new ((void *)p) U(std::forward<A>(a)...);
  }
};
// Element-indexed host arrays that are written in full after they are sized.
template <class T>
using hvec = std::vector<T, NoInitAlloc<T>>;

// Host mirror of the packed trees: built from nrt_problem arrays.
struct HostPack {
  int64_t ntot = 0;
  int32_t ninst = 0;
  std::vector<int64_t> off;         // element offset per instance (ninst + 1)
  hvec<Topo> topo;
  hvec<double> cdt, gax, wdx, kdx, inp, V0, V1;
  hvec<double> gate;                // [3][ntot]
  std::vector<double> hp;           // [HP_ROWS][hp_ld]
  bool hp_inst = false;             // one HH parameter column per instance
  hvec<uint32_t> hp_cls;            // column per element when classes are used
  int64_t hp_ld = 0;
  hvec<double> c_m_dx, radx;        // c_m dX and r_a dX per element (implicit assembly)
  hvec<double> Wfull, Kfull;        // W, K per element as given
  std::vector<InstDev> inst;
  std::vector<int32_t> hh_local;    // per instance: HH element indices (local), concatenated
  std::vector<int64_t> hh_off;      // per instance offsets into hh_local (ninst + 1)
  std::vector<int32_t> num_elem;    // per instance
  std::vector<int64_t> terms;       // global indices of all terminals
  bool fusable = true;              // every terminal neighbour copies its reader
  bool invariant = true;            // initial V already has terminals equal to their sources
};

int build_host_pack(const nrt_problem *probs, int32_t count, HostPack &hp);

// One column of the FP32 parameter table (three vector loads).
struct HHParams32 {
  float v[12];  // indexed by HP_*
};
__device__ __forceinline__ HHParams32 hh_params32(const float4 *hpq, int64_t col) {
  const float4 *q = hpq + 3 * col;
  const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
  HHParams32 r;
  r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
  r.v[4] = b.x; r.v[5] = b.y; r.v[6] = b.z; r.v[7] = b.w;
  r.v[8] = c.x; r.v[9] = c.y; r.v[10] = c.z; r.v[11] = c.w;
  return r;
}

// Column of the HH parameter tables for element j of instance `inst`.
__host__ __device__ inline int64_t hp_col(const PackView &p, int64_t j, uint32_t inst) {
  return p.hp_cls ? (int64_t)p.hp_cls[j] : (p.hp_inst ? (int64_t)inst : j);
}

// Kernel launchers (explicit.cu).  fold (mixed, fused form; strain.cuh): the step also
// writes the strained elements' coefficients of the next step.
struct StrainFold;
int launch_explicit_step(const PackView &pv, int precision, bool general, int k, int force,
                         const double *Vin, double *Vout, const float *Fin, float *Fout,
                         cudaStream_t st, const StrainFold *fold = nullptr);
int launch_terminal_fixup(const Topo *topo, const int64_t *terms, int64_t nterm, double *V,
                          float *Vf, cudaStream_t st);
int launch_advance_base(InstDev *inst, int32_t ninst, int64_t steps, cudaStream_t st);
int explicit_tile_blocks(int device, int64_t ntot, int per_sm_cap);
struct StrainView;  // strain.cuh
// nk fused-form steps of the time loop in one cooperative launch, with the probes' reads
// and the strained elements' rows (from the chunk table) between steps.  V0/F0 hold the
// current state; step k writes V1/F1 when k is even and V0/F0 when it is odd.
int launch_explicit_chunk(const PackView &pv, int precision, int nk, double *V0, double *V1,
                          float *F0, float *F1, const RecView &r, const StrainView &s,
                          GridBar *gb, int per_sm_cap, cudaStream_t st);
// Recording after explicit step k (record.cu); V is that step's output.
int launch_record_step(const RecView &r, const InstDev *inst, int k, const double *V,
                       cudaStream_t st);

}  // namespace nrt
