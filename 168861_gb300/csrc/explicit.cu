// Explicit (forward Euler) step: one fused kernel per time step.
//
// Replaces the reference's four launches per step -- Update_HH, explicit_solver_normal,
// explicit_solver_branch, explicit_solver_terminal (src/solverEx-gpu.cpp:87-194) -- and
// computes what SolverExCPU::update + ::calculate compute (src/solverEx-cpu.cpp:90-168):
//
//   gates_j   <- gates_j + dt (alpha (1 - gate) - beta gate)            (HH elements)
//   V'_j      =  V_j + dT/(c_m dX)_j [ b_j (V_DL - V_j) g_DL + (V_DR - V_j) g_DR
//                                      + (V_mo - V_j) g_j + W_j dX_j V_j + K_j dX_j + I_j ]
//   V'_t      =  V'_mother(t) for terminals, V'_0 = V'_1             (sealed ends)
//
// with g_x = 1/(r_a dX)_x.
//
// Sealed ends without a second launch: after every step a terminal holds an exact copy of
// its source element, so the flux a neighbour sees through it, (V_t - V_j) g_t, is
// exactly zero at the next step.  The kernel therefore skips flux terms through terminals
// (flag bits F_*_TERM, bit-identical to the reference's subtraction of equal values) and
// never writes terminal voltages during a run; `terminal_fixup` copies them into place
// before anything reads V (snapshot, export, device pointer).  A terminal that is itself
// a Hodgkin_Huxley element still advances its gates from its source's voltage, which is
// what the reference's update() reads for it.  When the caller's initial potential breaks
// the copy invariant, the first step runs in the general form (terminal terms evaluated,
// then the copy launch), exactly as the reference does.
//
// Instances: elements of many trees are packed back to back (global indices); the
// instance id in the flags selects dT, the stimulus window and the loop index, so one
// launch advances every tree.  An instance whose loop range is exhausted copies V.
#include <algorithm>

#include "hh.cuh"
#include "nrt_internal.h"
#include "pdl.cuh"
#include "record.cuh"
#include "strain.cuh"
#include "tma.cuh"

namespace nrt {

namespace {

__device__ __forceinline__ bool input_on(const InstDev &in, int64_t i, int force) {
  if (force >= 0) return force != 0;
  // t0 <= i*dT <= t1 (src/neurite.cpp:227-230), precomputed as loop-index bounds
  return i >= in.ion && i <= in.ioff;
}

__device__ __forceinline__ int64_t ghost_source(const Topo &t, int64_t j) {
  return (t.flags & F_ROOT) ? j + 1 : (int64_t)t.mother;
}

// Element j of step k in FP64 (the body of explicit_step_f64, of explicit_step_f64_lanes'
// lane 0 and of the chunk kernel).  rates: the element's six HH rates when its lanes have
// evaluated them (hh_rate64), else null (this thread evaluates them).
template <bool kGeneral>
__device__ __forceinline__ void f64_element(const PackView &p, int k, int force, int64_t j,
                                            const double *Vin, double *Vout,
                                            const double *rates = nullptr) {
  const Topo tj = p.topo[j];
  const InstDev in = p.inst[tj.flags >> INST_SHIFT];
  const int64_t i = in.base + k;
  if (i >= in.iend) {  // this instance is done: carry V over to the other buffer
    Vout[j] = Vin[j];
    return;
  }
  const int64_t N = p.ntot;
  const bool term = (tj.flags & F_TERM) != 0;
  if (term && !(tj.flags & F_HH)) return;
  const double v = Vin[(kGeneral || !term) ? j : ghost_source(tj, j)];
  double wdx = 0, kdx = 0;
  if (tj.flags & F_HH) {
    const int64_t L = p.hp_ld;
    const double *hp = p.hp + hp_col(p, j, tj.flags >> INST_SHIFT);
    GateStep64 g =
        rates ? hh_gates64(rates[0], rates[1], rates[2], rates[3], rates[4], rates[5],
                           p.gate[j], p.gate[N + j], p.gate[2 * N + j], hp[HP_DTMS * L],
                           hp[HP_GNA * L], hp[HP_GK * L], hp[HP_GL * L], hp[HP_ENA * L],
                           hp[HP_EK * L], hp[HP_EL * L])
              : hh_step64(v, p.gate[j], p.gate[N + j], p.gate[2 * N + j], hp[HP_LSNA * L],
                          hp[HP_LSK * L], hp[HP_REST * L], hp[HP_DTMS * L], hp[HP_GNA * L],
                          hp[HP_GK * L], hp[HP_GL * L], hp[HP_ENA * L], hp[HP_EK * L],
                          hp[HP_EL * L]);
    p.gate[j] = g.m;
    p.gate[N + j] = g.h;
    p.gate[2 * N + j] = g.n;
    if (term) return;  // ghost: only its gates move
    const double dx = hp[HP_DX * L];
    wdx = g.W * dx;
    kdx = g.K * dx;
  } else {
    wdx = p.wdx[j];
    kdx = p.kdx[j];
  }
  const bool active = input_on(in, i, force);
  // src/solverEx-cpu.cpp:141-152, same summation order
  double acc = 0.0;
  const bool skip_dl = !kGeneral && (tj.flags & F_DL_TERM);
  const bool skip_dr = !kGeneral && (tj.flags & F_DR_TERM);
  const bool skip_mo = !kGeneral && (tj.flags & F_MO_TERM);
  if ((tj.flags & F_BRANCH) && !skip_dl) acc = (Vin[tj.dl] - v) * p.gax[tj.dl];
  if (!skip_dr) acc = acc + (Vin[tj.dr] - v) * p.gax[tj.dr];
  if (!skip_mo) acc = acc + (Vin[tj.mother] - v) * p.gax[j];
  acc = acc + wdx * v;
  acc = acc + kdx;
  if (active && (tj.flags & F_INP)) acc = acc + p.inp[j];  // adding a zero input is exact
  Vout[j] = v + p.cdt[j] * acc;
}

template <bool kGeneral>
__global__ void __launch_bounds__(256) explicit_step_f64(PackView p, int k, int force,
                                                         const double *__restrict__ Vin,
                                                         double *__restrict__ Vout) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.ntot) return;
  f64_element<kGeneral>(p, k, force, j, Vin, Vout);
}

// Small FP64 packs: eight lanes per element.  One warp's FP64 work per element is the
// step's floor when each warp holds 32 elements (six exponentials and three divisions each
// on a pipe at 1/70 of FP32), so lanes 0-5 of an element's group evaluate one rate each with
// the same code (hh_rate64: no divergence), lane 0 gathers them by shuffles and finishes the
// element as explicit_step_f64 does.  Every lane of a warp takes part in the shuffles; lanes
// of elements that are out of range, finished, passive or sealed-end ghosts evaluate rates
// of a placeholder potential that nobody reads.  The same values as explicit_step_f64, bit
// for bit.
constexpr int kRateLanes = 8;

template <bool kGeneral>
__global__ void __launch_bounds__(256) explicit_step_f64_lanes(PackView p, int k, int force,
                                                               const double *__restrict__ Vin,
                                                               double *__restrict__ Vout) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / kRateLanes;
  const int q = (int)(threadIdx.x % kRateLanes);
  double vna = 0.0, vk = 0.0;
  if (j < p.ntot) {  // the element's potential and shifts, as f64_element reads them
    const Topo tj = p.topo[j];
    const InstDev in = p.inst[tj.flags >> INST_SHIFT];
    const bool term = (tj.flags & F_TERM) != 0;
    if (in.base + k < in.iend && (tj.flags & F_HH)) {
      const double v = Vin[(kGeneral || !term) ? j : ghost_source(tj, j)];
      const int64_t L = p.hp_ld;
      const double *hp = p.hp + hp_col(p, j, tj.flags >> INST_SHIFT);
      vna = ((v + hp[HP_LSNA * L]) - hp[HP_REST * L]) * 1000.0;
      vk = ((v + hp[HP_LSK * L]) - hp[HP_REST * L]) * 1000.0;
    }
  }
  const double r = hh_rate64(q < 6 ? q : 5, vna, vk);
  double rates[6];
  const int base = (int)(threadIdx.x & 31) & ~(kRateLanes - 1);
#pragma unroll
  for (int s = 0; s < 6; s++) rates[s] = __shfl_sync(0xffffffffu, r, base + s);
  if (q == 0 && j < p.ntot) f64_element<kGeneral>(p, k, force, j, Vin, Vout, rates);
}

// Mixed precision (element j of step k; the body of explicit_step_mixed and of the chunk
// kernel): gates, rates, conductances and currents in FP32; the potential is
// accumulated in FP64.  GB300's FP64 pipe runs at 1/70 of the FP32 rate, so the stencil
// reads an FP32 shadow of V (Vf = (float)V, refreshed from the FP64 value every step):
// neighbour differences carry an absolute error of ~4e-9 V, while the FP64 accumulator
// V' = V + dt-scaled current keeps long horizons free of drift.  FP64-pipe work is one
// conversion, one add and one conversion back per element.
template <bool kGeneral>
__device__ __forceinline__ void mixed_element(const PackView &p, int k, int force, int64_t j,
                                              const double *Vin, double *Vout, const float *Fin,
                                              float *Fout) {
  const int64_t N = p.ntot;
  // Loads that do not depend on the topology record go out together with it: the
  // element's own state and its neighbours j-1 and j+1 (the mother and DR of nearly
  // every element in the reference numbering), so most elements wait for one round trip.
  const int64_t jm = j > 0 ? j - 1 : j, jp = j + 1 < N ? j + 1 : j;
  // The flags word alone (4 B) stands for the 16-byte topology record unless a neighbour
  // is not adjacent (F_XTOPO), which only branch points, DL children, terminals and the
  // root are.
  const uint32_t fl = p.eflags ? p.eflags[j] : 0u;
  const float f0 = Fin[j], fm = Fin[jm], fp = Fin[jp];
  const float g0 = p.gaxf[j], gp = p.gaxf[jp];
  const double v64 = Vin[j];
  const float cdt = p.cdtf[j];
  const uint32_t cls = p.hp_cls ? p.hp_cls[j] : 0u;
  float m0 = 0.f, h0 = 0.f, n0 = 0.f;
  if (p.hh_dense) {
    m0 = p.gatef[j];
    h0 = p.gatef[N + j];
    n0 = p.gatef[2 * N + j];
  }
  Topo tj;
  if (!p.eflags || (fl & F_XTOPO)) {
    tj = p.topo[j];
  } else {
    tj.mother = (int32_t)jm;
    tj.dr = (int32_t)jp;
    tj.dl = (int32_t)j;
    tj.flags = fl;
  }
  const uint32_t inst = tj.flags >> INST_SHIFT;
  const InstDev in = p.inst[inst];
  const int64_t i = in.base + k;
  if (i >= in.iend) {
    Vout[j] = v64;
    Fout[j] = f0;
    return;
  }
  const bool term = (tj.flags & F_TERM) != 0;
  if (term && !(tj.flags & F_HH)) return;
  const int64_t self = (kGeneral || !term) ? j : ghost_source(tj, j);
  const float vf = self == j ? f0 : (self == jm ? fm : (self == jp ? fp : Fin[self]));
  float wdx, kdx;
  if (tj.flags & F_HH) {
    if (!p.hh_dense) {
      m0 = p.gatef[j];
      h0 = p.gatef[N + j];
      n0 = p.gatef[2 * N + j];
    }
    const HHParams32 q =
        hh_params32(p.hpq, p.hp_cls ? (int64_t)cls : (p.hp_inst ? (int64_t)inst : j));
    const float dv = vf - q.v[HP_REST];
    GateStep32 g = hh_step32(dv + q.v[HP_LSNA], dv + q.v[HP_LSK], m0, h0, n0, q.v[HP_DTMS],
                             q.v[HP_GNA], q.v[HP_GK], q.v[HP_GL], q.v[HP_ENA], q.v[HP_EK],
                             q.v[HP_EL]);
    p.gatef[j] = g.m;
    p.gatef[N + j] = g.h;
    p.gatef[2 * N + j] = g.n;
    if (term) return;
    const float dx = q.v[HP_DX];
    wdx = g.W * dx;
    kdx = g.K * dx;
  } else {
    wdx = p.wdxf[j];
    kdx = p.kdxf[j];
  }
  const bool active = input_on(in, i, force);
  float acc = 0.0f;
  if ((tj.flags & F_BRANCH) && (kGeneral || !(tj.flags & F_DL_TERM)))
    acc = (Fin[tj.dl] - vf) * p.gaxf[tj.dl];
  if (kGeneral || !(tj.flags & F_DR_TERM)) {
    const bool adj = tj.dr == jp && jp != j;
    const float fd = adj ? fp : Fin[tj.dr], gd = adj ? gp : p.gaxf[tj.dr];
    acc = fmaf(fd - vf, gd, acc);
  }
  if (kGeneral || !(tj.flags & F_MO_TERM)) {
    const float fo = (tj.mother == jm && jm != j) ? fm : Fin[tj.mother];
    acc = fmaf(fo - vf, g0, acc);
  }
  acc = fmaf(wdx, vf, acc) + kdx;
  if (active && (tj.flags & F_INP)) acc += p.inpf[j];
  const double vn = v64 + (double)(cdt * acc);
  Vout[j] = vn;
  Fout[j] = (float)vn;
}

template <bool kGeneral>
__global__ void __launch_bounds__(256) explicit_step_mixed(PackView p, int k, int force,
                                                           const double *__restrict__ Vin,
                                                           double *__restrict__ Vout,
                                                           const float *__restrict__ Fin,
                                                           float *__restrict__ Fout,
                                                           StrainFold fold) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  if (fold.row >= 0 && (int)blockIdx.x >= fold.first_block) {
    fold_rows(fold);  // the next step's strained rows, into the other copy
    return;
  }
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.ntot) return;
  mixed_element<kGeneral>(p, k, force, j, Vin, Vout, Fin, Fout);
}

// ---- the mixed step with TMA-staged tiles
//
// Same arithmetic as explicit_step_mixed<false> (bit for bit), reorganised for memory-level
// parallelism: persistent CTAs walk tiles of kTileE consecutive elements; one thread issues
// bulk copies (cp.async.bulk) of the tile's contiguous element arrays -- flags, FP32 shadow
// of V with its one-element halo, conductances with theirs, FP64 V, dT/(c_m dX), the class
// index, and the gates (or W dX, K dX when few elements are HH) -- into shared memory on an
// mbarrier, while the CTA computes the previous tile from the other buffer.  About 20 KB
// per tile are in flight per CTA instead of one load per thread.  Far neighbours (branch
// points, DL children), the per-instance record and the parameter tables come from global
// memory as before.
constexpr int kTileE = 512;                      // elements per tile
constexpr int kTileThreads = 256;                // two elements per thread
constexpr int kR4 = (kTileE + 8) * 4;            // a 4-byte array's window, 16-byte rounded
constexpr int kR8 = (kTileE + 4) * 8;            // the FP64 window
enum { TO_FL = 0, TO_F = kR4, TO_GAX = 2 * kR4, TO_V = 3 * kR4, TO_CDT = 3 * kR4 + kR8,
       TO_CLS = 4 * kR4 + kR8, TO_G0 = 5 * kR4 + kR8, TO_G1 = 6 * kR4 + kR8,
       TO_G2 = 7 * kR4 + kR8, kTileBufBytes = 8 * kR4 + kR8 };

// Bytes of the bulk copy of elements [o, o + n) of an array (16-byte aligned base): the
// window rounded out to 16-byte boundaries.
template <typename X>
__device__ __forceinline__ uint32_t stage_bytes(int64_t o, int64_t n) {
  const uint64_t lo = ((uint64_t)o * sizeof(X)) & ~(uint64_t)15;
  const uint64_t hi = ((uint64_t)(o + n) * sizeof(X) + 15) & ~(uint64_t)15;
  return (uint32_t)(hi - lo);
}
template <typename X>
__device__ __forceinline__ void stage(unsigned char *dst, const X *a, int64_t o, int64_t n,
                                      uint64_t *bar) {
  const uint64_t lo = ((uint64_t)o * sizeof(X)) & ~(uint64_t)15;
  bulk_load(dst, (const char *)a + lo, stage_bytes<X>(o, n), bar);
}
// The shared-memory copy of element o of a staged array.
template <typename X>
__device__ __forceinline__ const X *staged(const unsigned char *dst, int64_t o) {
  return (const X *)(dst + (((uint64_t)o * sizeof(X)) & 15));
}

struct TileWin {
  int64_t s, cnt, of, ngax, nf;  // first element, count, F window start, window lengths
};
__device__ __forceinline__ TileWin tile_win(int64_t t, int64_t N) {
  TileWin w;
  w.s = t * kTileE;
  w.cnt = N - w.s < kTileE ? N - w.s : kTileE;
  w.of = w.s > 0 ? w.s - 1 : 0;
  const int64_t end = w.s + w.cnt + 1 < N ? w.s + w.cnt + 1 : N;  // one past the halo
  w.nf = end - w.of;
  w.ngax = end - w.s;
  return w;
}

// Thread 0: expect and issue the copies of tile t into buffer `buf`.
__device__ __forceinline__ void issue_tile(const PackView &p, const float *Fin, const double *Vin,
                                           int64_t t, unsigned char *buf, uint64_t *bar) {
  const int64_t N = p.ntot;
  const TileWin w = tile_win(t, N);
  uint32_t bytes = stage_bytes<uint32_t>(w.s, w.cnt) + stage_bytes<float>(w.of, w.nf) +
                   stage_bytes<float>(w.s, w.ngax) + stage_bytes<double>(w.s, w.cnt) +
                   stage_bytes<float>(w.s, w.cnt);
  if (p.hp_cls) bytes += stage_bytes<uint32_t>(w.s, w.cnt);
  if (p.hh_dense)
    bytes += stage_bytes<float>(w.s, w.cnt) + stage_bytes<float>(N + w.s, w.cnt) +
             stage_bytes<float>(2 * N + w.s, w.cnt);
  else
    bytes += 2 * stage_bytes<float>(w.s, w.cnt);
  mbar_expect_tx(bar, bytes);
  stage(buf + TO_FL, p.eflags, w.s, w.cnt, bar);
  stage(buf + TO_F, Fin, w.of, w.nf, bar);
  stage(buf + TO_GAX, p.gaxf, w.s, w.ngax, bar);
  stage(buf + TO_V, Vin, w.s, w.cnt, bar);
  stage(buf + TO_CDT, p.cdtf, w.s, w.cnt, bar);
  if (p.hp_cls) stage(buf + TO_CLS, p.hp_cls, w.s, w.cnt, bar);
  if (p.hh_dense) {
    stage(buf + TO_G0, p.gatef, w.s, w.cnt, bar);
    stage(buf + TO_G1, p.gatef, N + w.s, w.cnt, bar);
    stage(buf + TO_G2, p.gatef, 2 * N + w.s, w.cnt, bar);
  } else {
    stage(buf + TO_G0, p.wdxf, w.s, w.cnt, bar);
    stage(buf + TO_G1, p.kdxf, w.s, w.cnt, bar);
  }
}

// One element of a staged tile (the body of explicit_step_mixed<false>).
__device__ __forceinline__ void tile_element(const PackView &p, int k, int force,
                                             const unsigned char *buf, const TileWin &w,
                                             int64_t j, const float *__restrict__ Fin,
                                             double *__restrict__ Vout,
                                             float *__restrict__ Fout) {
  const int64_t N = p.ntot;
  const int64_t jm = j > 0 ? j - 1 : j, jp = j + 1 < N ? j + 1 : j;
  const uint32_t fl = staged<uint32_t>(buf + TO_FL, w.s)[j - w.s];
  const float *sF = staged<float>(buf + TO_F, w.of) - w.of;     // sF[q] = Fin[q]
  const float *sG = staged<float>(buf + TO_GAX, w.s) - w.s;     // sG[q] = gaxf[q]
  const float f0 = sF[j], fm = sF[jm], fp = sF[jp];
  const float g0 = sG[j], gp = sG[jp];
  const double v64 = staged<double>(buf + TO_V, w.s)[j - w.s];
  const float cdt = staged<float>(buf + TO_CDT, w.s)[j - w.s];
  const uint32_t cls = p.hp_cls ? staged<uint32_t>(buf + TO_CLS, w.s)[j - w.s] : 0u;
  Topo tj;
  if (fl & F_XTOPO) {
    tj = p.topo[j];
  } else {
    tj.mother = (int32_t)jm;
    tj.dr = (int32_t)jp;
    tj.dl = (int32_t)j;
    tj.flags = fl;
  }
  const uint32_t inst = tj.flags >> INST_SHIFT;
  const InstDev in = p.inst[inst];
  const int64_t i = in.base + k;
  if (i >= in.iend) {
    Vout[j] = v64;
    Fout[j] = f0;
    return;
  }
  const bool term = (tj.flags & F_TERM) != 0;
  if (term && !(tj.flags & F_HH)) return;
  const int64_t self = term ? ghost_source(tj, j) : j;
  const float vf = self == j ? f0 : (self == jm ? fm : (self == jp ? fp : Fin[self]));
  float wdx, kdx;
  if (tj.flags & F_HH) {
    float m0, h0, n0;
    if (p.hh_dense) {
      m0 = staged<float>(buf + TO_G0, w.s)[j - w.s];
      h0 = staged<float>(buf + TO_G1, N + w.s)[j - w.s];
      n0 = staged<float>(buf + TO_G2, 2 * N + w.s)[j - w.s];
    } else {
      m0 = p.gatef[j];
      h0 = p.gatef[N + j];
      n0 = p.gatef[2 * N + j];
    }
    const HHParams32 q =
        hh_params32(p.hpq, p.hp_cls ? (int64_t)cls : (p.hp_inst ? (int64_t)inst : j));
    const float dv = vf - q.v[HP_REST];
    GateStep32 g = hh_step32(dv + q.v[HP_LSNA], dv + q.v[HP_LSK], m0, h0, n0, q.v[HP_DTMS],
                             q.v[HP_GNA], q.v[HP_GK], q.v[HP_GL], q.v[HP_ENA], q.v[HP_EK],
                             q.v[HP_EL]);
    p.gatef[j] = g.m;
    p.gatef[N + j] = g.h;
    p.gatef[2 * N + j] = g.n;
    if (term) return;
    const float dx = q.v[HP_DX];
    wdx = g.W * dx;
    kdx = g.K * dx;
  } else if (p.hh_dense) {
    wdx = p.wdxf[j];
    kdx = p.kdxf[j];
  } else {
    wdx = staged<float>(buf + TO_G0, w.s)[j - w.s];
    kdx = staged<float>(buf + TO_G1, w.s)[j - w.s];
  }
  const bool active = input_on(in, i, force);
  float acc = 0.0f;
  if ((tj.flags & F_BRANCH) && !(tj.flags & F_DL_TERM))
    acc = (Fin[tj.dl] - vf) * p.gaxf[tj.dl];
  if (!(tj.flags & F_DR_TERM)) {
    const bool adj = tj.dr == jp && jp != j;
    const float fd = adj ? fp : Fin[tj.dr], gd = adj ? gp : p.gaxf[tj.dr];
    acc = fmaf(fd - vf, gd, acc);
  }
  if (!(tj.flags & F_MO_TERM)) {
    const float fo = (tj.mother == jm && jm != j) ? fm : Fin[tj.mother];
    acc = fmaf(fo - vf, g0, acc);
  }
  acc = fmaf(wdx, vf, acc) + kdx;
  if (active && (tj.flags & F_INP)) acc += p.inpf[j];
  const double vn = v64 + (double)(cdt * acc);
  Vout[j] = vn;
  Fout[j] = (float)vn;
}

// Buffers pass between the issuing thread and the warps on mbarriers: `full[b]` completes
// when tile data has landed in buffer b, `empty[b]` when every warp is done with it.  A warp
// that finishes its part of a tile moves on to the other buffer without waiting for the
// rest of the CTA; only the issuing thread waits, for `empty`, before refilling a buffer.
constexpr int kTileWarps = kTileThreads / 32;

__global__ void __launch_bounds__(kTileThreads) explicit_step_mixed_tiled(
    PackView p, int k, int force, const double *__restrict__ Vin, double *__restrict__ Vout,
    const float *__restrict__ Fin, float *__restrict__ Fout, StrainFold fold) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  if (fold.row >= 0 && (int)blockIdx.x >= fold.first_block) {
    fold_rows(fold);  // the next step's strained rows, into the other copy
    return;
  }
  // the CTAs that walk tiles (the others write strain rows)
  const int nblk = fold.row >= 0 ? fold.first_block : (int)gridDim.x;
  extern __shared__ __align__(16) unsigned char tsm[];
  uint64_t *full = (uint64_t *)(tsm + 2 * kTileBufBytes);
  uint64_t *empty = full + 2;
  const int64_t N = p.ntot;
  const int64_t ntiles = (N + kTileE - 1) / kTileE;
  if (threadIdx.x == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], kTileWarps);
    mbar_init(&empty[1], kTileWarps);
    fence_proxy_async();
  }
  __syncthreads();
  const bool issuer = threadIdx.x == 0;
  int64_t t = blockIdx.x;
  // per buffer: phase bits of `full` and `empty`, and (issuer) copies in flight; bit q of
  // each word is buffer q (no per-thread arrays: they would live in local memory)
  uint32_t pf = 0, pe = 0, pending = 0;
  if (t < ntiles && issuer) {
    issue_tile(p, Fin, Vin, t, tsm, &full[0]);
    pending = 1;
  }
  int b = 0;
  bool first = true;
  for (; t < ntiles; t += nblk) {
    const int64_t tn = t + nblk;
    bool ok = true;
    if (issuer && tn < ntiles) {
      const int nb = b ^ 1;
      if (!first) {  // every warp released buffer nb (the previous tile) before its refill
        ok = mbar_wait_ok(&empty[nb], (pe >> nb) & 1u, p.err);
        pe ^= 1u << nb;
      }
      if (ok) {
        fence_proxy_async();
        issue_tile(p, Fin, Vin, tn, tsm + nb * kTileBufBytes, &full[nb]);
        pending |= 1u << nb;
      }
    }
    first = false;
    if (ok) ok = mbar_wait_ok(&full[b], (pf >> b) & 1u, p.err);
    if (!ok) {
      // a copy never landed or a warp never released its buffer (a device fault): the
      // issuer waits, bounded, for the copies it still has in flight; every thread returns
      if (issuer)
        for (int q = 0; q < 2; q++)
          if ((pending >> q) & 1u) mbar_wait_ok(&full[q], (pf >> q) & 1u, p.err);
      return;
    }
    pending &= ~(1u << b);
    pf ^= 1u << b;
    const TileWin w = tile_win(t, N);
    const unsigned char *buf = tsm + b * kTileBufBytes;
#pragma unroll
    for (int u = 0; u < kTileE / kTileThreads; u++) {
      const int64_t l = threadIdx.x + u * kTileThreads;
      if (l < w.cnt) tile_element(p, k, force, buf, w, w.s + l, Fin, Vout, Fout);
    }
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[b]);
    b ^= 1;
  }
}

// ---- a chunk of steps per launch (nrt_options.step_launch = 1)
//
// A step of a small pack (one axon; a myelinated fibre whose arrays sit in L2) is short, so
// the time loop pays a launch per step.  This kernel runs nk steps in one cooperative launch
// (every CTA resident) with a grid barrier after each step.  On a GB300 it is not the
// default: with the loop's launches chained and replayed from a graph, a launch boundary
// costs about what a grid barrier across both dies costs (1002-element FP64 axon 7.42 vs
// 8.17 us per step; the 199k-element myelinated axon without strain 4.63 vs 5.14-5.48 us).
// Every thread owns the same elements at every step (a stride over the grid), so an
// element's gates stay with one thread.  After the barrier that ends step k:
//  - the probes read step k's potentials (step k + 1 writes the other buffer, and step
//    k + 2, which overwrites it, starts after the next barrier);
//  - with a strain ramp, the strained elements take step k + 1's row of the chunk table,
//    behind a second barrier, since a step reads its neighbours' conductances.
// The arithmetic is the per-step kernels' element bodies, so results are theirs bit for bit.
// Data that this kernel writes (V, its FP32 shadow, the strained coefficients) is read with
// ordinary loads after the barrier, whose GPU-scope fences order them after the writes.

// Grid barrier over a cooperative launch.  Arrivals are counted on a 64-bit word that is 0
// when the launch starts; the b-th barrier completes when it reaches b * gridDim.x.  Thread
// 0 of each CTA arrives after a GPU-scope fence (the CTA's writes, gathered by the CTA
// barrier, become visible first) and polls.  It gives up after about two seconds of clock
// (every CTA is resident, so that means a device fault) and raises the error word.
__device__ __forceinline__ bool grid_barrier(GridBar *g, unsigned long long &target, int *err) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    target += gridDim.x;
    __threadfence();
    atomicAdd(&g->count, 1ull);
    int ok = 1;
    const volatile unsigned long long *c = &g->count;
    if (*c < target) {
      const long long t0 = clock64();
      while (*c < target) {
        if (clock64() - t0 > 4000000000ll) {
          atomicOr(err, 1);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// The last CTA to leave puts the barrier's words back to 0 for the next launch (no CTA polls
// them any more once every CTA has counted itself out).
__device__ __forceinline__ void grid_barrier_exit(GridBar *g) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&g->exits, 1u) == gridDim.x - 1) {
      atomicExch(&g->count, 0ull);
      atomicExch(&g->exits, 0u);
    }
  }
}

template <bool kMixed, int kThreads>
__global__ void __launch_bounds__(kThreads) explicit_steps_chunk(PackView p, int nk, double *V0,
                                                                 double *V1, float *F0, float *F1,
                                                                 RecView r, StrainView s,
                                                                 GridBar *gb) {
  chain_acquire();  // the previous launch of the time loop has finished
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  unsigned long long target = 0;
  bool ok = true;
  if (s.n > 0) {
    for (int64_t q = tid; q < s.n; q += nth) apply_row(s, p, (int)q, 0, kMixed);
    ok = grid_barrier(gb, target, p.err);
  }
  for (int k = 0; k < nk && ok; k++) {
    const double *Vin = (k & 1) ? V1 : V0;
    double *Vout = (k & 1) ? V0 : V1;
    for (int64_t j = tid; j < p.ntot; j += nth) {
      if (kMixed)
        mixed_element<false>(p, k, -1, j, Vin, Vout, (k & 1) ? F1 : F0, (k & 1) ? F0 : F1);
      else
        f64_element<false>(p, k, -1, j, Vin, Vout);
    }
    ok = grid_barrier(gb, target, p.err);
    if (!ok) break;
    for (int64_t q = tid; q < r.nprobe; q += nth) {  // as record_step after step k
      const InstDev in = p.inst[r.inst[q]];
      const int64_t i = in.base + k;
      if (i < in.iend) record_probe(r, (int)q, i, Vout[r.src[q]], in.dT);
    }
    if (s.n > 0 && k + 1 < nk) {
      for (int64_t q = tid; q < s.n; q += nth) apply_row(s, p, (int)q, k + 1, kMixed);
      ok = grid_barrier(gb, target, p.err);
    }
  }
  grid_barrier_exit(gb);
}

// V_t = V_source(t) for every terminal (src/solverEx-cpu.cpp:155-161).
__global__ void terminal_fixup(const Topo *__restrict__ topo, const int64_t *__restrict__ terms,
                               int64_t nterm, double *__restrict__ V, float *__restrict__ Vf) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nterm) return;
  const int64_t t = terms[q];
  const int64_t s = ghost_source(topo[t], t);
  V[t] = V[s];
  if (Vf) Vf[t] = Vf[s];
}

__global__ void advance_base(InstDev *inst, int32_t ninst, int64_t steps) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ninst) return;
  int64_t b = inst[i].base + steps;
  inst[i].base = b < inst[i].iend ? b : inst[i].iend;
}

}  // namespace

int launch_explicit_step(const PackView &pv, int precision, bool general, int k, int force,
                         const double *Vin, double *Vout, const float *Fin, float *Fout,
                         cudaStream_t st, const StrainFold *fold) {
  StrainFold f{};
  f.row = -1;
  if (fold && precision == NRT_MIXED && !general) f = *fold;
  // CTAs that write the next step's strained rows, after the ones that step
  const unsigned fold_blocks =
      f.row >= 0 ? (unsigned)std::min(64, (f.s.n + kTileThreads - 1) / kTileThreads) : 0u;
  // Small trees: spread the elements over as many SMs as possible (the FP64 pipe of one
  // SM, not memory, bounds a small block); large packs: 256-thread blocks.
  int threads = 256;
  while (threads > 32 && pv.ntot < (int64_t)threads * 2 * (pv.sms > 0 ? pv.sms : 1)) threads >>= 1;
  if (pv.step_threads > 0) threads = pv.step_threads;  // a tuned shape (same results)
  const unsigned blocks = (unsigned)((pv.ntot + threads - 1) / threads);
  if (precision == NRT_MIXED) {
    if (!general && pv.tile_blocks > 0 && pv.eflags && pv.err) {
      f.first_block = pv.tile_blocks;
      NRT_CUDA(launch_chained(explicit_step_mixed_tiled, pv.tile_blocks + fold_blocks,
                              kTileThreads, 2 * kTileBufBytes + 32, st, pv, k, force, Vin, Vout,
                              Fin, Fout, f));
    } else {
      f.first_block = (int)blocks;
      NRT_CUDA(launch_chained(general ? explicit_step_mixed<true> : explicit_step_mixed<false>,
                              blocks + (f.row >= 0 ? (unsigned)std::min(64, (f.s.n + threads - 1) /
                                                                                   threads)
                                                   : 0u),
                              threads, 0, st, pv, k, force, Vin, Vout, Fin, Fout, f));
    }
  } else if (pv.step_threads == 0 && pv.ntot * kRateLanes <= (int64_t)64 * 1024) {
    // small packs (up to 8192 elements): eight lanes per element, 128-thread blocks
    const unsigned lb = (unsigned)((pv.ntot * kRateLanes + 127) / 128);
    NRT_CUDA(launch_chained(general ? explicit_step_f64_lanes<true> : explicit_step_f64_lanes<false>,
                            lb, 128, 0, st, pv, k, force, Vin, Vout));
  } else {
    NRT_CUDA(launch_chained(general ? explicit_step_f64<true> : explicit_step_f64<false>, blocks,
                            threads, 0, st, pv, k, force, Vin, Vout));
  }
  return NRT_OK;
}

// nk steps of the time loop in one cooperative launch (explicit_steps_chunk).  Threads per
// CTA: step_threads when set, else up to 1024 (mixed; 256 in FP64, whose element body needs
// more than 64 registers) while the pack fills every SM at one element per thread, and fewer
// (down to 32) for small packs, which spreads them over more SMs (an FP64 pack over more
// FP64 pipes).  CTAs: as many as the elements need, at most the resident limit (at most
// per_sm_cap per SM when that is positive).
int launch_explicit_chunk(const PackView &pv, int precision, int nk, double *V0, double *V1,
                          float *F0, float *F1, const RecView &r, const StrainView &s,
                          GridBar *gb, int per_sm_cap, cudaStream_t st) {
  if (nk <= 0) return NRT_OK;
  const bool mixed = precision == NRT_MIXED;
  int threads = mixed ? 1024 : 256;
  while (threads > 32 && pv.ntot < (int64_t)threads * (pv.sms > 0 ? pv.sms : 1)) threads >>= 1;
  if (pv.step_threads > 0) threads = pv.step_threads;
  void *fn = !mixed ? (void *)explicit_steps_chunk<false, 256>
                    : (threads > 256 ? (void *)explicit_steps_chunk<true, 1024>
                                     : (void *)explicit_steps_chunk<true, 256>);
  int per_sm = 0;
  NRT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0));
  if (per_sm_cap > 0) per_sm = std::min(per_sm, per_sm_cap);
  if (per_sm <= 0) return NRT_EINVAL;
  const int64_t need = (pv.ntot + threads - 1) / threads;
  const unsigned blocks = (unsigned)std::min<int64_t>((int64_t)pv.sms * per_sm, need);
  PackView p = pv;
  RecView rv = r;
  StrainView sv = s;
  int nk_ = nk;
  void *args[] = {&p, &nk_, &V0, &V1, &F0, &F1, &rv, &sv, &gb};
  NRT_CUDA(cudaLaunchCooperativeKernel(fn, blocks, threads, args, 0, st));
  count_launch_on(st);
  return NRT_OK;
}

// Persistent CTAs for the tiled mixed step on this device (0 if it cannot run): as many
// per SM as fit, or at most per_sm_cap when that is positive (a tuned shape; the kernel
// strides over the tiles, so any grid gives the same results).
int explicit_tile_blocks(int device, int64_t ntot, int per_sm_cap) {
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, explicit_step_mixed_tiled,
                                                    kTileThreads, 2 * kTileBufBytes + 32) !=
          cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (per_sm_cap > 0) per_sm = std::min(per_sm, per_sm_cap);
  const int64_t ntiles = (ntot + kTileE - 1) / kTileE;
  return (int)std::min<int64_t>((int64_t)sms * per_sm, ntiles);
}

int launch_terminal_fixup(const Topo *topo, const int64_t *terms, int64_t nterm, double *V,
                          float *Vf, cudaStream_t st) {
  if (nterm <= 0) return NRT_OK;
  terminal_fixup<<<(unsigned)((nterm + 255) / 256), 256, 0, st>>>(topo, terms, nterm, V, Vf);
  count_launch_on(st);
  NRT_CUDA(cudaGetLastError());
  return NRT_OK;
}

int launch_advance_base(InstDev *inst, int32_t ninst, int64_t steps, cudaStream_t st) {
  NRT_CUDA(launch_chained(advance_base, (ninst + 255) / 256, 256, 0, st, inst, ninst, steps));
  return NRT_OK;
}

}  // namespace nrt
