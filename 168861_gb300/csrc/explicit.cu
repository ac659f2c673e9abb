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
#include "hh.cuh"
#include "nrt_internal.h"

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

template <bool kGeneral>
__global__ void __launch_bounds__(256) explicit_step_f64(PackView p, int k, int force,
                                                         const double *__restrict__ Vin,
                                                         double *__restrict__ Vout) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.ntot) return;
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
    GateStep64 g = hh_step64(v, p.gate[j], p.gate[N + j], p.gate[2 * N + j],
                             hp[HP_LSNA * L], hp[HP_LSK * L], hp[HP_REST * L],
                             hp[HP_DTMS * L], hp[HP_GNA * L], hp[HP_GK * L],
                             hp[HP_GL * L], hp[HP_ENA * L], hp[HP_EK * L],
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

// Mixed precision: gates, rates, conductances and currents in FP32; the potential is
// accumulated in FP64.  GB300's FP64 pipe runs at 1/61 of the FP32 rate, so the stencil
// reads an FP32 shadow of V (Vf = (float)V, refreshed from the FP64 value every step):
// neighbour differences carry an absolute error of ~4e-9 V, while the FP64 accumulator
// V' = V + dt-scaled current keeps long horizons free of drift.  FP64-pipe work is one
// conversion, one add and one conversion back per element.
template <bool kGeneral>
__global__ void __launch_bounds__(256) explicit_step_mixed(PackView p, int k, int force,
                                                           const double *__restrict__ Vin,
                                                           double *__restrict__ Vout,
                                                           const float *__restrict__ Fin,
                                                           float *__restrict__ Fout) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.ntot) return;
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
    const int64_t L = p.hp_ld;
    const float *hp = p.hpf + (p.hp_cls ? (int64_t)cls : (p.hp_inst ? (int64_t)inst : j));
    const float dv = vf - hp[HP_REST * L];
    GateStep32 g = hh_step32(dv + hp[HP_LSNA * L], dv + hp[HP_LSK * L], m0, h0, n0,
                             hp[HP_DTMS * L], hp[HP_GNA * L], hp[HP_GK * L], hp[HP_GL * L],
                             hp[HP_ENA * L], hp[HP_EK * L], hp[HP_EL * L]);
    p.gatef[j] = g.m;
    p.gatef[N + j] = g.h;
    p.gatef[2 * N + j] = g.n;
    if (term) return;
    const float dx = hp[HP_DX * L];
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
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ninst) return;
  int64_t b = inst[i].base + steps;
  inst[i].base = b < inst[i].iend ? b : inst[i].iend;
}

}  // namespace

int launch_explicit_step(const PackView &pv, int precision, bool general, int k, int force,
                         const double *Vin, double *Vout, const float *Fin, float *Fout,
                         cudaStream_t st) {
  // Small trees: spread the elements over as many SMs as possible (the FP64 pipe of one
  // SM, not memory, bounds a small block); large packs: 256-thread blocks.
  int threads = 256;
  while (threads > 32 && pv.ntot < (int64_t)threads * 2 * 152) threads >>= 1;
  const unsigned blocks = (unsigned)((pv.ntot + threads - 1) / threads);
  if (precision == NRT_MIXED) {
    if (general)
      explicit_step_mixed<true><<<blocks, threads, 0, st>>>(pv, k, force, Vin, Vout, Fin, Fout);
    else
      explicit_step_mixed<false><<<blocks, threads, 0, st>>>(pv, k, force, Vin, Vout, Fin, Fout);
  } else {
    if (general)
      explicit_step_f64<true><<<blocks, threads, 0, st>>>(pv, k, force, Vin, Vout);
    else
      explicit_step_f64<false><<<blocks, threads, 0, st>>>(pv, k, force, Vin, Vout);
  }
  NRT_CUDA(cudaGetLastError());
  return NRT_OK;
}

int launch_terminal_fixup(const Topo *topo, const int64_t *terms, int64_t nterm, double *V,
                          float *Vf, cudaStream_t st) {
  if (nterm <= 0) return NRT_OK;
  terminal_fixup<<<(unsigned)((nterm + 255) / 256), 256, 0, st>>>(topo, terms, nterm, V, Vf);
  NRT_CUDA(cudaGetLastError());
  return NRT_OK;
}

int launch_advance_base(InstDev *inst, int32_t ninst, int64_t steps, cudaStream_t st) {
  advance_base<<<(ninst + 255) / 256, 256, 0, st>>>(inst, ninst, steps);
  NRT_CUDA(cudaGetLastError());
  return NRT_OK;
}

}  // namespace nrt
