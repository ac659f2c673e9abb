// neurite_gb300_solver.hpp -- drop-in C++ solvers for the reference's driver (C++98).
//
// SolverExGB300 / SolverImGB300 derive from the reference's `Solver` (inc/solver.h:12-24)
// and take exactly the constructor arguments of SolverExGPU / SolverImGPU
// (inc/solverEx-gpu.h:79-82, inc/solverIm-gpu.h:111-114; also SolverExCPU / SolverImCPU,
// inc/solverEx-cpu.h:35-38, inc/solverIm-cpu.h:52-55).  They flatten the element objects
// into plain arrays -- the reads src/solverEx-gpu.cpp:266-399 performs -- and hand them to
// the C ABI in neurite_gb300.h.  Include the reference's "configuration.h",
// "discretization.h" and "solver.h" before this header (they define TYPE, Solver,
// discretization and Hodgkin_Huxley) and link libneurite_gb300.so.  The header is C++98,
// like the reference (whose logging macros do not compile as C++11).
//
// Differences from the reference classes, by design:
//  * inputs are copied; caller-owned Hodgkin_Huxley objects are never mutated (the GPU
//    reference behaves the same; SolverExCPU writes gates back into them);
//  * failures throw neurite_gb300::Error (a std::runtime_error) instead of calling
//    std::terminate through a throw() specification or exit(0);
//  * `input_val` is ignored, as in every reference solver (input comes from
//    element->get_input_current()).
#ifndef NEURITE_GB300_SOLVER_HPP
#define NEURITE_GB300_SOLVER_HPP

#include <algorithm>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "neurite_gb300.h"

namespace neurite_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string &where)
      : std::runtime_error(where + ": " + nrt_status_string(status) + " (" + nrt_last_error() + ")"),
        status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char *where) {
  if (status != NRT_OK) throw Error(status, where);
}

// Flattened copy of the reference's element objects (what nrt_problem points into).
struct Flat {
  std::vector<int32_t> mother, dr, dl, branching, terminals, hh_elem;
  std::vector<double> dx, c_m, r_a, W, K, input;
  std::vector<double> m, h, n, g_Na, g_K, G_L, E_Na, E_K, E_L, ls_Na, ls_K, rest, V0, V1;
  nrt_problem p;

  template <class Elem, class HH>
  Flat(double dT, double **potential, int num_term, const int *ind_terminals, int num_HH,
       HH **hh, int num_elem, Elem **element) {
    const size_t N = (size_t)num_elem;
    mother.resize(N); dr.resize(N); dl.resize(N); branching.resize(N);
    dx.resize(N); c_m.resize(N); r_a.resize(N); W.resize(N); K.resize(N); input.resize(N);
    for (size_t i = 0; i < N; i++) {
      mother[i] = element[i]->get_mother();
      dr[i] = element[i]->get_DR();
      dl[i] = element[i]->get_DL();
      branching[i] = element[i]->get_branching() ? 1 : 0;
      dx[i] = element[i]->get_dX();
      c_m[i] = element[i]->get_c_m();
      r_a[i] = element[i]->get_r_a();
      W[i] = element[i]->get_W();
      K[i] = element[i]->get_K();
      input[i] = element[i]->get_input_current();
    }
    terminals.assign(ind_terminals, ind_terminals + num_term);
    // HH elements in ascending element order (the reference builders already emit them so)
    std::vector<std::pair<int, int> > order;
    for (int k = 0; k < num_HH; k++) order.push_back(std::make_pair(hh[k]->get_element(), k));
    std::sort(order.begin(), order.end());
    for (size_t q = 0; q < order.size(); q++) {
      HH *e = hh[order[q].second];
      hh_elem.push_back(e->get_element());
      m.push_back(e->get_m()); h.push_back(e->get_h()); n.push_back(e->get_n());
      g_Na.push_back(e->get_g_Na()); g_K.push_back(e->get_g_K()); G_L.push_back(e->get_G_L());
      E_Na.push_back(e->get_E_Na()); E_K.push_back(e->get_E_K()); E_L.push_back(e->get_E_L());
      ls_Na.push_back(e->get_Left_Shift_Na()); ls_K.push_back(e->get_Left_Shift_K());
      rest.push_back(e->get_rest_pot());
    }
    V0.assign(potential[0], potential[0] + N);
    V1.assign(potential[1], potential[1] + N);
    p.num_elem = num_elem;
    p.mother = &mother[0]; p.dr = &dr[0]; p.dl = &dl[0]; p.branching = &branching[0];
    p.num_term = num_term; p.terminals = &terminals[0];
    p.dx = &dx[0]; p.c_m = &c_m[0]; p.r_a = &r_a[0]; p.W = &W[0]; p.K = &K[0];
    p.input = &input[0];
    p.num_hh = num_HH;
    p.hh_elem = num_HH ? &hh_elem[0] : 0;
    p.m = num_HH ? &m[0] : 0; p.h = num_HH ? &h[0] : 0; p.n = num_HH ? &n[0] : 0;
    p.g_Na = num_HH ? &g_Na[0] : 0; p.g_K = num_HH ? &g_K[0] : 0; p.G_L = num_HH ? &G_L[0] : 0;
    p.E_Na = num_HH ? &E_Na[0] : 0; p.E_K = num_HH ? &E_K[0] : 0; p.E_L = num_HH ? &E_L[0] : 0;
    p.ls_Na = num_HH ? &ls_Na[0] : 0; p.ls_K = num_HH ? &ls_K[0] : 0;
    p.rest = num_HH ? &rest[0] : 0;
    p.V0 = &V0[0]; p.V1 = &V1[0];
    p.dT = dT;
  }
};

// Common body of the two solvers: update / calculate / snapshot over one nrt_solver.
class SolverGB300 : public Solver {
 public:
  virtual void update(bool input_active) { check(nrt_update(s_, input_active ? 1 : 0), "update"); }
  virtual void calculate() { check(nrt_calculate(s_), "calculate"); }
  virtual void snapshot(TYPE *potential) { check(nrt_snapshot(s_, potential), "snapshot"); }
  virtual ~SolverGB300() { nrt_destroy(s_); }
  nrt_solver *handle() { return s_; }

 protected:
  template <class Elem, class HH>
  SolverGB300(int mode, const nrt_options *base, TYPE dT, TYPE **potential, int num_term,
              int *ind_terminals, int num_HH_elements, HH **HH_elements, int num_elem,
              Elem **element)
      : s_(0) {
    Flat f(dT, potential, num_term, ind_terminals, num_HH_elements, HH_elements, num_elem, element);
    nrt_options o;
    if (base) {
      o = *base;
    } else {
      nrt_options_default(&o);
    }
    o.mode = mode;
    check(nrt_create(&f.p, &o, &s_), "nrt_create");
  }

 private:
  nrt_solver *s_;
};

}  // namespace neurite_gb300

// Replaces `new SolverExGPU(dT, potential, num_term, terminals, input, num_HH, HH, N, element)`
// (src/neurite.cpp:190-191).
class SolverExGB300 : public neurite_gb300::SolverGB300 {
 public:
  SolverExGB300(TYPE dT, TYPE **potential, int num_term, int *ind_terminals, TYPE input_val,
                int num_HH_elements, Hodgkin_Huxley **HH_elements, int num_elem,
                discretization **element, const nrt_options *opt = 0)
      : SolverGB300(NRT_EXPLICIT, opt, dT, potential, num_term, ind_terminals, num_HH_elements,
                    HH_elements, num_elem, element) {
    (void)input_val;
  }
};

// Replaces `new SolverImGPU(...)` (src/neurite.cpp:193-194).  Default: plain FP64,
// tree-preconditioned GMRES(30), ||r||_2 <= 1e-14 (the reference's RANGE_ERROR test).
class SolverImGB300 : public neurite_gb300::SolverGB300 {
 public:
  SolverImGB300(TYPE dT, TYPE **potential, int num_term, int *ind_terminals, TYPE input_val,
                int num_HH_elements, Hodgkin_Huxley **HH_elements, int num_elem,
                discretization **element, const nrt_options *opt = 0)
      : SolverGB300(NRT_IMPLICIT_BE, opt, dT, potential, num_term, ind_terminals,
                    num_HH_elements, HH_elements, num_elem, element) {
    (void)input_val;
  }
};

#endif  // NEURITE_GB300_SOLVER_HPP
