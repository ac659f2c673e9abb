// Drives SolverExGB300 / SolverImGB300 through the reference's Solver* loop
// (src/neurite.cpp:185-255): construct with the reference constructor arguments, then
// update(t in window) + calculate() per step and snapshot() at the end.  Reads the
// flattened tree written by tests/test_dropin.py; writes the final potential.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "configuration.h"
#include "discretization.h"
#include "solver.h"
#include "neurite_gb300_solver.hpp"

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FILE *f = fopen(argv[1], "r");
  if (!f) return 2;
  int N, T, H, steps, mode;
  double dT, t0, t1;
  if (fscanf(f, "%d %d %d %d %lf %lf %lf", &mode, &N, &T, &steps, &dT, &t0, &t1) != 7) return 3;
  std::vector<int> term(T);
  for (int i = 0; i < T; i++) if (fscanf(f, "%d", &term[i]) != 1) return 3;
  if (fscanf(f, "%d", &H) != 1) return 3;
  std::vector<char> is_hh(N, 0);
  std::vector<int> hh_idx(H);
  for (int k = 0; k < H; k++) { if (fscanf(f, "%d", &hh_idx[k]) != 1) return 3; is_hh[hh_idx[k]] = 1; }
  std::vector<discretization *> el(N);
  std::vector<Hodgkin_Huxley *> hh;
  std::vector<double> V0(N);
  for (int i = 0; i < N; i++) {
    discretization *e = is_hh[i] ? new Hodgkin_Huxley() : new discretization();
    int br;
    if (fscanf(f, "%d %d %d %d %lf %lf %lf %lf %lf %lf %lf", &e->mother, &e->DR, &e->DL, &br, &e->dX,
               &e->c_m, &e->r_a, &e->W, &e->K, &e->input_current, &V0[i]) != 11) return 3;
    e->element = i;
    e->branching = br != 0;
    el[i] = e;
  }
  for (int k = 0; k < H; k++) {
    Hodgkin_Huxley *e = (Hodgkin_Huxley *)el[hh_idx[k]];
    if (fscanf(f, "%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", &e->m, &e->h, &e->n, &e->g_Na,
               &e->g_K, &e->G_L, &e->E_Na, &e->E_K, &e->E_L, &e->LS_Na, &e->LS_K, &e->rest_pot) != 12)
      return 3;
    hh.push_back(e);
  }
  fclose(f);
  double *potential[2] = {&V0[0], &V0[0]};
  Solver *solver;
  try {
    if (mode == 0)
      solver = new SolverExGB300(dT, potential, T, &term[0], 0, H, H ? &hh[0] : 0, N, &el[0]);
    else
      solver = new SolverImGB300(dT, potential, T, &term[0], 0, H, H ? &hh[0] : 0, N, &el[0]);
    for (int i = 1; i <= steps; i++) {
      double time_run = i * dT;
      solver->update((time_run >= t0) && (time_run <= t1));
      solver->calculate();
    }
    std::vector<double> out(N);
    solver->snapshot(&out[0]);
    delete solver;
    FILE *o = fopen(argv[2], "w");
    for (int i = 0; i < N; i++) fprintf(o, "%.17g\n", out[i]);
    fclose(o);
  } catch (neurite_gb300::Error &e) {
    fprintf(stderr, "%s\n", e.what());
    return 4;
  }
  return 0;
}
