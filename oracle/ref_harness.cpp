// Headless driver around the reference's own CPU code (test infrastructure only).
//
// This file is linked against the UNMODIFIED reference sources (src/solverEx-cpu.cpp,
// src/discretization.cpp, src/coupling.cpp, src/init.cpp, src/space.cpp,
// src/mechanical_model.cpp, src/configuration.cpp; and, for the implicit
// solver, src/solverIm-cpu.cpp with the RCI shim in mkl_shim.cpp) by oracle/Makefile into oracle/_ref/.
// It replaces the GL-bound src/neurite.cpp:84-291 with a driver that
//   1. reads a tree description written by the package's model builder
//      (one row per element: kind, mother, DR, DL, branching, geometry, strain,
//      stimulus, material constants),
//   2. builds reference `Cable` / `Hodgkin_Huxley` objects from it,
//   3. runs the reference's own parameter pipeline in the order of
//      src/neurite.cpp:151-177 (mechanical_model_initialization, electrical_properties,
//      setting_rest_pot, hhIconds, cable_init_constants, critical_time_step_class,
//      critical_time_step_selection),
//   4. runs the reference's own solver through the `Solver` interface with the
//      loop semantics of src/neurite.cpp:224-255 (t = i*dT, i = 1 .. numStepsT-2,
//      update(init_time <= t <= end_input), calculate()),
//   5. writes the derived parameters, a probe trace and the final state as text.
//
// Material constants that the reference keeps in protected fields (rho_a, rest
// potential, membrane constants, channel densities) are set directly; the Makefile
// compiles this unit with -Dprivate=public -Dprotected=public for that purpose
// (no reference file is edited).  E_Na0/E_K0 are re-derived from the element's
// rest potential with the constructor's own rule (src/discretization.cpp:80-84).
#include "configuration.h"
#include "neurite.h"
#include "discretization.h"
#include "init.h"
#include "coupling.h"
#include "solver.h"
#include "solverEx-cpu.h"
#include "space.h"
#ifdef WITH_IMPLICIT
#include "solverIm-cpu.h"
#endif
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

// Globals the reference sources declare extern (src/neurite.cpp:69-81 defines them there).
int numStepsX = 0, numStepsT = 0;
TYPE xspan = 0., tspan = 0., dist_mes = 0;
const TYPE pi = 3.14159265;
int *terminals;
int num_terminals;
TYPE **potential, *potentialR;
TYPE *open_GL_graphE, **open_GL_graphR, ***open_GL_graph;
char *log_file, *output;
FILE *standard, *study;
TYPE unit_x = 0.;
int open_GL_steps = 1000;
char *simulation;
TYPE *neuriteE, **neuriteR, ***neurite;
TYPE ***act_trans, **props, *ini;
int tot_santa, alloc_santa, num_props;
int **n_micro, *n_microE;

static void die(const char *msg) {
  fprintf(stderr, "ref_harness: %s\n", msg);
  exit(2);
}

static void expect(FILE *f, const char *key) {
  char buf[128];
  if (fscanf(f, "%127s", buf) != 1 || strcmp(buf, key) != 0) {
    fprintf(stderr, "ref_harness: expected '%s', got '%s'\n", key, buf);
    exit(2);
  }
}

// Mode L: the reference's own loader of a segmented neuron (src/space.cpp:37-183, selected
// by simulation=CT_segmented_neuron at src/init.cpp:120-121) reads <dir>/neuron_for_neurite.txt
// (through the working_directory variable, as the reference's driver arranges it); the
// elements it builds are written to <out.txt>: one line "n num_terminals", the terminals,
// then per element "mother DR DL branching dX diameter input_current" (%.17g).
static int dump_loader(const char *dir, const char *out_path) {
  setenv("working_directory", dir, 1);
  standard = stdout;
  input in;
  memset(&in, 0, sizeof(in));
  discretization **element = NULL;
  Cable **ct = NULL;
  int num_ct = 0;
  loading_neuron_passive_dendritic_tree(in, element, ct, num_ct);
  FILE *o = fopen(out_path, "w");
  if (!o) die("cannot open output");
  fprintf(o, "%d %d\n", numStepsX, num_terminals);
  for (int i = 0; i < num_terminals; i++) fprintf(o, "%d ", terminals[i]);
  fprintf(o, "\n");
  for (int i = 0; i < numStepsX; i++) {
    discretization *e = element[i];
    fprintf(o, "%d %d %d %d %.17g %.17g %.17g\n", e->get_mother(), e->get_DR(), e->get_DL(),
            e->get_branching() ? 1 : 0, e->get_dX(), e->get_diameter(), e->get_input_current());
  }
  fclose(o);
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 4) die("usage: ref_harness <spec.txt | dir> <out.txt> <e|i|L>");
  if (argv[3][0] == 'L') return dump_loader(argv[1], argv[2]);
  FILE *f = fopen(argv[1], "r");
  if (!f) die("cannot open spec");
  bool implicit_mode = (argv[3][0] == 'i');

  int N = 0, T = 0, record_every = 1, nprobe = 0, myelin_global = 0;
  double dt_abs = 0, dtf = 1, t_span = 0, init_time = 0, end_input = 0, e_max = 1;
  expect(f, "NEURITE_SPEC");
  int version; if (fscanf(f, "%d", &version) != 1) die("version");
  expect(f, "num_elem"); if (fscanf(f, "%d", &N) != 1) die("num_elem");
  expect(f, "num_term"); if (fscanf(f, "%d", &T) != 1) die("num_term");
  std::vector<int> term(T);
  expect(f, "terminals");
  for (int i = 0; i < T; i++) if (fscanf(f, "%d", &term[i]) != 1) die("terminals");
  expect(f, "dt_abs"); if (fscanf(f, "%lf", &dt_abs) != 1) die("dt_abs");
  expect(f, "dtf"); if (fscanf(f, "%lf", &dtf) != 1) die("dtf");
  expect(f, "tspan"); if (fscanf(f, "%lf", &t_span) != 1) die("tspan");
  expect(f, "init_time"); if (fscanf(f, "%lf", &init_time) != 1) die("init_time");
  expect(f, "end_input"); if (fscanf(f, "%lf", &end_input) != 1) die("end_input");
  expect(f, "e_max"); if (fscanf(f, "%lf", &e_max) != 1) die("e_max");
  expect(f, "myelin"); if (fscanf(f, "%d", &myelin_global) != 1) die("myelin");
  expect(f, "record_every"); if (fscanf(f, "%d", &record_every) != 1) die("record_every");
  expect(f, "num_probes"); if (fscanf(f, "%d", &nprobe) != 1) die("num_probes");
  std::vector<int> probes(nprobe);
  expect(f, "probes");
  for (int i = 0; i < nprobe; i++) if (fscanf(f, "%d", &probes[i]) != 1) die("probes");
  expect(f, "elements");

  numStepsX = N;
  num_terminals = T;
  terminals = new int[T];
  for (int i = 0; i < T; i++) terminals[i] = term[i];
  tspan = t_span;

  discretization **element = new discretization *[N];
  std::vector<Hodgkin_Huxley *> hh;
  std::vector<Cable *> ct;
  for (int i = 0; i < N; i++) {
    int kind, mother, dr, dl, branching;
    double dX, diam, eps, iinj, ro_a, ro_m, per_m, th, rest, sNa, sK, sL;
    if (fscanf(f, "%d %d %d %d %d %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf",
               &kind, &mother, &dr, &dl, &branching, &dX, &diam, &eps, &iinj, &ro_a,
               &ro_m, &per_m, &th, &rest, &sNa, &sK, &sL) != 17)
      die("element row");
    discretization *e;
    if (kind == 1) {
      Hodgkin_Huxley *h = new Hodgkin_Huxley(i, dr, mother, dX);
      h->rest_pot = rest;
      h->E_Na = 0.115 + rest;  // src/discretization.cpp:80-84 with this element's rest potential
      h->E_Na0 = h->E_Na;
      h->E_K = -0.012 + rest;
      h->E_K0 = h->E_K;
      h->sigma_Na = sNa;
      h->sigma_K = sK;
      h->sigma_L = sL;
      hh.push_back(h);
      e = h;
    } else {
      Cable *c = new Cable(i, dr, mother, dX);
      c->rest_pot = rest;
      ct.push_back(c);
      e = c;
    }
    e->set_epsilon(eps);
    e->set_DL(dl);
    e->set_branching(branching != 0);
    e->set_diameter(diam);
    e->set_input_current(iinj);
    e->ro_a = ro_a;
    e->ro_m = ro_m;
    e->per_m = per_m;
    e->thickness = th;
    element[i] = e;
  }
  fclose(f);

  int num_HH = (int)hh.size(), num_CT = (int)ct.size();
  Hodgkin_Huxley **HH_elements = new Hodgkin_Huxley *[num_HH > 0 ? num_HH : 1];
  Cable **CT_elements = new Cable *[num_CT > 0 ? num_CT : 1];
  for (int i = 0; i < num_HH; i++) HH_elements[i] = hh[i];
  for (int i = 0; i < num_CT; i++) CT_elements[i] = ct[i];

  // src/neurite.cpp:151 with a zero macroscopic strain: only the per-element dX scaling runs.
  input in;
  memset(&in, 0, sizeof(in));
  in.epsilon = 0;
  in.E_MAX = e_max;
  in.init_time = init_time;
  in.end_input = end_input;
  TYPE dm = 0;
  mechanical_model_initialization(in, element, dm);

  // src/neurite.cpp:153: the reference's measurement point (src/init.cpp:339-358) for a
  // few distances: zero, the first element's dX, fractions of the total length, the
  // total itself and twice it (never reached).
  double total = 0;
  for (int i = 0; i < N; i++) total += element[i]->get_dX();
  std::vector<double> mp_dist;
  mp_dist.push_back(0.0);
  mp_dist.push_back(element[0]->get_dX());
  mp_dist.push_back(element[0]->get_dX() + element[1]->get_dX());
  const double frac[] = {0.1, 0.25, 0.5, 0.75, 0.999};
  for (int q = 0; q < 5; q++) mp_dist.push_back(frac[q] * total);
  mp_dist.push_back(total);
  mp_dist.push_back(2.0 * total);
  std::vector<int> mp_index;
  for (size_t q = 0; q < mp_dist.size(); q++) mp_index.push_back(measurement_point(element, mp_dist[q]));

  // src/neurite.cpp:165-177 (neuriteInit replaced by the two potential buffers it allocates).
  potentialR = new TYPE[2 * N]();
  potential = new TYPE *[2];
  potential[0] = potentialR;
  potential[1] = potentialR + N;
  TYPE E_MAX = e_max;
  electrical_properties(HH_elements, num_HH, E_MAX);
  setting_rest_pot(potential, element);
  hhIconds(potential[0], HH_elements, num_HH, E_MAX);
  cable_init_constants(CT_elements, num_CT, myelin_global != 0);
  critical_time_step_class(HH_elements, num_HH, CT_elements, num_CT);
  TYPE dT_crit = critical_time_step_selection(element);
  TYPE dT = (dt_abs > 0) ? dt_abs : dT_crit * dtf;
  TYPE temp = tspan / dT;
  numStepsT = int(temp);

  FILE *o = fopen(argv[2], "w");
  if (!o) die("cannot open output");
  fprintf(o, "dT_crit %.17g\n", dT_crit);
  fprintf(o, "dT %.17g\n", dT);
  fprintf(o, "numStepsT %d\n", numStepsT);
  fprintf(o, "measurement_points %d\n", (int)mp_dist.size());
  for (size_t q = 0; q < mp_dist.size(); q++) fprintf(o, "%.17g %d\n", mp_dist[q], mp_index[q]);
  fprintf(o, "elem_params %d\n", N);  // c_m r_a dX W K critical_dT
  for (int i = 0; i < N; i++)
    fprintf(o, "%.17g %.17g %.17g %.17g %.17g %.17g\n", element[i]->get_c_m(),
            element[i]->get_r_a(), element[i]->get_dX(), element[i]->get_W(),
            element[i]->get_K(), element[i]->get_critical_dT());
  fprintf(o, "hh_params %d\n", num_HH);  // elem m h n g_Na g_K G_L E_Na E_K E_L LS_Na LS_K rest
  for (int i = 0; i < num_HH; i++) {
    Hodgkin_Huxley *h = HH_elements[i];
    fprintf(o, "%d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n",
            h->get_element(), h->get_m(), h->get_h(), h->get_n(), h->get_g_Na(), h->get_g_K(),
            h->get_G_L(), h->get_E_Na(), h->get_E_K(), h->get_E_L(), h->get_Left_Shift_Na(),
            h->get_Left_Shift_K(), h->get_rest_pot());
  }

  Solver *solver;
  if (implicit_mode) {
#ifdef WITH_IMPLICIT
    solver = new SolverImCPU(dT, potential, num_terminals, terminals, 0, num_HH, HH_elements, N, element);
#else
    die("built without the implicit solver");
    return 2;
#endif
  } else {
    solver = new SolverExCPU(dT, potential, num_terminals, terminals, 0, num_HH, HH_elements, N, element);
  }

  std::vector<double> snap(N);
  int nrec = 0;
  std::vector<double> trace;
  for (int i = 1; i < numStepsT - 1; i++) {
    TYPE time_run = i * dT;
    solver->update((time_run >= in.init_time) && (time_run <= in.end_input));
    solver->calculate();
    if (record_every > 0 && (i % record_every) == 0) {
      solver->snapshot(&snap[0]);
      trace.push_back((double)i);
      for (int p = 0; p < nprobe; p++) trace.push_back(snap[probes[p]]);
      nrec++;
    }
  }
  solver->snapshot(&snap[0]);
  fprintf(o, "trace %d %d\n", nrec, nprobe);
  for (int r = 0; r < nrec; r++) {
    for (int p = 0; p <= nprobe; p++) fprintf(o, p ? " %.17g" : "%.17g", trace[r * (nprobe + 1) + p]);
    fprintf(o, "\n");
  }
  fprintf(o, "final_V %d\n", N);
  for (int i = 0; i < N; i++) fprintf(o, "%.17g\n", snap[i]);
  fprintf(o, "final_gates %d\n", num_HH);
  for (int i = 0; i < num_HH; i++)
    fprintf(o, "%.17g %.17g %.17g\n", HH_elements[i]->get_m(), HH_elements[i]->get_h(),
            HH_elements[i]->get_n());
  fclose(o);
  delete solver;
  return 0;
}
