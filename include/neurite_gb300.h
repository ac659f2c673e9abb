/* neurite_gb300.h -- C ABI of the GB300-native Neurite solver hot path.
 *
 * This is the drop-in boundary for the reference's `Solver` objects (inc/solver.h:12-24):
 * explicit forward Euler (src/solverEx-cpu.cpp, src/solverEx-gpu.cpp) and implicit
 * backward Euler (src/solverIm-cpu.cpp, src/solverIm-gpu.cpp).  Plain pointers and
 * sizes only; every function returns an nrt_status.  The C++ adapter classes with the
 * reference's constructor signature live in neurite_gb300_solver.hpp.
 *
 * Units are the reference's: SI (V, m, s, A, S, F); HH rates use mV relative to rest
 * and dt in ms internally, as src/coupling.cpp:25-48 and src/solverEx-cpu.cpp:96 do.
 *
 * Threading: a handle is not thread-safe; distinct handles are independent.  All work of
 * a handle runs on its own CUDA stream on the device that was current (or named in
 * nrt_options.device) when it was created.
 */
#ifndef NEURITE_GB300_H
#define NEURITE_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference throws cudaException from throw() methods
 * (inc/cudaException.h:81-191, inc/solverEx-gpu.h:83-85) or calls exit(0) on solver
 * failure (src/solverIm-cpu.cpp:247-250); here every failure is a returned code. */
typedef enum nrt_status {
  NRT_OK = 0,
  NRT_EINVAL = 1,         /* null pointer, bad size or option */
  NRT_ETOPOLOGY = 2,      /* tree violates the numbering convention */
  NRT_ENOMEM = 3,         /* device or host allocation failed */
  NRT_ENOCONV = 4,        /* Krylov solve hit its iteration budget (state still advanced) */
  NRT_EDEVICE = 5,        /* CUDA error; see nrt_last_error() */
  NRT_EBUDGET = 6,        /* serving: request exceeds the HBM budget */
  NRT_ESTATE = 7,         /* call out of order (e.g. unknown request id) */
  NRT_ENOTREADY = 8       /* serving: result not finished yet */
} nrt_status;

typedef enum nrt_mode {
  NRT_EXPLICIT = 0,       /* forward Euler, src/solverEx-cpu.cpp:90-168 */
  NRT_IMPLICIT_BE = 1     /* backward Euler, src/solverIm-cpu.cpp:29-370 */
} nrt_mode;

typedef enum nrt_precision {
  NRT_FP64 = 0,           /* plain double everywhere (the drop-in) */
  NRT_MIXED = 1           /* FP32 gates/stencil/inner Krylov; FP64 V accumulator, outer
                             residual and Krylov inner products */
} nrt_precision;

typedef enum nrt_krylov {
  NRT_GMRES = 0,          /* restarted GMRES(m), classical Gram-Schmidt */
  NRT_BICGSTAB = 1        /* BiCGSTAB, src/solverIm-gpu.cpp:725-843; right-preconditioned by
                             precond (NRT_PRECOND_NONE: the reference's form); restarts only
                             for FP64 refinement (mixed) or a breakdown; needs restart >= 3 */
} nrt_krylov;

typedef enum nrt_precond {
  NRT_PRECOND_NONE = 0,
  NRT_PRECOND_JACOBI = 1,    /* diagonal scaling */
  NRT_PRECOND_SEGMENT = 2,   /* exact tridiagonal solve of every unbranched segment
                                (block Jacobi with the branch-point couplings cut) */
  NRT_PRECOND_TREE = 3       /* exact solve of the whole tree (Hines elimination, parallel
                                over the segments of each branch level); GMRES then needs
                                about one iteration per refinement cycle */
} nrt_precond;

/* Implicit time discretisation.  The reference is backward Euler only
 * (src/solverIm-cpu.cpp:83,115).  Crank-Nicolson applies the trapezoidal rule to the same
 * operator: with A = C/dT + L the backward-Euler matrix and b = C/dT V^n + K dX + I, it
 * solves (A + C/dT) x = 2 b + C/dT V^n - A V^n (gates, W and K as in backward Euler). */
typedef enum nrt_scheme {
  NRT_BACKWARD_EULER = 0,
  NRT_CRANK_NICOLSON = 1
} nrt_scheme;

typedef enum nrt_tol_mode {
  NRT_TOL_ABS = 0,        /* ||b - A x||_2 <= tol (the reference's test, RANGE_ERROR 1e-14) */
  NRT_TOL_REL = 1         /* ||b - A x||_2 <= tol * ||b||_2 over the physical rows */
} nrt_tol_mode;

/* One tree, after the reference's parameter pipeline (src/init.cpp:235-298), i.e. what
 * the reference solver constructors read from their `discretization` and
 * `Hodgkin_Huxley` objects (src/solverEx-gpu.cpp:266-434, src/solverIm-gpu.cpp:514-672).
 * Element arrays have num_elem entries, HH arrays num_hh entries.  Nothing is retained:
 * nrt_create copies what it needs. */
typedef struct nrt_problem {
  int32_t num_elem;              /* numStepsX */
  const int32_t *mother;         /* get_mother(); -1 for element 0 */
  const int32_t *dr;             /* get_DR(); == itself for terminals */
  const int32_t *dl;             /* get_DL(); 0 where not branching */
  const int32_t *branching;      /* get_branching() (0/1) */
  int32_t num_term;
  const int32_t *terminals;      /* terminals[0] == 0 is the fictitious root */
  const double *dx, *c_m, *r_a;  /* get_dX(), get_c_m(), get_r_a() */
  const double *W, *K;           /* get_W(), get_K() (HH entries are recomputed) */
  const double *input;           /* get_input_current() */
  int32_t num_hh;
  const int32_t *hh_elem;        /* HH_elements[i]->get_element(), ascending */
  const double *m, *h, *n;       /* gates */
  const double *g_Na, *g_K, *G_L;
  const double *E_Na, *E_K, *E_L;
  const double *ls_Na, *ls_K;    /* get_Left_Shift_Na/K() */
  const double *rest;            /* get_rest_pot() */
  const double *V0;              /* potential[0] (the reference's prevT); NULL -> rest */
  const double *V1;              /* potential[1] (currT); NULL -> V0 */
  double dT;                     /* time step, s */
} nrt_problem;

typedef struct nrt_options {
  int32_t mode;                  /* nrt_mode */
  int32_t precision;             /* nrt_precision */
  int32_t krylov;                /* nrt_krylov */
  int32_t precond;               /* nrt_precond */
  int32_t restart;               /* GMRES restart length (<= 32) */
  int32_t tol_mode;              /* nrt_tol_mode */
  double tol;                    /* residual tolerance per step */
  int32_t max_iter;              /* Krylov iterations per step; 0 -> num_elem */
  int32_t device;                /* CUDA device ordinal; -1 -> current device */
  int32_t use_graphs;            /* capture nrt_run time loops in CUDA graphs (default 1) */
  int32_t schedule;              /* implicit: 0 = auto (one tree -> cooperative whole-GPU
                                    launch), 1 = always block per instance */
  int32_t tiled;                 /* mixed explicit: 1 (default) = element arrays staged into
                                    shared memory by bulk copies, tile by tile; 0 = one
                                    thread per element loading its own (same results) */
  int32_t scheme;                /* implicit: NRT_BACKWARD_EULER (default, the reference's)
                                    or NRT_CRANK_NICOLSON */
  int32_t tile_ctas_per_sm;      /* persistent CTAs per SM, 1 .. as many as fit (0 = as many
                                    as fit, the default): of the mixed explicit tiled step,
                                    and of the implicit block-per-instance kernel (batches) */
  int32_t step_threads;          /* explicit, one thread per element: threads per block, a
                                    multiple of 32 up to 256 (0 = chosen from the tree size;
                                    FP64 packs of up to 8192 elements then take eight lanes
                                    per element).  Launch shapes only: results do not depend
                                    on them */
  double inner_tol;              /* implicit, mixed precision: each FP64 refinement cycle's
                                    inner FP32 Krylov solve stops once its residual estimate
                                    is below inner_tol times the cycle's starting residual
                                    (0 = the default, NRT_INNER_TOL_DEFAULT).  FP64 mode
                                    solves each cycle to the outer tolerance and ignores it */
  int32_t step_launch;           /* explicit time loops (nrt_run, nrt_batch_advance, the
                                    server): 0 = one launch per step (default; chained launches
                                    replayed from a captured graph), 1 = up to 64 steps per
                                    cooperative launch with a grid barrier between steps (on a
                                    GB300 a barrier across both dies costs about what a chained
                                    launch does, so this is not faster there).  Launch shapes
                                    only: results do not depend on it */
  int32_t refinement;            /* implicit, mixed precision, GMRES with the tree
                                    preconditioner: 0 = auto: each FP64 refinement cycle is
                                    one preconditioned Richardson step, x += M^-1 r (M, the
                                    FP32 factorisation of A, solves A up to rounding, so
                                    GMRES's single Arnoldi step would scale M^-1 r by ~1),
                                    for as long as every cycle lowers the true residual at
                                    least tenfold; GMRES cycles from the first that does not.
                                    1 = GMRES cycles always.  Both stop on the same FP64
                                    residual test */
} nrt_options;

/* One FP32 cycle cannot reduce the true residual by much more than 1e-4 on a stiff
 * cable (its preconditioner and products are FP32), so a tighter inner target buys
 * Krylov iterations that the next FP64 residual does not see. */
#define NRT_INNER_TOL_DEFAULT 1e-3

typedef struct nrt_stats {
  int64_t steps;                 /* calculate() calls so far */
  int64_t krylov_iters;          /* total Krylov iterations (implicit) */
  int32_t last_iters;            /* iterations of the last step */
  int32_t nonconverged_steps;    /* steps that hit max_iter */
  double last_residual;          /* ||b - A x||_2 of the last step (FP64) */
  int64_t device_bytes;          /* device memory held by the handle */
} nrt_stats;

typedef struct nrt_solver nrt_solver;

/* Fills the defaults: explicit, FP64, GMRES(30), exact tree preconditioner, absolute
 * tolerance 1e-14 (RANGE_ERROR, inc/configuration.h:16), max_iter 0, device -1. */
int nrt_options_default(nrt_options *opt);

/* Replaces `new SolverExGPU(...)` / `new SolverImGPU(...)`
 * (src/solverEx-gpu.cpp:204-439, src/solverIm-gpu.cpp:381-682): validates the tree,
 * copies every array to device-resident SoA buffers and returns a handle. */
int nrt_create(const nrt_problem *p, const nrt_options *opt, nrt_solver **out);

/* Solver::update(bool input_active), inc/solver.h:16; src/solverEx-gpu.cpp:443-476.
 * Selects the stimulus for the next calculate(); the gating update itself is fused into
 * calculate() (the reference's separate Update_HH launch), so an update() must precede
 * every calculate(), as the reference's driver loop does (src/neurite.cpp:230-236). */
int nrt_update(nrt_solver *s, int input_active);

/* Solver::calculate(), inc/solver.h:18; src/solverEx-gpu.cpp:481-530 and
 * src/solverIm-gpu.cpp:725-843: advances V (and the gates) by one step. */
int nrt_calculate(nrt_solver *s);

/* Solver::snapshot(TYPE *potential), inc/solver.h:21; src/solverEx-gpu.cpp:534-541:
 * copies the latest potential (num_elem doubles) to host memory; synchronous. */
int nrt_snapshot(nrt_solver *s, double *potential);

/* The driver loop of src/neurite.cpp:224-236 on the device: for i in [i_begin, i_end):
 * t = i*dT; update(init_time <= t <= end_input); calculate().  Runs as CUDA-graph
 * replays when use_graphs is set.  Asynchronous on the handle's stream. */
int nrt_run(nrt_solver *s, int64_t i_begin, int64_t i_end, double init_time, double end_input);

/* Waits for the handle's stream. */
int nrt_synchronize(nrt_solver *s);

/* The handle's CUDA stream (a cudaStream_t), e.g. to record timing events on it. */
int nrt_get_stream(nrt_solver *s, void **stream);

/* Device pointer of the latest potential (valid until the next calculate/run). */
int nrt_potential_device(nrt_solver *s, const double **dev_ptr);

/* Exports the gate state (num_hh each, HH order) to host memory; synchronous.  The
 * reference has no such export (snapshot copies V only). */
int nrt_get_gates(nrt_solver *s, double *m, double *h, double *n);

/* Exports the implicit system assembled for the next step in the reference's CSR layout
 * (src/solverIm-cpu.cpp:29-183): row_ptr[num_elem+1], col/val[capacity >= 4*num_elem+2],
 * rhs[num_elem] (rows the reference leaves untouched hold the stale second buffer).
 * Runs the assembly phase for the given stimulus flag without advancing the state. */
int nrt_export_system(nrt_solver *s, int input_active, int32_t *row_ptr, int32_t *col,
                      double *val, double *rhs, int32_t *nnz_out);

int nrt_get_stats(nrt_solver *s, nrt_stats *st);

/* The reference's destructor (src/solverEx-gpu.cpp:546-582): frees everything. */
int nrt_destroy(nrt_solver *s);

/* Human-readable text for a status code, and the last error recorded on this thread. */
const char *nrt_status_string(int status);
const char *nrt_last_error(void);

/* Kernels this library has launched in this process so far, over all handles and threads
 * (a replay of a captured time-loop graph counts each of its kernel nodes; copies and
 * memsets are not kernels).  The difference across a region is its launch count. */
int64_t nrt_kernel_launches(void);

/* ----------------------------------------------------------------------------------
 * Parameter pipeline on the host: the reference's src/init.cpp:320-333 (strain on dX),
 * :235-254 (electrical_properties), :273-298 (hhIconds), :180-198
 * (cable_init_constants), :138-174 (critical time step) for a tree description.
 *   ispec [5][n]  int32: kind (1 HH / 0 cable), mother, DR, DL, branching
 *   dspec [12][n] double: dX, diameter, epsilon, input_current, ro_a, ro_m, per_m,
 *                         thickness, rest_pot, sigma_Na, sigma_K, sigma_L
 * Outputs: eparam [6][n] (c_m, r_a, dX, W, K, critical dT), hh_elem [num_hh],
 * hparam [12][num_hh] (m, h, n, g_Na, g_K, G_L, E_Na, E_K, E_L, LS_Na, LS_K, rest). */
int nrt_derive(int32_t n, const int32_t *ispec, const double *dspec, int32_t myelin,
               double e_max, double *eparam, int32_t *hh_elem, double *hparam,
               int32_t *num_hh_out, double *dT_crit_out);

/* The same pipeline on the GPU for many trees in one call (one CTA per tree), for front
 * ends that admit thousands of trees at once.  Trees are packed back to back: tree t owns
 * elements [offsets[t], offsets[t+1]) of ispec [5][total] and dspec [12][total] (nrt_derive's
 * rows, each spanning all trees; total = offsets[count]).  myelin and e_max are per tree.
 * Outputs: eparam [6][total], hh_offsets [count + 1] (tree t's HH elements are
 * [hh_offsets[t], hh_offsets[t+1]) of hh_elem and of hparam's rows), hh_elem (indices local
 * to the tree), hparam [12][hh_offsets[count]], dT_crit [count].  All arrays are host
 * memory; the call allocates and frees its device buffers.  Results are nrt_derive's up
 * to the last bits of the device's exp, pow, sqrt and fused multiply-adds. */
int nrt_derive_batch(int32_t count, const int64_t *offsets, const int32_t *ispec,
                     const double *dspec, const int32_t *myelin, const double *e_max,
                     double *eparam, int32_t *hh_elem, double *hparam, int64_t *hh_offsets,
                     double *dT_crit);

/* ----------------------------------------------------------------------------------
 * Batches: many independent trees of uneven size advanced together, one persistent
 * block-per-instance launch per chunk of steps.  Each instance keeps its own dT,
 * stimulus window and step counter.  No reference counterpart (the reference runs one
 * tree per process, src/neurite.cpp:84-291). */
typedef struct nrt_batch nrt_batch;

typedef struct nrt_instance_run {
  int64_t i_begin;               /* first loop index (the reference starts at 1) */
  int64_t i_end;                 /* one past the last loop index (numStepsT - 1) */
  double init_time, end_input;   /* stimulus window, s */
} nrt_instance_run;

int nrt_batch_create(const nrt_problem *problems, int32_t count, const nrt_options *opt,
                     nrt_batch **out);
/* Sets every instance's loop range and stimulus window. */
int nrt_batch_set_runs(nrt_batch *b, const nrt_instance_run *runs);
/* Advances every unfinished instance by up to `steps` loop iterations. */
int nrt_batch_advance(nrt_batch *b, int64_t steps);
int nrt_batch_synchronize(nrt_batch *b);
int nrt_batch_get_stream(nrt_batch *b, void **stream);
/* Latest potential of one instance (its num_elem doubles) to host memory. */
int nrt_batch_snapshot(nrt_batch *b, int32_t instance, double *potential);
/* Latest potential of every instance in one copy: the instances' num_elem doubles back
 * to back, in instance order. */
int nrt_batch_snapshot_all(nrt_batch *b, double *potential);
/* Number of loop iterations still to run per instance (count entries). */
int nrt_batch_remaining(nrt_batch *b, int64_t *remaining);
int nrt_batch_get_stats(nrt_batch *b, nrt_stats *st);
/* Per-instance Krylov statistics (implicit): total iterations, iterations of the last
 * step, non-converged steps and the last step's residual; arrays of `count` entries,
 * any of which may be NULL. */
int nrt_batch_instance_stats(nrt_batch *b, int64_t *iters, int32_t *last_iters,
                             int32_t *nonconverged, double *last_residual);
/* Per-instance counts of the implicit kernel's passes over the rows since creation
 * (GMRES): FP64 residuals after the one fused into each step's assembly, preconditioner
 * applications, solution updates, basis vectors read by the Arnoldi steps (the sum of
 * j + 1 over steps j), and Richardson refinement steps (nrt_options.refinement; not
 * counted as Krylov iterations).  With the iteration count they give the bytes a step
 * moved.  Arrays of `count` entries; any may be NULL.  No reference counterpart. */
int nrt_batch_pass_counts(nrt_batch *b, int64_t *residuals, int64_t *precond_applies,
                          int64_t *xupdates, int64_t *basis_reads, int64_t *richardson_steps);
int nrt_batch_destroy(nrt_batch *b);

/* ----------------------------------------------------------------------------------
 * Time-varying strain (explicit stepper).  The reference applies a static strain once,
 * before the run (src/init.cpp:235-254,320-333).  Here the listed elements follow
 *   e(t) = e0 + (e1 - e0) (t - t0) / (t1 - t0), clamped to [t0, t1],
 * and before each step of nrt_run / nrt_batch_advance (t = i dT) the static formulas are
 * re-evaluated for them at e(t): the element length and diameter, r_a, c_m, r_m (with the
 * 45-layer myelin when `myelin`), the damage shifts of E_Na, E_K and the left shifts, the
 * channel conductances and E_L.  The gates are state and keep their values.  A constant
 * ramp (e0 == e1) gives what a static strain of e0 gives.  Steps taken through
 * nrt_update / nrt_calculate see the parameters as they were last set.  No reference
 * counterpart (a time ramp is an extension). */
typedef struct nrt_strain_config {
  int32_t num_elem;              /* strained elements; 0 stops the ramp */
  const int32_t *instance;       /* batch: instance of each element; NULL -> 0 */
  const int32_t *element;        /* element index, local to its instance */
  const int32_t *kind;           /* 1 HH / 0 cable, as in the tree */
  const double *dspec;           /* [12][num_elem]: the elements' unstrained description in
                                    nrt_derive's dspec rows (the epsilon row is ignored) */
  int32_t myelin;                /* the tree's myelin flag (cables) */
  double e_max;                  /* the damage threshold E_MAX */
  double eps0, eps1;             /* strain at t0 and from t1 on */
  double t0, t1;                 /* ramp window, s (t1 > t0) */
  int32_t reserved[4];
} nrt_strain_config;

int nrt_set_strain(nrt_solver *s, const nrt_strain_config *cfg);
int nrt_batch_set_strain(nrt_batch *b, const nrt_strain_config *cfg);

/* ----------------------------------------------------------------------------------
 * State export / import, for checkpoints and for moving a tree between handles (serving
 * preemption).  The reference exports V only (Solver::snapshot, inc/solver.h:21) and keeps
 * its gates inside the Hodgkin_Huxley objects; no reference counterpart.
 *
 * The state of a tree is:
 *   V        the latest potential (num_elem), as nrt_snapshot returns it;
 *   V_other  the other potential buffer (num_elem): in implicit mode V^{n-1}, which the
 *            next step's initial guess 2 V^n - V^{n-1} uses (the reference's prevT/currT
 *            pair, src/neurite.cpp:165-170); in explicit mode scratch;
 *   m, h, n  the gates of its HH elements (num_hh each, HH order).
 * Any pointer may be NULL (that part is neither read nor written).  Restoring a state taken
 * from a handle with the same tree and options continues the run exactly as the original
 * would have (same arithmetic; mixed-precision gates are FP32 and round-trip exactly).  The
 * loop index is the caller's: pass it to nrt_run or nrt_batch_set_runs.  In explicit mode a
 * V whose terminals do not copy their source elements makes the next step take the
 * reference's general form (as a first step from such a state does). */
int nrt_get_state(nrt_solver *s, double *V, double *V_other, double *m, double *h, double *n);
int nrt_set_state(nrt_solver *s, const double *V, const double *V_other, const double *m,
                  const double *h, const double *n);
int nrt_batch_get_state(nrt_batch *b, int32_t instance, double *V, double *V_other, double *m,
                        double *h, double *n);
int nrt_batch_set_state(nrt_batch *b, int32_t instance, const double *V, const double *V_other,
                        const double *m, const double *h, const double *n);

/* ----------------------------------------------------------------------------------
 * Recording at measurement points, on the device.
 *
 * The reference's driver copies the whole potential to the host every interval + 1 loop
 * iterations and prints one element of it (src/neurite.cpp:238-249: a snapshot when
 * `++GL_cont > interval`, then `fprintf(study, "%.20f %.20f\n", time_run,
 * potential[1][dist_mes_points])`); src/init.cpp:339-358 picks that element.  Here probes
 * are read on the device after every step of nrt_run / nrt_batch_advance, so a time loop
 * needs no copy of V:
 *   - samples follow the same counter: loop index i is sampled when i - origin + 1 is a
 *     positive multiple of interval + 1 (origin 1 gives the reference's loop);
 *   - spikes are upward crossings of `threshold` between consecutive steps (value before
 *     < threshold <= value after), timed by linear interpolation between (i-1) dT and i dT.
 *     The value at configuration time counts as the value before loop index `origin`.
 * Steps taken through nrt_update / nrt_calculate are not recorded: that loop snapshots on
 * the host, as the reference's does.  A probe on a terminal reads what the reference's
 * snapshot shows there (the copy of its source element, explicit mode). */
typedef struct nrt_record_config {
  int32_t num_probes;            /* 0 stops recording */
  const int32_t *instance;       /* batch: instance of each probe; NULL -> instance 0 */
  const int32_t *element;        /* element of each probe, local to its instance */
  int64_t origin;                /* loop index at which the counter starts (reference: 1) */
  int64_t interval;              /* the reference's `interval` (>= 0) */
  int64_t capacity;              /* samples kept per probe; later ones are counted only */
  double threshold;              /* spike threshold, V */
  int32_t max_spikes;            /* spike times kept per probe; later ones counted only */
  int32_t reserved[3];
} nrt_record_config;

/* The reference's measurement point for a distance (src/init.cpp:339-358): the first
 * element k at which dx[0] + ... + dx[k] >= dist_mes; n/2 when there is none or it is
 * element 0.  dx is the per-element length after the strain scaling (nrt_problem.dx).
 * Host only. */
int nrt_measurement_point(int32_t n, const double *dx, double dist_mes, int32_t *point);

/* Starts recording (replacing an earlier configuration and its data).  Allocates the
 * recording's device buffers outside any time loop. */
int nrt_record(nrt_solver *s, const nrt_record_config *cfg);
int nrt_batch_record(nrt_batch *b, const nrt_record_config *cfg);

/* Copies the recording to host memory (synchronises), probes in configuration order;
 * any pointer may be NULL.  For probe p:
 *   num_samples[p]                     samples taken (may exceed capacity);
 *   times[p*capacity + k], values[...] sample k (k < min(num_samples[p], capacity)), the
 *                                      time as the reference prints it: i * dT;
 *   num_spikes[p]                      crossings found (may exceed max_spikes);
 *   spike_times[p*max_spikes + k]      crossing k, s. */
int nrt_record_read(nrt_solver *s, int64_t *num_samples, double *times, double *values,
                    int32_t *num_spikes, double *spike_times);
int nrt_batch_record_read(nrt_batch *b, int64_t *num_samples, double *times, double *values,
                          int32_t *num_spikes, double *spike_times);

/* ----------------------------------------------------------------------------------
 * Serving: a request loop (worker thread) that admits simulation requests by device
 * memory budget, packs the requests admitted together into one batch, keeps every
 * batch's state resident, advances all resident batches each tick on their own streams
 * (work of requests that arrived at different times overlaps on the device), and hands
 * results back as each request finishes.  No reference counterpart.
 *
 * A request is one tree (copied at submit) with its loop range and stimulus window;
 * `implicit` selects the backward-Euler engine.  The server's two option sets (explicit,
 * implicit) fix precision and solver settings for all requests of that kind.  Implicit
 * requests of 20,000 elements or more each get a batch of their own on the cooperative
 * whole-GPU launch (their steps take a fraction of the time one CTA would need); smaller
 * ones share block-per-instance batches. */
typedef struct nrt_server nrt_server;

typedef struct nrt_server_config {
  int64_t budget_bytes;          /* device memory the resident batches may use */
  int32_t chunk_steps;           /* steps per tick for every resident batch (default 64) */
  int32_t max_batch;             /* most requests packed into one batch (default 4096) */
  int32_t max_wait_us;           /* admission waits this long to gather a batch (default 200) */
  int32_t reserved[5];
} nrt_server_config;

typedef struct nrt_server_stats {
  int64_t submitted, completed, rejected;
  int64_t batches_created;
  int64_t compartment_steps;     /* sum over completed requests of num_elem * steps */
  double p50_ms, p99_ms, max_ms; /* submit -> result-ready latency of completed requests */
  double busy_seconds;           /* wall time with at least one resident batch */
  int64_t peak_bytes;            /* largest device memory held at once */
} nrt_server_stats;

int nrt_server_create(const nrt_server_config *cfg, const nrt_options *explicit_opt,
                      const nrt_options *implicit_opt, nrt_server **out);
/* Copies the request; returns its id.  NRT_EBUDGET if it can never fit the budget. */
int nrt_server_submit(nrt_server *s, const nrt_problem *p, int implicit,
                      const nrt_instance_run *run, int64_t *request_id);
/* As nrt_server_submit, with probes recorded on the device while the request runs
 * (nrt_record_config: elements of this tree; `instance` is ignored).  Requests are batched
 * only with requests of the same recording settings (origin, interval, capacity, threshold,
 * max_spikes). */
int nrt_server_submit_recorded(nrt_server *s, const nrt_problem *p, int implicit,
                               const nrt_instance_run *run, const nrt_record_config *rec,
                               int64_t *request_id);
/* The recording of a finished request, laid out as nrt_record_read's.  Call it before
 * nrt_server_result, which releases the request.  NRT_ENOTREADY while it runs;
 * NRT_ESTATE for a request submitted without probes. */
int nrt_server_recording(nrt_server *s, int64_t request_id, int64_t *num_samples,
                         double *times, double *values, int32_t *num_spikes,
                         double *spike_times);
/* NRT_ENOTREADY until the request finished; then copies its final potential
 * (num_elem doubles) and releases it.  Returns the request's solver status. */
int nrt_server_result(nrt_server *s, int64_t request_id, double *potential);
/* Blocks until every submitted request has finished (or failed). */
int nrt_server_drain(nrt_server *s);
int nrt_server_get_stats(nrt_server *s, nrt_server_stats *st);
int nrt_server_destroy(nrt_server *s);

/* ----------------------------------------------------------------------------------
 * Allocation-free solve.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc -- a host application that owns the device memory pool and
 * forbids other allocators, a loop that must not allocate once it runs, or a plugin that
 * is handed pre-allocated device buffers only.
 *
 * Solves A x = b for one tree's backward-Euler system in the reference's CSR layout
 * (row_ptr[n+1], col, val -- what nrt_export_system returns, copied to device memory by
 * the caller).  Method: FP64 right-preconditioned GMRES(restart) with an exact
 * tridiagonal solve of fixed 64-row blocks as the preconditioner.  Stops on
 * ||b - A x||_2 <= tol (NRT_TOL_ABS) or <= tol * ||b||_2 (NRT_TOL_REL, with ||b|| taken over
 * the rows that have off-diagonal entries: decoupled rows such as the reference's identity
 * rows are solved exactly and would otherwise dominate it), or after max_iter iterations
 * (0 -> n; then NRT_ENOCONV, x still holds the last iterate).
 * All array pointers are DEVICE memory; x holds the initial guess on entry and the
 * solution on return.  The call is asynchronous only up to the final read of the
 * iteration count: it returns after the work on `stream` (a cudaStream_t; NULL = legacy
 * default stream) has finished.
 *
 * Memory: nothing is allocated by this function or by anything it calls.  Every
 * temporary lives in one static device array of NRT_STATIC_SCRATCH_BYTES.  CUDA reserves
 * that array on a device when it loads this code onto the device, which under CUDA's
 * default lazy module loading happens at the first call on that device (with
 * CUDA_MODULE_LOADING=EAGER, when the process first uses CUDA).  A host that will later
 * claim the device's whole memory pool must therefore make one call per device before it
 * does; from then on the device holds the array until the process exits, and later calls
 * leave the device's free memory unchanged.  The array must hold
 * n * (2*restart + 6) + 2*1024*(NRT_STATIC_MAX_RESTART + 1) + 4 doubles (about 109,000 rows
 * at restart 16, 189,000 at restart 8); larger systems are refused with NRT_EBUDGET.
 * The first call on a device also looks up the array's device address (a one-time set-up
 * with that device current).  No call can be captured into a CUDA graph: each one reads
 * the iteration count back to the host and synchronises `stream` before it returns.
 * A system, right-hand side or initial guess holding NaN or Inf ends the solve with
 * NRT_EINVAL (x keeps its last finite iterate).  In relative mode a right-hand side that is
 * zero on every coupled row is measured over all rows, and one that is zero everywhere
 * against the first residual.
 * Every call shares the one array and leaves its contents behind; each region is written
 * before it is read within a call, so nothing needs clearing, but calls that overlap on the
 * GPU (other streams or host threads without ordering) race on it. */
#define NRT_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)
#define NRT_STATIC_MAX_RESTART 16
int nrt_solve_csr_static(int32_t n, const int32_t *row_ptr, const int32_t *col,
                         const double *val, const double *b, double *x, int32_t restart,
                         double tol, int32_t tol_mode, int32_t max_iter, void *stream,
                         int32_t *iters_out, double *residual_out);

#ifdef __cplusplus
}
#endif
#endif /* NEURITE_GB300_H */
