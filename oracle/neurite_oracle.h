/* CPU oracle for the Neurite solver hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU algorithms, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.  The
 * product (the CUDA library under 168861_gb300/) never links or calls this.
 *
 * Pinning: the explicit path and the parameter pipeline are checked bit-for-bit against
 * the reference's own src/solverEx-cpu.cpp / src/init.cpp compiled from source
 * (oracle/_ref, golden fixtures under tests/golden/).  The implicit matrix assembly and
 * the FGMRES driver are checked against the reference's src/solverIm-cpu.cpp compiled
 * with an RCI shim (oracle/mkl_shim.cpp) that restates Intel MKL's published RCI FGMRES.
 *
 * Array conventions (all column blocks are contiguous, length n unless stated):
 *   ispec [5][n] : kind (1 = Hodgkin_Huxley, 0 = Cable), mother, DR, DL, branching
 *   dspec [12][n]: dX, diameter, epsilon, input_current, ro_a, ro_m, per_m, thickness,
 *                  rest_pot, sigma_Na, sigma_K, sigma_L                   (SI units)
 *   eparam [6][n]: c_m, r_a, dX, W, K, critical_dT   (after strain and derivation)
 *   hparam [12][num_hh]: m, h, n, g_Na, g_K, G_L, E_Na, E_K, E_L, LS_Na, LS_K, rest_pot
 *   hh_elem [num_hh]: element index of each HH element, ascending
 */
#ifndef NEURITE_ORACLE_H
#define NEURITE_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { NRO_OK = 0, NRO_EINVAL = 1, NRO_ENOCONV = 2, NRO_ENOMEM = 3 };

/* Parameter pipeline: src/init.cpp:320-333 (dX strain), :235-254 (electrical_properties),
 * :260-267 (setting_rest_pot), :273-298 (hhIconds), :180-198 (cable_init_constants),
 * :138-146 (critical_time_step_class), :165-174 (critical_time_step_selection).
 * Returns the number of HH elements in *num_hh_out. */
int nro_derive(int n, const int32_t *ispec, const double *dspec, int myelin, double e_max,
               double *eparam, int32_t *hh_elem, double *hparam, int *num_hh_out,
               double *dT_crit_out);

/* Explicit solver, src/solverEx-cpu.cpp:90-174, driven with the loop semantics of
 * src/neurite.cpp:224-236: for i in [i_begin, i_end): t = i*dT;
 * update(init_time <= t <= end_input); calculate().
 * V [n] holds the latest potential on entry and exit; hparam gates are updated in place.
 * If record_every > 0, every step i with i % record_every == 0 appends
 * (i, V[probes[0..nprobe)]) to trace (rows of nprobe+1 doubles); *nrec_out counts rows. */
int nro_explicit_run(int n, const int32_t *ispec, const double *eparam, const double *input_on,
                     int num_term, const int32_t *terminals, int num_hh, const int32_t *hh_elem,
                     double *hparam, double dT, int i_begin, int i_end, double init_time,
                     double end_input, double *V, int record_every, int nprobe,
                     const int32_t *probes, double *trace, int *nrec_out);

/* Implicit (backward Euler) system of src/solverIm-cpu.cpp:29-183 (createMatrix) for the
 * current W, K.  Writes CSR (row_ptr [n+1], col [nnz], val [nnz]) and the right-hand side
 * into rhs (rows the reference leaves untouched keep rhs's incoming value).
 * Capacity of col/val must be >= 4n+2.  Returns nnz in *nnz_out. */
int nro_implicit_matrix(int n, const int32_t *ispec, const double *eparam, const double *W,
                        const double *K, const double *input, double dT, const double *Vprev,
                        int32_t *row_ptr, int32_t *col, double *val, double *rhs, int *nnz_out);

/* Exact solve of a CSR system whose graph is a forest with every row having at most one
 * off-diagonal column below its own index (the tree ordering of the reference's
 * numbering).  Leaf-to-root elimination, root-to-leaf substitution (Hines).  x may alias b. */
int nro_tree_solve(int n, const int32_t *row_ptr, const int32_t *col, const double *val,
                   const double *b, double *x);

/* Restarted GMRES(m) with x0 = 0 and the absolute stopping test ||r||_2 <= tol of
 * src/solverIm-cpu.cpp:192-272 (restart min(150, n), at most max_it iterations).
 * Returns NRO_ENOCONV when max_it is reached; *iters_out gets the iteration count. */
int nro_gmres(int n, const int32_t *row_ptr, const int32_t *col, const double *val,
              const double *b, double *x, int restart, double tol, int max_it, int *iters_out);

/* Implicit run: SolverImCPU::update + calculate (src/solverIm-cpu.cpp:307-370) per step.
 * linsolve = 0: exact tree solve; 1: GMRES(min(150,n)) with ||r|| <= 1e-14, x0 = 0;
 * 2: as 1, but a step that reaches the n-iteration limit keeps its last iterate and the
 * run goes on (the reference program exits there instead, src/solverIm-cpu.cpp:247-250).
 * V [n] is the latest potential (the reference's prevT), Vother [n] its second buffer
 * (currT), which supplies the right-hand side of the rows the reference never writes. */
int nro_implicit_run(int n, const int32_t *ispec, const double *eparam, const double *input_on,
                     int num_hh, const int32_t *hh_elem, double *hparam, double dT, int i_begin,
                     int i_end, double init_time, double end_input, double *V, double *Vother,
                     int linsolve, int record_every, int nprobe, const int32_t *probes,
                     double *trace, int *nrec_out, long long *krylov_iters_out, int scheme);

#ifdef __cplusplus
}
#endif
#endif
