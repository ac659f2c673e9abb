// The engine behind a solver handle or a batch: one device arena holding the packed
// trees, the two potential buffers, and (implicit mode) the Krylov workspace.
#pragma once
#include "nrt_internal.h"

namespace nrt {

constexpr int kChunk = 64;        // steps per captured graph (even: buffer parity returns)
constexpr int kMaxRestart = 32;   // GMRES restart limit (dot accumulators live in registers)

struct Arena {
  void *base = nullptr;
  size_t cap = 0, used = 0;
  int reserve(size_t bytes);
  void *take(size_t bytes);
  void release();
};

struct ImplicitState;  // implicit.cu
struct RecState;       // record.cu
struct StrainState;    // strain.cu

struct Engine {
  nrt_options opt{};
  int device = -1;
  cudaStream_t stream = nullptr;
  HostPack host;
  Arena arena;
  PackView pv{};
  double *V[2] = {nullptr, nullptr};
  float *Vf[2] = {nullptr, nullptr};  // FP32 shadow of V (mixed explicit mode only)
  int cur = 0;
  int64_t *terms = nullptr;
  int64_t steps_done = 0;
  bool terminals_dirty = false;
  bool general_next = false;  // explicit: the next step runs in the general form
  cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};  // one per starting buffer parity
  int64_t graph_nodes[2] = {0, 0};                       // kernels per replay of each
  std::vector<hvec<float>> hostf;  // staging for FP32 uploads
  ImplicitState *im = nullptr;
  RecState *rec = nullptr;                // recording at probes, or null
  StrainState *strain = nullptr;          // time-varying strain of some elements, or null
  GridBar *gbar = nullptr;                // the explicit chunk kernel's barrier words
  std::vector<void *> extra_mem;          // device tables that replaced the arena's (freed last)

  int init(const nrt_problem *probs, int32_t count, const nrt_options *o);
  int step(int k, int force);
  int advance(int64_t steps);
  bool chunk_kernel() const;  // explicit time loops run a chunk of steps per launch
  int fixup();
  bool needs_general() const { return general_next || (!host.invariant && steps_done == 0); }
  int get_state(int32_t q, double *Vc, double *Vo, double *m, double *h, double *n);
  int set_state(int32_t q, const double *Vc, const double *Vo, const double *m, const double *h,
                const double *n);
  int get_stats(nrt_stats *st);
  // implicit.cu
  int implicit_plan(size_t &bytes);
  int implicit_init();
  int implicit_step(int k, int force);
  void implicit_release();
  // record.cu
  int record_config(const nrt_record_config *c);
  int record_read(int64_t *num_samples, double *times, double *values, int32_t *num_spikes,
                  double *spike_times);
  const RecView *record_view() const;  // device copy for the implicit kernel, or null
  const RecView &rec_view_host() const;  // host copy (device pointers) for kernel arguments
  int upload_and_init(RecState *R, const std::vector<int64_t> &src,
                      const std::vector<int64_t> &raw, const std::vector<int32_t> &sinst,
                      const std::vector<int32_t> &p0);
  void record_release();
  // strain.cu
  int strain_config(const nrt_strain_config *c);
  void strain_release();
  ~Engine();
};

// strain.cu: the strained elements' coefficients for explicit step k, derived and written
// in one launch; or, in a graph chunk, derived ahead for steps 0 .. nk-1 in one launch
// (when strain_tabled) and written by one launch per step
int launch_strain_update(const Engine &e, int k, cudaStream_t st);
bool strain_tabled(const Engine &e);
int launch_strain_derive(const Engine &e, int nk, cudaStream_t st);
int launch_strain_apply(const Engine &e, int k, cudaStream_t st);
const StrainView *strain_view(const Engine &e);  // null without strain

// implicit.cu
int implicit_advance(Engine &e, int64_t steps);
int export_system(Engine &e, int input_active, int32_t *row_ptr, int32_t *col, double *val,
                  double *rhs, int32_t *nnz_out);
int64_t nonconverged_total(Engine &e);
int implicit_check(Engine &e);
int instance_stats(Engine &e, int64_t *iters, int32_t *last_iters, int32_t *nonconv,
                   double *last_res);
int pass_counts(Engine &e, int64_t *residuals, int64_t *applies, int64_t *xupdates,
                int64_t *basis, int64_t *rich);

}  // namespace nrt
