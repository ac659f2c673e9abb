// Recording at probes on the device (nrt_record / nrt_record_read and the batch forms).
//
// The reference's driver copies all of V to the host every interval + 1 steps and prints
// one element (src/neurite.cpp:238-249).  Here each probe is read on the device after
// every step: the explicit time loop gets one small launch per step (a node of the same
// captured graph), the persistent implicit kernel reads its probes itself between steps
// (record.cuh).  Nothing crosses to the host until nrt_record_read.
#include <algorithm>
#include <numeric>

#include "nrt_solver.h"
#include "pdl.cuh"
#include "record.cuh"

namespace nrt {

namespace {

__global__ void record_step(RecView r, const InstDev *__restrict__ inst, int k,
                            const double *__restrict__ V) {
  chain_acquire();  // the previous launch of the time loop has finished
  chain_release();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= r.nprobe) return;
  const InstDev in = inst[r.inst[p]];
  const int64_t i = in.base + k;
  if (i >= in.iend) return;  // this instance's run is over
  record_probe(r, p, i, V[r.src[p]], in.dT);
}

// The value each probe starts from (read at its own element: what a snapshot shows now).
__global__ void record_init(RecView r, const int64_t *__restrict__ raw,
                            const double *__restrict__ V) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= r.nprobe) return;
  r.prev_v[p] = V[raw[p]];
  r.prev_i[p] = r.origin - 1;
  r.nsamp[p] = 0;
  r.nspike[p] = 0;
}

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

struct RecState {
  void *mem = nullptr;
  RecView view{};
  RecView *d_view = nullptr;
  int64_t *d_raw = nullptr;    // each probe's own element (initial values)
  std::vector<int32_t> order;  // sorted slot -> configuration index
  std::vector<int32_t> inst;   // instance per sorted slot
  ~RecState() {
    if (mem) cudaFree(mem);
  }
};

int launch_record_step(const RecView &r, const InstDev *inst, int k, const double *V,
                       cudaStream_t st) {
  if (r.nprobe <= 0) return NRT_OK;
  NRT_CUDA(launch_chained(record_step, (r.nprobe + 127) / 128, 128, 0, st, r, inst, k, V));
  return NRT_OK;
}

const RecView *Engine::record_view() const { return rec ? rec->d_view : nullptr; }
const RecView &Engine::rec_view_host() const { return rec->view; }

void Engine::record_release() {
  delete rec;
  rec = nullptr;
}

int Engine::record_config(const nrt_record_config *c) {
  if (!c) {
    set_error("null record configuration");
    return NRT_EINVAL;
  }
  const int32_t P = c->num_probes;
  if (P < 0 || c->interval < 0 || c->capacity < 0 || c->max_spikes < 0 ||
      (P > 0 && !c->element)) {
    set_error("bad record configuration (negative size or null element array)");
    return NRT_EINVAL;
  }
  if ((double)P * (double)(c->capacity + c->max_spikes) * 8.0 > 1e12) {  // sizes cannot wrap
    set_error("recording buffers would exceed 1 TB");
    return NRT_EINVAL;
  }
  std::vector<int32_t> pin(P), pel(P);
  for (int32_t p = 0; p < P; p++) {
    const int32_t q = c->instance ? c->instance[p] : 0;
    if (q < 0 || q >= host.ninst || c->element[p] < 0 || c->element[p] >= host.num_elem[q]) {
      set_error("probe " + std::to_string(p) + " names no element of its instance");
      return NRT_EINVAL;
    }
    pin[p] = q;
    pel[p] = c->element[p];
  }
  // the graphs of the explicit time loop carry (or lack) the record launches: recapture
  NRT_CUDA(cudaStreamSynchronize(stream));
  for (int q = 0; q < 2; q++)
    if (graph_exec[q]) {
      cudaGraphExecDestroy(graph_exec[q]);
      graph_exec[q] = nullptr;
    }
  record_release();
  if (P == 0) return NRT_OK;

  RecState *R = new (std::nothrow) RecState();
  if (!R) {
    set_error("host allocation");
    return NRT_ENOMEM;
  }
  R->order.resize(P);
  std::iota(R->order.begin(), R->order.end(), 0);
  std::stable_sort(R->order.begin(), R->order.end(),
                   [&](int32_t a, int32_t b) { return pin[a] < pin[b]; });
  std::vector<int64_t> src(P), raw(P);
  std::vector<int32_t> sinst(P), p0(host.ninst + 1, 0);
  const bool expl = opt.mode == NRT_EXPLICIT;
  for (int32_t s = 0; s < P; s++) {
    const int32_t p = R->order[s];
    const int64_t j = host.off[pin[p]] + pel[p];
    raw[s] = j;
    src[s] = j;
    // explicit: terminals are not written during a run; their value is their source's
    const Topo &t = host.topo[j];
    if (expl && (t.flags & F_TERM)) src[s] = (t.flags & F_ROOT) ? j + 1 : (int64_t)t.mother;
    sinst[s] = pin[p];
    p0[pin[p] + 1]++;
  }
  for (int32_t q = 0; q < host.ninst; q++) p0[q + 1] += p0[q];
  R->inst = sinst;

  const int64_t cap = c->capacity, ms = c->max_spikes;
  const size_t bytes = al(sizeof(RecView)) + 2 * al(8 * (size_t)P) + al(4 * (size_t)P) +
                       al(4 * (size_t)(host.ninst + 1)) + al(8 * (size_t)P) +
                       al(4 * (size_t)P) + 2 * al(8 * (size_t)P) +
                       al(8 * (size_t)P * (size_t)std::max<int64_t>(cap, 1)) +
                       al(8 * (size_t)P * (size_t)std::max<int64_t>(ms, 1));
  if (cudaMalloc(&R->mem, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete R;
    set_error("device allocation for the recording (" + std::to_string(bytes) + " bytes)");
    return NRT_ENOMEM;
  }
  char *m = (char *)R->mem;
  auto take = [&](size_t b) {
    char *r = m;
    m += al(b);
    return (void *)r;
  };
  RecView &v = R->view;
  R->d_view = (RecView *)take(sizeof(RecView));
  v.nprobe = P;
  v.max_spikes = (int32_t)ms;
  v.origin = c->origin;
  v.interval = c->interval;
  v.cap = cap;
  v.thresh = c->threshold;
  int64_t *d_src = (int64_t *)take(8 * (size_t)P);
  R->d_raw = (int64_t *)take(8 * (size_t)P);
  int32_t *d_inst = (int32_t *)take(4 * (size_t)P);
  int32_t *d_p0 = (int32_t *)take(4 * (size_t)(host.ninst + 1));
  v.src = d_src;
  v.inst = d_inst;
  v.p0 = d_p0;
  v.nsamp = (int64_t *)take(8 * (size_t)P);
  v.nspike = (int32_t *)take(4 * (size_t)P);
  v.prev_i = (int64_t *)take(8 * (size_t)P);
  v.prev_v = (double *)take(8 * (size_t)P);
  v.val = (double *)take(8 * (size_t)P * (size_t)std::max<int64_t>(cap, 1));
  v.spk = (double *)take(8 * (size_t)P * (size_t)std::max<int64_t>(ms, 1));
  // installed only once complete: a failed call leaves no recording behind
  int rc = upload_and_init(R, src, raw, sinst, p0);
  if (rc) {
    cudaStreamSynchronize(stream);
    delete R;
    return rc;
  }
  rec = R;
  return NRT_OK;
}

int Engine::upload_and_init(RecState *R, const std::vector<int64_t> &src,
                            const std::vector<int64_t> &raw, const std::vector<int32_t> &sinst,
                            const std::vector<int32_t> &p0) {
  const RecView &v = R->view;
  const int32_t P = v.nprobe;
  int64_t *d_raw = R->d_raw;
  NRT_CUDA(cudaMemcpyAsync((void *)v.src, src.data(), 8 * (size_t)P, cudaMemcpyHostToDevice,
                           stream));
  NRT_CUDA(cudaMemcpyAsync(d_raw, raw.data(), 8 * (size_t)P, cudaMemcpyHostToDevice, stream));
  NRT_CUDA(cudaMemcpyAsync((void *)v.inst, sinst.data(), 4 * (size_t)P, cudaMemcpyHostToDevice,
                           stream));
  NRT_CUDA(cudaMemcpyAsync((void *)v.p0, p0.data(), 4 * p0.size(), cudaMemcpyHostToDevice,
                           stream));
  NRT_CUDA(cudaMemcpyAsync(R->d_view, &v, sizeof(RecView), cudaMemcpyHostToDevice, stream));
  int rc = fixup();  // explicit: terminals hold their current value before the first read
  if (rc) return rc;
  record_init<<<(P + 127) / 128, 128, 0, stream>>>(v, d_raw, V[cur]);
  count_launch_on(stream);
  NRT_CUDA(cudaGetLastError());
  NRT_CUDA(cudaStreamSynchronize(stream));  // the host vectors go out of scope after this
  return NRT_OK;
}

int Engine::record_read(int64_t *num_samples, double *times, double *values, int32_t *num_spikes,
                        double *spike_times) {
  NRT_CUDA(cudaStreamSynchronize(stream));
  if (!rec) {
    set_error("no recording configured");
    return NRT_ESTATE;
  }
  const RecView &v = rec->view;
  const int32_t P = v.nprobe;
  const int64_t cap = v.cap, ms = v.max_spikes;
  std::vector<int64_t> ns(P);
  std::vector<int32_t> nk(P);
  std::vector<double> val((size_t)P * cap), spk((size_t)P * ms);
  NRT_CUDA(cudaMemcpyAsync(ns.data(), v.nsamp, 8 * (size_t)P, cudaMemcpyDeviceToHost, stream));
  NRT_CUDA(cudaMemcpyAsync(nk.data(), v.nspike, 4 * (size_t)P, cudaMemcpyDeviceToHost, stream));
  if (cap)
    NRT_CUDA(cudaMemcpyAsync(val.data(), v.val, 8 * val.size(), cudaMemcpyDeviceToHost, stream));
  if (ms)
    NRT_CUDA(cudaMemcpyAsync(spk.data(), v.spk, 8 * spk.size(), cudaMemcpyDeviceToHost, stream));
  NRT_CUDA(cudaStreamSynchronize(stream));
  for (int32_t s = 0; s < P; s++) {
    const int32_t p = rec->order[s];
    const double dT = host.inst[rec->inst[s]].dT;
    if (num_samples) num_samples[p] = ns[s];
    const int64_t kept = std::min<int64_t>(ns[s], cap);
    for (int64_t k = 0; k < kept; k++) {
      const int64_t i = v.origin + (k + 1) * (v.interval + 1) - 1;
      if (times) times[(size_t)p * cap + k] = (double)i * dT;  // time_run = i*dT
      if (values) values[(size_t)p * cap + k] = val[(size_t)s * cap + k];
    }
    if (num_spikes) num_spikes[p] = nk[s];
    const int64_t kept_sp = std::min<int64_t>(nk[s], ms);
    if (spike_times)
      for (int64_t k = 0; k < kept_sp; k++)
        spike_times[(size_t)p * ms + k] = spk[(size_t)s * ms + k];
  }
  return NRT_OK;
}

}  // namespace nrt
