// Serving loop (nrt_server_*): continuous batching of simulation requests.
//
// A worker thread owns every device handle.  Each tick it
//   1. admits pending requests (FIFO, grouped by kind) while their estimated device
//      footprint fits what the budget leaves free, and packs the admitted requests of
//      one kind into a new batch (one device-resident pack, one launch per step);
//   2. advances every resident batch by `chunk_steps` on the batch's own stream, all
//      launches enqueued before any wait, so batches admitted at different times run
//      concurrently on the device;
//   3. collects the requests whose loop range is exhausted (their potential is copied
//      out at once) and frees a batch when all of its requests are done.
// Latency is measured from submit to result-ready on the host clock.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "guard.h"
#include "neurite_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

struct OwnedProblem {
  std::vector<int32_t> mother, dr, dl, branching, terminals, hh_elem;
  std::vector<double> dx, c_m, r_a, W, K, input, m, h, n, g_Na, g_K, G_L, E_Na, E_K, E_L,
      ls_Na, ls_K, rest, V0, V1;
  nrt_problem p;

  template <class T>
  static void take(std::vector<T> &dst, const T *src, size_t n) {
    if (src) dst.assign(src, src + n); else dst.clear();
  }
  template <class T>
  static const T *ptr(const std::vector<T> &v) {
    return v.empty() ? nullptr : v.data();
  }

  void copy(const nrt_problem &s) {
    const size_t N = (size_t)s.num_elem, H = (size_t)s.num_hh, T = (size_t)s.num_term;
    take(mother, s.mother, N); take(dr, s.dr, N); take(dl, s.dl, N);
    take(branching, s.branching, N); take(terminals, s.terminals, T);
    take(dx, s.dx, N); take(c_m, s.c_m, N); take(r_a, s.r_a, N); take(W, s.W, N);
    take(K, s.K, N); take(input, s.input, N); take(V0, s.V0, N); take(V1, s.V1, N);
    take(hh_elem, s.hh_elem, H); take(m, s.m, H); take(h, s.h, H); take(n, s.n, H);
    take(g_Na, s.g_Na, H); take(g_K, s.g_K, H); take(G_L, s.G_L, H); take(E_Na, s.E_Na, H);
    take(E_K, s.E_K, H); take(E_L, s.E_L, H); take(ls_Na, s.ls_Na, H); take(ls_K, s.ls_K, H);
    take(rest, s.rest, H);
    p = s;
    p.mother = ptr(mother); p.dr = ptr(dr); p.dl = ptr(dl); p.branching = ptr(branching);
    p.terminals = ptr(terminals); p.dx = ptr(dx); p.c_m = ptr(c_m); p.r_a = ptr(r_a);
    p.W = ptr(W); p.K = ptr(K); p.input = ptr(input); p.V0 = ptr(V0); p.V1 = ptr(V1);
    p.hh_elem = ptr(hh_elem); p.m = ptr(m); p.h = ptr(h); p.n = ptr(n);
    p.g_Na = ptr(g_Na); p.g_K = ptr(g_K); p.G_L = ptr(G_L); p.E_Na = ptr(E_Na);
    p.E_K = ptr(E_K); p.E_L = ptr(E_L); p.ls_Na = ptr(ls_Na); p.ls_K = ptr(ls_K);
    p.rest = ptr(rest);
  }
};

// Recording settings of a request (nrt_server_submit_recorded); requests are batched only
// with requests of equal settings, since a batch records under one configuration.
struct RecSpec {
  bool on = false;
  int64_t origin = 1, interval = 0, capacity = 0;
  double threshold = 0;
  int32_t max_spikes = 0;
  bool operator<(const RecSpec &o) const {
    if (on != o.on) return on < o.on;
    if (origin != o.origin) return origin < o.origin;
    if (interval != o.interval) return interval < o.interval;
    if (capacity != o.capacity) return capacity < o.capacity;
    if (threshold != o.threshold) return threshold < o.threshold;
    return max_spikes < o.max_spikes;
  }
};

struct Request {
  int64_t id = 0;
  bool implicit = false;
  RecSpec rec;
  std::vector<int32_t> probes;          // elements of this tree
  std::vector<int64_t> rec_ns;          // per probe: samples taken
  std::vector<int32_t> rec_nk;          // per probe: crossings found
  std::vector<double> rec_t, rec_v, rec_sp;  // [probe][capacity], [probe][max_spikes]
  OwnedProblem prob;
  nrt_instance_run run{};
  size_t bytes = 0;
  Clock::time_point t_submit, t_done;
  std::vector<double> result;
  int status = NRT_OK;
  bool done = false;
};

struct MicroBatch {
  nrt_batch *b = nullptr;
  std::vector<Request *> reqs;
  RecSpec rec;                     // the batch's recording settings (rec.on: recording)
  std::vector<int32_t> probe0;     // per request: first probe in the batch's configuration
  std::vector<char> finished;
  size_t bytes = 0;
  size_t open = 0;
  int64_t per_tick = 0;            // steps per tick, adapted to the target tick time
  int adv_rc = NRT_OK;             // first failure of nrt_batch_advance: ends every open request
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaStream_t stream = nullptr;
};

constexpr double kTickMs = 10.0;   // target device time of one tick per resident batch
constexpr int32_t kWideRows = 20000;  // implicit requests this large step on the whole GPU

// Device footprint of one tree in a batch (the arena sizes of the engine, rounded up).
size_t estimate_bytes(const nrt_problem &p, const nrt_options &o) {
  const double N = (double)p.num_elem;
  const bool mixed = o.precision == NRT_MIXED;
  const double tb = mixed ? 4 : 8;
  double per = 16 + 16 + 16 + (mixed ? (7 * 4 + 12 + 44) : (5 * 8 + 24 + 88));
  if (o.mode == NRT_IMPLICIT_BE) per += 48 + 8 + 8 + 2 * tb * (o.restart + 1) + 3 * tb + 16;
  return (size_t)(N * per * 1.15) + (1 << 20);
}

}  // namespace

struct nrt_server {
  nrt_server_config cfg{};
  nrt_options opt[2];  // [0] explicit, [1] implicit
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> pending;
  std::map<int64_t, Request *> reqs;
  std::vector<MicroBatch *> active;  // worker-owned
  std::thread worker;
  bool stop = false;
  int64_t next_id = 1;
  size_t used = 0, peak = 0;
  int64_t outstanding = 0;
  nrt_server_stats st{};
  std::vector<double> lat_ms;
  double busy = 0;

  void loop();
  MicroBatch *admit(bool implicit, std::vector<Request *> &batch, bool wide = false);
};

// `wide`: one large implicit request on the cooperative whole-GPU launch (its steps take a
// fraction of the time one CTA needs; it shares the SMs with the resident batches).
MicroBatch *nrt_server::admit(bool implicit, std::vector<Request *> &batch, bool wide) {
  std::vector<nrt_problem> probs;
  std::vector<nrt_instance_run> runs;
  for (Request *r : batch) {
    probs.push_back(r->prob.p);
    runs.push_back(r->run);
  }
  MicroBatch *mb = new MicroBatch();
  nrt_options o = opt[implicit ? 1 : 0];
  if (wide) o.schedule = 0;
  int rc = nrt_batch_create(probs.data(), (int32_t)probs.size(), &o, &mb->b);
  if (rc == NRT_OK) rc = nrt_batch_set_runs(mb->b, runs.data());
  mb->rec = batch.empty() ? RecSpec() : batch[0]->rec;
  if (rc == NRT_OK && mb->rec.on) {  // every request's probes, instance = its batch position
    std::vector<int32_t> inst, elem;
    mb->probe0.assign(batch.size() + 1, 0);
    for (size_t q = 0; q < batch.size(); q++) {
      for (int32_t e : batch[q]->probes) {
        inst.push_back((int32_t)q);
        elem.push_back(e);
      }
      mb->probe0[q + 1] = (int32_t)elem.size();
    }
    nrt_record_config rc_cfg;
    memset(&rc_cfg, 0, sizeof(rc_cfg));
    rc_cfg.num_probes = (int32_t)elem.size();
    rc_cfg.instance = inst.data();
    rc_cfg.element = elem.data();
    rc_cfg.origin = mb->rec.origin;
    rc_cfg.interval = mb->rec.interval;
    rc_cfg.capacity = mb->rec.capacity;
    rc_cfg.threshold = mb->rec.threshold;
    rc_cfg.max_spikes = mb->rec.max_spikes;
    rc = nrt_batch_record(mb->b, &rc_cfg);
  }
  std::lock_guard<std::mutex> lk(mu);
  if (rc != NRT_OK) {
    for (Request *r : batch) {
      r->status = rc;
      r->done = true;
      r->t_done = Clock::now();
      used -= r->bytes;
      outstanding--;
    }
    if (mb->b) nrt_batch_destroy(mb->b);
    delete mb;
    cv_done.notify_all();
    return nullptr;
  }
  mb->reqs = batch;
  mb->finished.assign(batch.size(), 0);
  mb->open = batch.size();
  for (Request *r : batch) mb->bytes += r->bytes;
  mb->per_tick = cfg.chunk_steps;
  void *sp = nullptr;
  nrt_batch_get_stream(mb->b, &sp);
  mb->stream = (cudaStream_t)sp;
  cudaEventCreate(&mb->ev0);
  cudaEventCreate(&mb->ev1);
  st.batches_created++;
  return mb;
}

static void release(MicroBatch *mb) {
  if (mb->ev0) cudaEventDestroy(mb->ev0);
  if (mb->ev1) cudaEventDestroy(mb->ev1);
  nrt_batch_destroy(mb->b);
  delete mb;
}

void nrt_server::loop() {
  for (;;) {
    std::vector<Request *> take[2];
    {
      std::unique_lock<std::mutex> lk(mu);
      if (active.empty()) {
        cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        if (stop && pending.empty()) break;
        if (cfg.max_wait_us > 0) {  // let a burst of arrivals gather into one batch
          lk.unlock();
          std::this_thread::sleep_for(std::chrono::microseconds(cfg.max_wait_us));
          lk.lock();
        }
      }
      // admission: FIFO within each kind, while the budget leaves room
      size_t free_bytes = (size_t)cfg.budget_bytes > used ? (size_t)cfg.budget_bytes - used : 0;
      for (auto it = pending.begin(); it != pending.end();) {
        Request *r = *it;
        std::vector<Request *> &t = take[r->implicit ? 1 : 0];
        if (r->bytes <= free_bytes && (int)t.size() < cfg.max_batch) {
          free_bytes -= r->bytes;
          used += r->bytes;
          peak = std::max(peak, used);
          t.push_back(r);
          it = pending.erase(it);
        } else {
          ++it;
        }
      }
      if (stop && pending.empty() && active.empty() && take[0].empty() && take[1].empty()) break;
    }
    {  // large implicit requests each get their own whole-GPU micro-batch
      std::vector<Request *> narrow;
      for (Request *r : take[1]) {
        if (r->prob.p.num_elem >= kWideRows) {
          std::vector<Request *> one(1, r);
          MicroBatch *mb = admit(true, one, true);
          if (mb) active.push_back(mb);
        } else {
          narrow.push_back(r);
        }
      }
      take[1].swap(narrow);
    }
    for (int k = 0; k < 2; k++) {
      std::map<RecSpec, std::vector<Request *>> groups;  // one batch per recording setting
      for (Request *r : take[k]) groups[r->rec].push_back(r);
      for (auto &g : groups) {
        MicroBatch *mb = admit(k == 1, g.second);
        if (mb) active.push_back(mb);
      }
    }
    if (active.empty()) continue;
    const auto t0 = Clock::now();
    // one tick: every resident batch advances on its own stream (all enqueued first)
    for (MicroBatch *mb : active) {
      cudaEventRecord(mb->ev0, mb->stream);
      const int arc = nrt_batch_advance(mb->b, mb->per_tick);
      if (arc != NRT_OK && mb->adv_rc == NRT_OK) mb->adv_rc = arc;
      cudaEventRecord(mb->ev1, mb->stream);
    }
    // collect finished requests
    std::vector<int64_t> rem;
    for (MicroBatch *mb : active) {
      rem.assign(mb->reqs.size(), 0);
      int rc = mb->adv_rc != NRT_OK ? mb->adv_rc : nrt_batch_remaining(mb->b, rem.data());
      float ms = 0;
      if (cudaEventElapsedTime(&ms, mb->ev0, mb->ev1) == cudaSuccess && ms > 0) {
        // steps per tick toward the target tick time (explicit steps are ~1000x cheaper)
        const double want = (double)mb->per_tick * kTickMs / ms;
        mb->per_tick = (int64_t)std::max(1.0, std::min(want, 4.0 * mb->per_tick + 1));
        mb->per_tick = std::min<int64_t>(mb->per_tick, 1 << 20);
      }
      nrt_stats bs;
      const bool bad = rc != NRT_OK;
      // the batch's recording, read once per tick in which one of its requests finished
      std::vector<int64_t> rns;
      std::vector<int32_t> rnk;
      std::vector<double> rt, rv, rsp;
      bool rec_read = false;
      int rec_rc = NRT_OK;
      for (size_t q = 0; q < mb->reqs.size(); q++) {
        if (mb->finished[q] || (!bad && rem[q] > 0)) continue;
        Request *r = mb->reqs[q];
        if (mb->rec.on && !bad && !rec_read) {
          const size_t P = (size_t)mb->probe0.back(), cap = (size_t)mb->rec.capacity,
                       ms = (size_t)mb->rec.max_spikes;
          rns.resize(P);
          rnk.resize(P);
          rt.resize(P * std::max<size_t>(cap, 1));
          rv.resize(P * std::max<size_t>(cap, 1));
          rsp.resize(P * std::max<size_t>(ms, 1));
          rec_rc = nrt_batch_record_read(mb->b, rns.data(), rt.data(), rv.data(), rnk.data(),
                                         rsp.data());
          rec_read = true;
        }
        if (mb->rec.on && rec_read && rec_rc == NRT_OK) {
          const size_t p0 = (size_t)mb->probe0[q], p1 = (size_t)mb->probe0[q + 1];
          const size_t cap = (size_t)mb->rec.capacity, ms = (size_t)mb->rec.max_spikes;
          r->rec_ns.assign(rns.begin() + p0, rns.begin() + p1);
          r->rec_nk.assign(rnk.begin() + p0, rnk.begin() + p1);
          r->rec_t.assign(rt.begin() + p0 * cap, rt.begin() + p1 * cap);
          r->rec_v.assign(rv.begin() + p0 * cap, rv.begin() + p1 * cap);
          r->rec_sp.assign(rsp.begin() + p0 * ms, rsp.begin() + p1 * ms);
        }
        r->result.resize(r->prob.p.num_elem);
        int src = bad ? rc : nrt_batch_snapshot(mb->b, (int32_t)q, r->result.data());
        if (src == NRT_OK && rec_rc != NRT_OK) src = rec_rc;
        std::lock_guard<std::mutex> lk(mu);
        r->status = src;
        r->done = true;
        r->t_done = Clock::now();
        mb->finished[q] = 1;
        mb->open--;
        outstanding--;
        st.completed++;
        st.compartment_steps += (int64_t)r->prob.p.num_elem * (r->run.i_end - r->run.i_begin);
        lat_ms.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
      }
      if (nrt_batch_get_stats(mb->b, &bs) == NRT_OK && bs.nonconverged_steps > 0) {
        // report non-convergence on the requests that finished in this batch
        std::lock_guard<std::mutex> lk(mu);
        for (size_t q = 0; q < mb->reqs.size(); q++)
          if (mb->finished[q] && mb->reqs[q]->status == NRT_OK) mb->reqs[q]->status = NRT_ENOCONV;
      }
    }
    cv_done.notify_all();
    for (size_t a = 0; a < active.size();) {
      MicroBatch *mb = active[a];
      if (mb->open == 0) {
        {
          std::lock_guard<std::mutex> lk(mu);
          used -= mb->bytes;
        }
        release(mb);
        active.erase(active.begin() + a);
      } else {
        a++;
      }
    }
    const double tick_s = std::chrono::duration<double>(Clock::now() - t0).count();
    std::lock_guard<std::mutex> lk(mu);  // nrt_server_get_stats reads it
    busy += tick_s;
  }
}

static int submit_request(nrt_server *s, const nrt_problem *p, int implicit,
                          const nrt_instance_run *run, const nrt_record_config *rec,
                          int64_t *request_id) {
  if (!s || !p || !run || !request_id) return NRT_EINVAL;
  if (p->num_elem < 4 || run->i_end < run->i_begin) return NRT_EINVAL;
  if (rec) {
    if (rec->num_probes < 0 || (rec->num_probes > 0 && !rec->element) || rec->interval < 0 ||
        rec->capacity < 0 || rec->max_spikes < 0)
      return NRT_EINVAL;
    for (int32_t q = 0; q < rec->num_probes; q++)
      if (rec->element[q] < 0 || rec->element[q] >= p->num_elem) return NRT_EINVAL;
  }
  Request *r = new (std::nothrow) Request();
  if (!r) return NRT_ENOMEM;
  try {  // host copies of the request: no exception crosses the C boundary
    r->implicit = implicit != 0;
    r->prob.copy(*p);
    r->run = *run;
    if (rec && rec->num_probes > 0) {  // complete before the worker can see the request
      r->rec.on = true;
      r->rec.origin = rec->origin;
      r->rec.interval = rec->interval;
      r->rec.capacity = rec->capacity;
      r->rec.threshold = rec->threshold;
      r->rec.max_spikes = rec->max_spikes;
      r->probes.assign(rec->element, rec->element + rec->num_probes);
    }
  } catch (const std::exception &) {
    delete r;
    return NRT_ENOMEM;
  }
  r->bytes = estimate_bytes(*p, s->opt[r->implicit ? 1 : 0]);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  s->st.submitted++;
  if (r->bytes > (size_t)s->cfg.budget_bytes) {
    s->st.rejected++;
    delete r;
    return NRT_EBUDGET;
  }
  r->id = s->next_id++;
  *request_id = r->id;
  s->reqs[r->id] = r;
  s->pending.push_back(r);
  s->outstanding++;
  s->cv_work.notify_one();
  return NRT_OK;
}

extern "C" {

int nrt_server_create(const nrt_server_config *cfg, const nrt_options *explicit_opt,
                      const nrt_options *implicit_opt, nrt_server **out) {
  return nrt::guarded([&]() -> int {
    if (!cfg || !out || cfg->budget_bytes <= 0) return NRT_EINVAL;
    nrt_server *s = new (std::nothrow) nrt_server();
    if (!s) return NRT_ENOMEM;
    s->cfg = *cfg;
    if (s->cfg.chunk_steps <= 0) s->cfg.chunk_steps = 64;
    if (s->cfg.max_batch <= 0) s->cfg.max_batch = 4096;
    if (s->cfg.max_wait_us < 0) s->cfg.max_wait_us = 0;
    nrt_options_default(&s->opt[0]);
    nrt_options_default(&s->opt[1]);
    if (explicit_opt) s->opt[0] = *explicit_opt;
    if (implicit_opt) s->opt[1] = *implicit_opt;
    s->opt[0].mode = NRT_EXPLICIT;
    s->opt[1].mode = NRT_IMPLICIT_BE;
    s->opt[1].schedule = 1;  // block per instance: resident batches share the GPU
    try {
      s->worker = std::thread([s] { s->loop(); });
    } catch (const std::exception &) {
      delete s;
      return NRT_ENOMEM;
    }
    *out = s;
    return NRT_OK;
  });
}

int nrt_server_submit(nrt_server *s, const nrt_problem *p, int implicit,
                      const nrt_instance_run *run, int64_t *request_id) {
  return nrt::guarded([&]() -> int {
    return submit_request(s, p, implicit, run, nullptr, request_id);
  });
}

int nrt_server_submit_recorded(nrt_server *s, const nrt_problem *p, int implicit,
                               const nrt_instance_run *run, const nrt_record_config *rec,
                               int64_t *request_id) {
  return nrt::guarded([&]() -> int {
    if (!rec) return NRT_EINVAL;
    return submit_request(s, p, implicit, run, rec, request_id);
  });
}

int nrt_server_recording(nrt_server *s, int64_t id, int64_t *num_samples, double *times,
                         double *values, int32_t *num_spikes, double *spike_times) {
  return nrt::guarded([&]() -> int {
    if (!s) return NRT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return NRT_ESTATE;
    Request *r = it->second;
    if (!r->done) return NRT_ENOTREADY;
    if (!r->rec.on) return NRT_ESTATE;
    if (r->rec_ns.size() != r->probes.size()) return r->status != NRT_OK ? r->status : NRT_EDEVICE;
    if (num_samples) std::copy(r->rec_ns.begin(), r->rec_ns.end(), num_samples);
    if (num_spikes) std::copy(r->rec_nk.begin(), r->rec_nk.end(), num_spikes);
    if (times) std::copy(r->rec_t.begin(), r->rec_t.end(), times);
    if (values) std::copy(r->rec_v.begin(), r->rec_v.end(), values);
    if (spike_times) std::copy(r->rec_sp.begin(), r->rec_sp.end(), spike_times);
    return NRT_OK;
  });
}

int nrt_server_result(nrt_server *s, int64_t id, double *potential) {
  return nrt::guarded([&]() -> int {
    if (!s || !potential) return NRT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return NRT_ESTATE;
    Request *r = it->second;
    if (!r->done) return NRT_ENOTREADY;
    const int status = r->status;
    if (!r->result.empty()) memcpy(potential, r->result.data(), sizeof(double) * r->result.size());
    s->reqs.erase(it);
    delete r;
    return status;
  });
}

int nrt_server_drain(nrt_server *s) {
  return nrt::guarded([&]() -> int {
    if (!s) return NRT_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->outstanding == 0; });
    return NRT_OK;
  });
}

int nrt_server_get_stats(nrt_server *s, nrt_server_stats *st) {
  return nrt::guarded([&]() -> int {
    if (!s || !st) return NRT_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    *st = s->st;
    std::vector<double> l = s->lat_ms;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
      if (l.empty()) return 0.0;
      const size_t k = (size_t)std::min<double>(l.size() - 1, floor(q * (l.size() - 1) + 0.5));
      return l[k];
    };
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    st->max_ms = l.empty() ? 0.0 : l.back();
    st->busy_seconds = s->busy;
    st->peak_bytes = (int64_t)s->peak;
    return NRT_OK;
  });
}

int nrt_server_destroy(nrt_server *s) {
  return nrt::guarded([&]() -> int {
    if (!s) return NRT_EINVAL;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (auto &kv : s->reqs) delete kv.second;
    delete s;
    return NRT_OK;
  });
}

}  // extern "C"
