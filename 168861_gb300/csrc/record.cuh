// One probe's recording update after the step at loop index i (device side; used by the
// explicit record kernel and inside the persistent implicit kernel).
//
// Samples follow the reference driver's counter (src/neurite.cpp:241-248, a snapshot
// when ++GL_cont > interval, the loop starting at `origin`): loop index i is sampled when
// i - origin + 1 is a positive multiple of interval + 1.  A spike is an upward crossing of
// the threshold between consecutive loop indices, timed by linear interpolation between
// (i - 1) dT and i dT.  One thread owns a probe for a whole launch, so the per-probe state
// needs no atomics.
#pragma once
#include "nrt_internal.h"

namespace nrt {

__device__ __forceinline__ void record_probe(const RecView &r, int p, int64_t i, double v,
                                             double dT) {
  const double pv = r.prev_v[p];
  if (r.prev_i[p] == i - 1 && pv < r.thresh && v >= r.thresh) {
    const int n = r.nspike[p];
    if (n < r.max_spikes) {
      const double t0 = (double)(i - 1) * dT, t1 = (double)i * dT;
      const double frac = (r.thresh - pv) * (t1 - t0);
      r.spk[(int64_t)p * r.max_spikes + n] = t0 + frac / (v - pv);
    }
    r.nspike[p] = n + 1;
  }
  r.prev_v[p] = v;
  r.prev_i[p] = i;
  const int64_t q = i - r.origin + 1;
  if (q > 0 && q % (r.interval + 1) == 0) {
    const int64_t s = q / (r.interval + 1) - 1;
    if (s < r.cap) r.val[(int64_t)p * r.cap + s] = v;
    if (s + 1 > r.nsamp[p]) r.nsamp[p] = s + 1;
  }
}

}  // namespace nrt
