// Host parameter pipeline (nrt_derive): the reference's src/init.cpp:320-333,
// :235-298, :180-198, :138-174 and the formulas of inc/discretization.h:61-65,126-151,
// 208-238 for a tree description.  Used by the batch and serving front ends to turn
// geometry into solver inputs; the solver handles themselves take derived arrays, like
// the reference solver constructors do.
#include <math.h>
#include <string.h>

#include "derive_elem.h"
#include "neurite_gb300.h"

extern "C" int nrt_derive(int32_t n, const int32_t *ispec, const double *dspec, int32_t myelin,
                          double e_max, double *eparam, int32_t *hh_elem, double *hparam,
                          int32_t *num_hh_out, double *dT_crit_out) {
  if (n < 4 || !ispec || !dspec || !eparam) return NRT_EINVAL;
  const size_t N = (size_t)n;
  const int32_t *kind = ispec;
  int32_t num_hh = 0;
  for (size_t i = 0; i < N; i++) num_hh += kind[i] == 1;
  if (num_hh > 0 && (!hh_elem || !hparam)) return NRT_EINVAL;
  const double *dX0 = dspec, *diam0 = dspec + N, *eps_a = dspec + 2 * N;
  const double *ro_a_a = dspec + 4 * N, *ro_m_a = dspec + 5 * N, *per_m_a = dspec + 6 * N;
  const double *th_a = dspec + 7 * N, *rest_a = dspec + 8 * N;
  const double *sna_a = dspec + 9 * N, *sk_a = dspec + 10 * N, *sl_a = dspec + 11 * N;
  const size_t H = (size_t)num_hh;
  for (size_t i = 0, k = 0; i < N; i++) {
    nrt_param::ElemIn in;
    in.kind = kind[i];
    in.dX0 = dX0[i]; in.diam0 = diam0[i]; in.eps = eps_a[i]; in.ro_a = ro_a_a[i];
    in.ro_m = ro_m_a[i]; in.per_m = per_m_a[i]; in.th = th_a[i]; in.rest = rest_a[i];
    in.sna = sna_a[i]; in.sk = sk_a[i]; in.sl = sl_a[i];
    double ep[6], hp[12];
    nrt_param::derive_element(in, myelin, e_max, ep, hp);
    for (int q = 0; q < 6; q++) eparam[q * N + i] = ep[q];
    if (kind[i] == 1) {
      hh_elem[k] = (int32_t)i;
      for (int q = 0; q < 12; q++) hparam[q * H + k] = hp[q];
      k++;
    }
  }
  double t = eparam[5 * N + 1];
  for (size_t i = 2; i < N - 1; i++)
    if (t > eparam[5 * N + i]) t = eparam[5 * N + i];
  if (dT_crit_out) *dT_crit_out = t;
  if (num_hh_out) *num_hh_out = num_hh;
  return NRT_OK;
}

// src/init.cpp:339-358: walk the elements accumulating dX until the distance is reached;
// the reference treats "not reached" and "reached at element 0" alike (its index stays 0)
// and then measures at the middle element.
extern "C" int nrt_measurement_point(int32_t n, const double *dx, double dist_mes,
                                     int32_t *point) {
  if (n < 1 || !dx || !point) return NRT_EINVAL;
  double acc = 0;
  int32_t k_at = 0;
  for (int32_t k = 0; k < n; k++) {
    acc = acc + dx[k];
    if (acc >= dist_mes) {
      k_at = k;
      break;
    }
  }
  *point = k_at == 0 ? n / 2 : k_at;
  return NRT_OK;
}
