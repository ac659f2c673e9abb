// Host parameter pipeline (nrt_derive): the reference's src/init.cpp:320-333,
// :235-298, :180-198, :138-174 and the formulas of inc/discretization.h:61-65,126-151,
// 208-238 for a tree description.  Used by the batch and serving front ends to turn
// geometry into solver inputs; the solver handles themselves take derived arrays, like
// the reference solver constructors do.
#include <math.h>
#include <string.h>

#include "neurite_gb300.h"

namespace {

// Model constants as the reference defines them: its truncated pi (src/neurite.cpp:72),
// the HH voltage scale (src/coupling.cpp:162), the strain-damage exponent
// (src/discretization.cpp:94) and the 45-layer myelin constants (src/discretization.cpp:54-58).
const double kPi = 3.14159265;
const double kScale = 0.001;
const double kNDamage = 2.0;
const double kThMy = 18E-9, kPerMy = 1.08E-10, kRoMy = 4.44E6;
const int kLayersMy = 45;

struct Rates {
  double am, bm, ah, bh, an, bn;
};

Rates rates(double rest, double v, double ls_na, double ls_k) {
  double vna = ((v + ls_na) - rest) / kScale;
  double vk = ((v + ls_k) - rest) / kScale;
  Rates r;
  r.am = (2.5 - 0.1 * vna) / (exp(2.5 - 0.1 * vna) - 1);
  r.bm = 4 * exp(-vna / 18);
  r.ah = 0.07 * exp(-vna / 20);
  r.bh = 1 / (exp(3 - 0.1 * vna) + 1);
  r.an = (0.1 - 0.01 * vk) / (exp(1 - 0.1 * vk) - 1);
  r.bn = 0.125 * exp(-vk / 80);
  return r;
}

}  // namespace

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
    const double eps = eps_a[i];
    const double eps_s = sqrt(1 + eps) - 1;
    const double dX = dX0[i] * (1 + eps);
    const double d = diam0[i] / (sqrt(1 + eps));
    const double th = th_a[i], rest = rest_a[i];
    const double r_a = 4 * ro_a_a[i] / (kPi * d * d);
    double r_m = (ro_m_a[i] * th) / (kPi * d);
    double c_m = (per_m_a[i] * kPi * d) / (th);
    double W = 0, K = 0, crit;
    if (kind[i] == 1) {
      const double ENa0 = 0.115 + rest, EK0 = -0.012 + rest;
      double ENa, EK, lsna, lsk;
      if (eps_s <= e_max) {
        const double f = pow((eps_s / e_max), kNDamage);
        ENa = ENa0 - f * (ENa0);
        EK = EK0 - f * (EK0);
        lsna = f * (ENa0);
        lsk = f * (EK0);
      } else {
        ENa = 0;
        EK = 0;
        lsna = ENa0;
        lsk = EK0;
      }
      const double gL = sl_a[i] * kPi * d / th;
      double gNa = sna_a[i] * kPi * d / th;
      double gK = sk_a[i] * kPi * d / th;
      gNa = gNa / (sqrt(1 + eps));
      gK = gK / (sqrt(1 + eps));
      Rates r = rates(rest, rest, lsna, lsk);
      const double m = r.am / (r.am + r.bm), h = r.ah / (r.ah + r.bh), nn = r.an / (r.an + r.bn);
      const double EL = (gNa * m * m * m * h * (rest - ENa) + gK * nn * nn * nn * nn * (rest - EK) +
                         gL * rest) / gL;
      hh_elem[k] = (int32_t)i;
      const double vals[12] = {m, h, nn, gNa, gK, gL, ENa, EK, EL, lsna, lsk, rest};
      for (int q = 0; q < 12; q++) hparam[q * H + k] = vals[q];
      k++;
      crit = (2 * r_a * c_m * dX * dX) / 4;
    } else {
      if (myelin) {
        double temp = 0;
        for (int l = 1; l <= kLayersMy; l++) temp = temp + 1 / (d + th * 2 + 2 * (l - 1) * kThMy);
        const double c_my = 1 / (kThMy * temp / (kPerMy * kPi));
        const double r_my = (kRoMy * kThMy * temp) / kPi;
        r_m = r_m + r_my;
        c_m = (c_m * c_my) / (c_my + c_m);
      }
      W = -1 / r_m;
      K = rest / r_m;
      crit = (2 * r_a * c_m * dX * dX) / (4 + (r_a * dX * dX) / r_m);
    }
    eparam[0 * N + i] = c_m;
    eparam[1 * N + i] = r_a;
    eparam[2 * N + i] = dX;
    eparam[3 * N + i] = W;
    eparam[4 * N + i] = K;
    eparam[5 * N + i] = crit;
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
