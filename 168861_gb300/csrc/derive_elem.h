// Per-element parameter pipeline shared by nrt_derive (host) and nrt_derive_batch (device):
// the reference's src/init.cpp:320-333 (strain on dX), :235-254 (electrical_properties),
// :273-298 (hhIconds), :180-198 (cable_init_constants), :138-174 (critical time step) and
// the formulas of inc/discretization.h:61-65,126-151,208-238, in the reference's order of
// operations.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define NRT_HD __host__ __device__
#else
#define NRT_HD
#endif

namespace nrt_param {

// Model constants as the reference defines them: its truncated pi (src/neurite.cpp:72),
// the HH voltage scale (src/coupling.cpp:162), the strain-damage exponent
// (src/discretization.cpp:94) and the 45-layer myelin constants (src/discretization.cpp:54-58).
constexpr double kPi = 3.14159265;
constexpr double kScale = 0.001;
constexpr double kNDamage = 2.0;
constexpr double kThMy = 18E-9, kPerMy = 1.08E-10, kRoMy = 4.44E6;
constexpr int kLayersMy = 45;

struct Rates {
  double am, bm, ah, bh, an, bn;
};

NRT_HD inline Rates rates(double rest, double v, double ls_na, double ls_k) {
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

// One element: kind (1 HH / 0 cable) and its dspec column in; eparam column
// (c_m, r_a, dX, W, K, critical dT) and, for HH, the hparam column
// (m, h, n, g_Na, g_K, G_L, E_Na, E_K, E_L, LS_Na, LS_K, rest) out.
struct ElemIn {
  int kind;
  double dX0, diam0, eps, ro_a, ro_m, per_m, th, rest, sna, sk, sl;
};

NRT_HD inline void derive_element(const ElemIn &in, int myelin, double e_max, double ep[6],
                                  double hp[12]) {
  const double eps = in.eps;
  const double eps_s = sqrt(1 + eps) - 1;
  const double dX = in.dX0 * (1 + eps);
  const double d = in.diam0 / (sqrt(1 + eps));
  const double th = in.th, rest = in.rest;
  const double r_a = 4 * in.ro_a / (kPi * d * d);
  double r_m = (in.ro_m * th) / (kPi * d);
  double c_m = (in.per_m * kPi * d) / (th);
  double W = 0, K = 0, crit;
  if (in.kind == 1) {
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
    const double gL = in.sl * kPi * d / th;
    double gNa = in.sna * kPi * d / th;
    double gK = in.sk * kPi * d / th;
    gNa = gNa / (sqrt(1 + eps));
    gK = gK / (sqrt(1 + eps));
    Rates r = rates(rest, rest, lsna, lsk);
    const double m = r.am / (r.am + r.bm), h = r.ah / (r.ah + r.bh), nn = r.an / (r.an + r.bn);
    const double EL = (gNa * m * m * m * h * (rest - ENa) + gK * nn * nn * nn * nn * (rest - EK) +
                       gL * rest) / gL;
    hp[0] = m; hp[1] = h; hp[2] = nn; hp[3] = gNa; hp[4] = gK; hp[5] = gL;
    hp[6] = ENa; hp[7] = EK; hp[8] = EL; hp[9] = lsna; hp[10] = lsk; hp[11] = rest;
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
  ep[0] = c_m; ep[1] = r_a; ep[2] = dX; ep[3] = W; ep[4] = K; ep[5] = crit;
}

}  // namespace nrt_param
