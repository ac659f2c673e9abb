// Hodgkin-Huxley rate functions and the forward-Euler gate step, FP64 and FP32 forms.
//
// Model: src/coupling.cpp:25-48 (hhRate_Const), gate and conductance update
// src/solverEx-cpu.cpp:106-127, W and K src/discretization.cpp:99-104.  Voltages enter in
// mV relative to rest (SCALE 0.001, inc/configuration.h:36) and dt in ms.
#pragma once
#include <cuda_runtime.h>

namespace nrt {

struct GateStep64 {
  double m, h, n;   // gates after the step
  double W, K;      // membrane coefficients with the new gates
};

// The six FP64 rates (order: alpha_m, beta_m, alpha_h, beta_h, alpha_n, beta_n) are
// each one exponential and one quotient or product of it.  hh_rate64 gives rate q with the
// same code for every q -- so lanes of a warp can evaluate different rates of one element
// without diverging -- and with exactly the value of the reference's expression:
//   alpha_m = xm / (e^xm - 1),            xm = 2.5 - 0.1 v_Na
//   beta_m  = 4 e^(-v_Na/18)              alpha_h = 0.07 e^(-v_Na/20)
//   beta_h  = 1 / (e^(3 - 0.1 v_Na) + 1)
//   alpha_n = (0.1 - 0.01 v_K) / (e^xn - 1),  xn = 1 - 0.1 v_K
//   beta_n  = 0.125 e^(-v_K/80)
// (a product is divided by 1.0, which is exact; the selects keep e^x = inf from meeting a 0).
// The a - b c terms are explicit fused multiply-adds, so that a constant q and a q chosen
// per lane round them alike (left to contraction, a shared 0.1 v_Na product could be
// rounded on its own in one and fused in the other).
__device__ __forceinline__ double hh_rate64(int q, double vna, double vk) {
  const double xm = fma(-0.1, vna, 2.5);
  const double xn = fma(-0.1, vk, 1.0);
  const double x = q == 0 ? xm : q == 1 ? vna * (-1.0 / 18.0) : q == 2 ? vna * (-1.0 / 20.0)
                 : q == 3 ? fma(-0.1, vna, 3.0) : q == 4 ? xn : vk * (-1.0 / 80.0);
  const double e = exp(x);
  const double c = q == 1 ? 4.0 : q == 2 ? 0.07 : 0.125;
  const double num = q == 0 ? xm : q == 3 ? 1.0 : q == 4 ? fma(-0.01, vk, 0.1) : c * e;
  const double den = (q == 0 || q == 4) ? e - 1.0 : q == 3 ? e + 1.0 : 1.0;
  return num / den;
}

// The forward-Euler gate step and W, K from the six rates.  The fused multiply-adds are
// written out: a - b c + d e style sums have two ways to fuse, and left to the compiler the
// choice could differ between kernels that inline this (the lanes kernel and the others
// must agree bit for bit).
__device__ __forceinline__ GateStep64 hh_gates64(double am, double bm, double ah, double bh,
                                                 double an, double bn, double m0, double h0,
                                                 double n0, double dt_ms, double gNa,
                                                 double gK, double GL, double ENa, double EK,
                                                 double EL) {
  GateStep64 r;
  r.m = fma(dt_ms, fma(am, 1.0 - m0, -(bm * m0)), m0);
  r.h = fma(dt_ms, fma(ah, 1.0 - h0, -(bh * h0)), h0);
  r.n = fma(dt_ms, fma(an, 1.0 - n0, -(bn * n0)), n0);
  const double G_Na = gNa * r.m * r.m * r.m * r.h;
  const double G_K = gK * r.n * r.n * r.n * r.n;
  r.W = -(G_Na + G_K + GL);
  r.K = fma(GL, EL, fma(G_K, EK, G_Na * ENa));
  return r;
}

// FP64: the reference's expressions with constant divisions turned into products.
__device__ __forceinline__ GateStep64 hh_step64(double v, double m0, double h0, double n0,
                                                double ls_na, double ls_k, double rest,
                                                double dt_ms, double gNa, double gK, double GL,
                                                double ENa, double EK, double EL) {
  const double vna = ((v + ls_na) - rest) * 1000.0;
  const double vk = ((v + ls_k) - rest) * 1000.0;
  return hh_gates64(hh_rate64(0, vna, vk), hh_rate64(1, vna, vk), hh_rate64(2, vna, vk),
                    hh_rate64(3, vna, vk), hh_rate64(4, vna, vk), hh_rate64(5, vna, vk), m0,
                    h0, n0, dt_ms, gNa, gK, GL, ENa, EK, EL);
}

// x / (e^x - 1), the shape of alpha_m and alpha_n, with its removable singularity at 0
// handled by the series 1 / (1 + x/2 + x^2/6) for |x| < 1e-3.  Both branches use the fast
// reciprocal (a relative error of a few 1e-7, far below the FP32 gates' own rounding).
__device__ __forceinline__ float xexpm1_ratio(float x, float ex) {
  const float den = fabsf(x) < 1e-3f ? fmaf(x, fmaf(x, 1.0f / 6.0f, 0.5f), 1.0f) : ex - 1.0f;
  const float num = fabsf(x) < 1e-3f ? 1.0f : x;
  return __fdividef(num, den);
}

struct GateStep32 {
  float m, h, n, W, K;
};

// FP32 form for the mixed-precision path.  dv_na / dv_k are (V + LS - rest) in volts,
// formed in FP64 by the caller and rounded once.  exp(3 - 0.1 v) is e^0.5 * exp(2.5 - 0.1 v).
__device__ __forceinline__ GateStep32 hh_step32(float dv_na, float dv_k, float m0, float h0,
                                                float n0, float dt_ms, float gNa, float gK,
                                                float GL, float ENa, float EK, float EL) {
  const float vna = dv_na * 1000.0f;
  const float vk = dv_k * 1000.0f;
  const float xm = fmaf(-0.1f, vna, 2.5f);
  const float exm = __expf(xm);
  const float am = xexpm1_ratio(xm, exm);
  const float bm = 4.0f * __expf(vna * (-1.0f / 18.0f));
  const float ah = 0.07f * __expf(vna * (-1.0f / 20.0f));
  const float bh = __fdividef(1.0f, fmaf(exm, 1.6487212707001282f, 1.0f));
  const float xn = fmaf(-0.1f, vk, 1.0f);
  const float an = 0.1f * xexpm1_ratio(xn, __expf(xn));
  const float bn = 0.125f * __expf(vk * (-1.0f / 80.0f));
  GateStep32 r;
  r.m = fmaf(dt_ms, am * (1.0f - m0) - bm * m0, m0);
  r.h = fmaf(dt_ms, ah * (1.0f - h0) - bh * h0, h0);
  r.n = fmaf(dt_ms, an * (1.0f - n0) - bn * n0, n0);
  const float G_Na = gNa * r.m * r.m * r.m * r.h;
  const float n2 = r.n * r.n;
  const float G_K = gK * n2 * n2;
  r.W = -(G_Na + G_K + GL);
  r.K = fmaf(G_Na, ENa, fmaf(G_K, EK, GL * EL));
  return r;
}

}  // namespace nrt
