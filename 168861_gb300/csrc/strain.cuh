// The strained elements of an engine as the device sees them (strain.cu), and the write of
// one class's derived coefficients into an element (shared by the strain kernels and the
// explicit step's chunk kernel).
#pragma once
#include "nrt_internal.h"

namespace nrt {

// The strained elements are grouped into classes of identical input columns (instance,
// kind and the ten description values): the derivation is a pure function of those and
// of t, so one evaluation per class gives every member bit for bit what its own would.
// Elements are stored sorted by class, and a class's members are consecutive.
struct StrainView {
  int32_t n;             // strained elements
  int32_t ncls;          // classes
  const int64_t *elem;   // global element index, sorted by class
  const int64_t *col;    // parameter column of an HH element (same order)
  const int32_t *cls;    // class of each element (same order; non-decreasing)
  const int32_t *inst;   // [ncls] instance (time and dT)
  const int32_t *kind;   // [ncls] 1 HH / 0 cable
  const double *spec;    // [10][ncls]: dX, diameter, ro_a, ro_m, per_m, thickness, rest, sigma_Na, sigma_K, sigma_L
  double *tab;           // [kChunk][ncls][kStrainOut] derived ahead for a chunk of steps, or null
  int32_t *tlive;        // [kChunk][ncls]: the class's instance still runs at that step
  int32_t myelin;
  double e_max, eps0, eps1, t0, t1;
};

constexpr int kStrainOut = 2 + HP_ROWS;  // dT/(c_m dX), 1/(r_a dX), then W dX, K dX or the column

// Element q (class-sorted position) takes its class's coefficients o.
__device__ __forceinline__ void apply_element(const StrainView &s, const PackView &p, int q,
                                              const double *o, int mixed) {
  const int64_t j = s.elem[q];
  if (mixed) {
    ((float *)p.cdtf)[j] = (float)o[0];
    ((float *)p.gaxf)[j] = (float)o[1];
  } else {
    ((double *)p.cdt)[j] = o[0];
    ((double *)p.gax)[j] = o[1];
  }
  if (s.kind[s.cls[q]] == 1) {
    const int64_t cc = s.col[q];
    if (mixed) {
      float *col = (float *)(p.hpq + 3 * cc);
      for (int r = 0; r < HP_ROWS; r++) col[r] = (float)o[2 + r];
    } else {
      for (int r = 0; r < HP_ROWS; r++) ((double *)p.hp)[r * p.hp_ld + cc] = o[2 + r];
    }
  } else if (mixed) {
    ((float *)p.wdxf)[j] = (float)o[2];
    ((float *)p.kdxf)[j] = (float)o[3];
  } else {
    ((double *)p.wdx)[j] = o[2];
    ((double *)p.kdx)[j] = o[3];
  }
}

// Element q takes its class's row of the table for step k of a chunk.
__device__ __forceinline__ void apply_row(const StrainView &s, const PackView &p, int q, int k,
                                          int mixed) {
  const int64_t g = (int64_t)k * s.ncls + s.cls[q];
  if (s.tlive[g]) apply_element(s, p, q, s.tab + g * kStrainOut, mixed);
}

}  // namespace nrt
