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
  // mixed, with the table: the second copy of the coefficient rows and parameter table
  // that a graph chunk's odd steps read (the even steps read the pack's own)
  float *alt_cdtf, *alt_gaxf, *alt_wdxf, *alt_kdxf;
  float4 *alt_hpq;
  int32_t myelin;
  double e_max, eps0, eps1, t0, t1;
};

// A step that also writes the strained elements' coefficients of the next step (mixed
// explicit steps of a graph chunk).  The step's CTAs from first_block on do that instead of
// elements, at the same time as the others step.  Step k reads the copy of its parity and
// writes row k + 1 into the other (`next`), so no element of a step sees a value of the next.
struct StrainFold {
  StrainView s;
  PackView next;     // the pack with the coefficient copy step k + 1 reads
  int row;           // table row written (k + 1 of the chunk), or -1: none
  int first_block;   // the first CTA that writes rows
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

// The row-writing CTAs of a folded step: every strained element's row for the next step.
__device__ __forceinline__ void fold_rows(const StrainFold &f) {
  const int nb = gridDim.x - f.first_block;
  for (int q = (blockIdx.x - f.first_block) * blockDim.x + threadIdx.x; q < f.s.n;
       q += nb * blockDim.x)
    apply_row(f.s, f.next, q, f.row, 1);
}

}  // namespace nrt
