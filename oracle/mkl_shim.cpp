// Reverse-communication (RCI) FGMRES with the calling protocol of Intel MKL's RCI ISS
// interface (dfgmres_init / dfgmres_check / dfgmres / dfgmres_get), restated from its
// published documentation and Saad's GMRES algorithm, so that the reference's own
// src/solverIm-cpu.cpp (createMatrix + its fgmres driver, :192-272) runs unmodified.
// TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/ref_harness_im, never into the product.
//
// Third-party dependency restated: Intel MKL (version unpinned by the reference,
// Makefile:3).  Protocol used by the reference:
//   ipar[3]  iteration count, ipar[4] max iterations, ipar[7] max-iteration test on,
//   ipar[8]  residual test (off in the reference), ipar[9] user test -> RCI_request 2,
//   ipar[11] automatic zero-norm test, ipar[12] > 0 -> dfgmres_get writes into b,
//   ipar[14] restart length, ipar[21]/ipar[22] 1-based tmp offsets of the RCI 1 input
//   and output vectors; dpar[4] current residual-norm estimate (the user test reads it),
//   dpar[7] zero-norm tolerance.  RCI_request 1 = compute y = A x, 2 = stopping test,
//   0 = finished, negative = failure.
// No preconditioner (the reference never sets ipar[10]), x0 as supplied (zeros).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "mkl_rci.h"
#include "mkl_service.h"
#include "mkl_spblas.h"

namespace {

enum Stage { ST_IDLE, ST_WANT_R0, ST_HAVE_R0, ST_WANT_AV, ST_AFTER_TEST, ST_WANT_RESTART_R };

struct State {
  int n = 0, m = 0;
  Stage stage = ST_IDLE;
  std::vector<double> x;    // current iterate (x0 + committed corrections)
  std::vector<double> V;    // (m+1) x n Krylov basis
  std::vector<double> H;    // (m+1) x m Hessenberg, rotated
  std::vector<double> cs, sn, g;
  int k = 0;                // basis vectors generated in this cycle (columns of H filled)
  bool zero_norm = false;
};
State S;

void csr_mv(int n, const double *a, const MKL_INT *ia, const MKL_INT *ja, const double *x, double *y) {
  for (int i = 0; i < n; i++) {
    double s = 0;
    for (int p = ia[i]; p < ia[i + 1]; p++) s += a[p] * x[ja[p]];
    y[i] = s;
  }
}

// x_cur = x + V_k y_k with y_k from the rotated Hessenberg system (k columns).
void current_solution(std::vector<double> &out) {
  const int n = S.n, m = S.m, k = S.k;
  std::vector<double> y(k > 0 ? k : 1);
  for (int i = k - 1; i >= 0; i--) {
    double s = S.g[i];
    for (int l = i + 1; l < k; l++) s -= S.H[(size_t)i * m + l] * y[l];
    y[i] = s / S.H[(size_t)i * m + i];
  }
  out = S.x;
  for (int i = 0; i < k; i++)
    for (int r = 0; r < n; r++) out[r] += y[i] * S.V[(size_t)i * n + r];
}

void request_matvec(const double *src, double *tmp, MKL_INT *ipar, MKL_INT *req) {
  memcpy(tmp, src, sizeof(double) * S.n);
  ipar[21] = 1;
  ipar[22] = S.n + 1;
  *req = 1;
}

// Starts a cycle from the residual r currently in tmp[n..2n) (holding A x).
void start_cycle(const double *b, double *tmp, MKL_INT *ipar, double *dpar) {
  const int n = S.n;
  double *v0 = &S.V[0];
  double beta = 0;
  for (int i = 0; i < n; i++) {
    v0[i] = b[i] - tmp[n + i];
    beta += v0[i] * v0[i];
  }
  beta = sqrt(beta);
  if (S.stage == ST_WANT_R0) {
    dpar[2] = beta;
    dpar[3] = dpar[0] * beta + dpar[1];
  }
  dpar[4] = beta;
  std::fill(S.g.begin(), S.g.end(), 0.0);
  S.g[0] = beta;
  S.k = 0;
  S.zero_norm = beta == 0;
  if (beta != 0)
    for (int i = 0; i < n; i++) v0[i] /= beta;
  ipar[13] = 0;
}

}  // namespace

void dfgmres_init(const MKL_INT *n, const double *x, const double *b, MKL_INT *req, MKL_INT *ipar,
                  double *dpar, double *tmp) {
  (void)b;
  (void)tmp;
  memset(ipar, 0, sizeof(MKL_INT) * 128);
  memset(dpar, 0, sizeof(double) * 128);
  ipar[0] = *n;
  ipar[1] = 6;
  ipar[2] = 1;
  ipar[4] = *n < 150 ? *n : 150;
  ipar[5] = 1;
  ipar[6] = 1;
  ipar[7] = 1;
  ipar[8] = 0;
  ipar[9] = 1;
  ipar[14] = *n < 150 ? *n : 150;
  dpar[0] = 1e-6;
  dpar[7] = 1e-12;
  S = State();
  S.n = *n;
  S.x.assign(x, x + *n);
  *req = 0;
}

void dfgmres_check(const MKL_INT *n, const double *x, const double *b, MKL_INT *req, MKL_INT *ipar,
                   double *dpar, double *tmp) {
  (void)x;
  (void)b;
  (void)dpar;
  (void)tmp;
  if (*n <= 0 || ipar[14] <= 0) {
    *req = -1100;
    return;
  }
  if (ipar[14] > *n) ipar[14] = *n;
  S.m = ipar[14];
  S.V.assign((size_t)(S.m + 1) * S.n, 0.0);
  S.H.assign((size_t)(S.m + 1) * S.m, 0.0);
  S.cs.assign(S.m, 0.0);
  S.sn.assign(S.m, 0.0);
  S.g.assign(S.m + 1, 0.0);
  S.stage = ST_IDLE;
  *req = 0;
}

void dfgmres(const MKL_INT *n, double *x, double *b, MKL_INT *req, MKL_INT *ipar, double *dpar,
             double *tmp) {
  (void)n;
  (void)x;
  const int N = S.n, m = S.m;
  for (;;) {
    switch (S.stage) {
      case ST_IDLE:  // first call: residual of x0
        S.stage = ST_WANT_R0;
        request_matvec(S.x.data(), tmp, ipar, req);
        return;
      case ST_WANT_R0:
      case ST_WANT_RESTART_R:
        start_cycle(b, tmp, ipar, dpar);
        if (S.zero_norm) {  // exact solution already
          S.stage = ST_AFTER_TEST;
          if (ipar[9]) { *req = 2; return; }
          *req = 0;
          return;
        }
        S.stage = ST_HAVE_R0;
        break;
      case ST_HAVE_R0:  // ask for A v_k
        if (ipar[7] && ipar[3] >= ipar[4]) {
          *req = -1;
          return;
        }
        S.stage = ST_WANT_AV;
        request_matvec(&S.V[(size_t)S.k * N], tmp, ipar, req);
        return;
      case ST_WANT_AV: {  // Arnoldi step with modified Gram-Schmidt, Givens update
        const int k = S.k;
        double *w = &S.V[(size_t)(k + 1) * N];
        memcpy(w, tmp + N, sizeof(double) * N);
        for (int i = 0; i <= k; i++) {
          const double *vi = &S.V[(size_t)i * N];
          double h = 0;
          for (int r = 0; r < N; r++) h += w[r] * vi[r];
          S.H[(size_t)i * m + k] = h;
          for (int r = 0; r < N; r++) w[r] -= h * vi[r];
        }
        double hn = 0;
        for (int r = 0; r < N; r++) hn += w[r] * w[r];
        hn = sqrt(hn);
        dpar[5] = dpar[6];
        dpar[6] = hn;
        S.H[(size_t)(k + 1) * m + k] = hn;
        if (hn != 0)
          for (int r = 0; r < N; r++) w[r] /= hn;
        for (int i = 0; i < k; i++) {
          const double a = S.H[(size_t)i * m + k], c = S.H[(size_t)(i + 1) * m + k];
          S.H[(size_t)i * m + k] = S.cs[i] * a + S.sn[i] * c;
          S.H[(size_t)(i + 1) * m + k] = -S.sn[i] * a + S.cs[i] * c;
        }
        const double a = S.H[(size_t)k * m + k], c = S.H[(size_t)(k + 1) * m + k];
        const double den = sqrt(a * a + c * c);
        S.cs[k] = den == 0 ? 1 : a / den;
        S.sn[k] = den == 0 ? 0 : c / den;
        S.H[(size_t)k * m + k] = den;
        S.H[(size_t)(k + 1) * m + k] = 0;
        S.g[k + 1] = -S.sn[k] * S.g[k];
        S.g[k] = S.cs[k] * S.g[k];
        S.k = k + 1;
        ipar[3] += 1;
        ipar[13] = S.k;
        dpar[4] = fabs(S.g[k + 1]);
        S.zero_norm = ipar[11] && hn <= dpar[7];
        S.stage = ST_AFTER_TEST;
        if (ipar[8] && dpar[4] <= dpar[3]) {
          *req = 0;
          return;
        }
        if (ipar[9]) {
          *req = 2;
          return;
        }
        break;
      }
      case ST_AFTER_TEST:  // the caller chose to continue
        if (S.zero_norm && S.k > 0) {
          *req = 0;
          return;
        }
        if (S.k == m) {  // restart: commit x, recompute the true residual
          std::vector<double> xn;
          current_solution(xn);
          S.x.swap(xn);
          S.k = 0;
          S.stage = ST_WANT_RESTART_R;
          request_matvec(S.x.data(), tmp, ipar, req);
          return;
        }
        S.stage = ST_HAVE_R0;
        break;
    }
  }
}

void dfgmres_get(const MKL_INT *n, double *x, double *b, MKL_INT *req, const MKL_INT *ipar,
                 const double *dpar, double *tmp, MKL_INT *itercount) {
  (void)dpar;
  (void)tmp;
  std::vector<double> sol;
  current_solution(sol);
  double *dst = ipar[12] > 0 ? b : x;
  memcpy(dst, sol.data(), sizeof(double) * (*n));
  *itercount = ipar[3];
  *req = 0;
}

void mkl_cspblas_dcsrgemv(const char *transa, const MKL_INT *m, const double *a, const MKL_INT *ia,
                          const MKL_INT *ja, const double *x, double *y) {
  (void)transa;  // the reference passes 'N'
  csr_mv(*m, a, ia, ja, x, y);
}

void MKL_Free_Buffers(void) { S = State(); }
