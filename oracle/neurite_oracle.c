/* CPU oracle for the Neurite solver hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates the reference's CPU algorithms with the reference's own expression order so
 * that, compiled with -ffp-contract=off, it reproduces the reference binary bit-for-bit
 * (checked by tests/test_oracle_golden.py against fixtures made by oracle/_ref).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and only
 * as the checker or the timed CPU baseline; the product never calls it.
 * See neurite_oracle.h for the array conventions.
 */
#include "neurite_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Constants the reference hard-codes (kept identical; they define the model). */
static const double NRO_PI = 3.14159265;   /* src/neurite.cpp:72 (truncated pi is part of the model) */
static const double NRO_SCALE = 0.001;     /* src/coupling.cpp:162, inc/configuration.h:36 */
static const double NRO_N_DAMAGE = 2.0;    /* src/discretization.cpp:94 */
/* Cable myelin constants, src/discretization.cpp:54-58 (45-layer myelin model). */
static const double NRO_TH_MY = 18E-9, NRO_PER_MY = 1.08E-10, NRO_RO_MY = 4.44E6;
static const int NRO_LAYERS_MY = 45;

#define ISPEC(k, i) ispec[(size_t)(k) * n + (i)]
#define DSPEC(k, i) dspec[(size_t)(k) * n + (i)]
#define EP(k, i) eparam[(size_t)(k) * n + (i)]
#define HP(k, i) hparam[(size_t)(k) * num_hh + (i)]

enum { IS_KIND, IS_MOTHER, IS_DR, IS_DL, IS_BRANCH };
enum { DS_DX, DS_DIAM, DS_EPS, DS_IINJ, DS_ROA, DS_ROM, DS_PERM, DS_TH, DS_REST, DS_SNA, DS_SK, DS_SL };
enum { EP_CM, EP_RA, EP_DX, EP_W, EP_K, EP_CRIT };
enum { HP_M, HP_H, HP_N, HP_GNA, HP_GK, HP_GL, HP_ENA, HP_EK, HP_EL, HP_LSNA, HP_LSK, HP_REST };

typedef struct { double m, h, n; } rates_t;

/* src/coupling.cpp:25-48 (hhRate_Const) */
static void hh_rates(rates_t *a, rates_t *b, double rest_pot, double potential, double ls_na,
                     double ls_k) {
  double vna = potential + ls_na;
  double vk = potential + ls_k;
  vna = (vna - rest_pot) / NRO_SCALE;
  vk = (vk - rest_pot) / NRO_SCALE;
  a->m = (2.5 - 0.1 * vna) / (exp(2.5 - 0.1 * vna) - 1);
  b->m = 4 * exp(-vna / 18);
  a->h = 0.07 * exp(-vna / 20);
  b->h = 1 / (exp(3 - 0.1 * vna) + 1);
  a->n = (0.1 - 0.01 * vk) / (exp(1 - 0.1 * vk) - 1);
  b->n = 0.125 * exp(-vk / 80);
}

int nro_derive(int n, const int32_t *ispec, const double *dspec, int myelin, double e_max,
               double *eparam, int32_t *hh_elem, double *hparam, int *num_hh_out,
               double *dT_crit_out) {
  if (n < 4 || !ispec || !dspec || !eparam) return NRO_EINVAL;
  int num_hh = 0;
  for (int i = 0; i < n; i++) num_hh += ISPEC(IS_KIND, i) == 1;
  for (int i = 0, k = 0; i < n; i++) {
    double eps = DSPEC(DS_EPS, i);
    double eps_s = sqrt(1 + eps) - 1;                  /* inc/discretization.h:50-53 */
    double dX = DSPEC(DS_DX, i) * (1 + eps);           /* src/init.cpp:329-331 */
    double d = DSPEC(DS_DIAM, i) / (sqrt(1 + eps));    /* src/init.cpp:184,239 */
    double ro_a = DSPEC(DS_ROA, i), ro_m = DSPEC(DS_ROM, i), per_m = DSPEC(DS_PERM, i);
    double th = DSPEC(DS_TH, i), rest = DSPEC(DS_REST, i);
    double r_a = 4 * ro_a / (NRO_PI * d * d);          /* inc/discretization.h:61-65 */
    double r_m = (ro_m * th) / (NRO_PI * d);
    double c_m = (per_m * NRO_PI * d) / (th);
    double W = 0, K = 0, crit;
    if (ISPEC(IS_KIND, i) == 1) {
      /* src/init.cpp:235-254 and inc/discretization.h:208-238 */
      double ENa0 = 0.115 + rest, EK0 = -0.012 + rest, ENa, EK, lsna, lsk;
      if (eps_s <= e_max) {
        ENa = ENa0 - pow((eps_s / e_max), NRO_N_DAMAGE) * (ENa0);
        EK = EK0 - pow((eps_s / e_max), NRO_N_DAMAGE) * (EK0);
        lsna = pow(eps_s / e_max, NRO_N_DAMAGE) * (ENa0);
        lsk = pow(eps_s / e_max, NRO_N_DAMAGE) * (EK0);
      } else {
        ENa = 0;
        EK = 0;
        lsna = ENa0;
        lsk = EK0;
      }
      double gL = DSPEC(DS_SL, i) * NRO_PI * d / th;
      double gNa = DSPEC(DS_SNA, i) * NRO_PI * d / th;
      double gK = DSPEC(DS_SK, i) * NRO_PI * d / th;
      gNa = gNa / (sqrt(1 + eps));
      gK = gK / (sqrt(1 + eps));
      /* src/init.cpp:273-298 (hhIconds): steady-state gates and the leak reversal */
      rates_t a, b;
      hh_rates(&a, &b, rest, rest, lsna, lsk);
      double m = a.m / (a.m + b.m), h = a.h / (a.h + b.h), nn = a.n / (a.n + b.n);
      double EL = (gNa * m * m * m * h * (rest - ENa) + gK * nn * nn * nn * nn * (rest - EK) +
                   gL * rest) / gL;
      if (hh_elem) {
        hh_elem[k] = i;
        HP(HP_M, k) = m; HP(HP_H, k) = h; HP(HP_N, k) = nn;
        HP(HP_GNA, k) = gNa; HP(HP_GK, k) = gK; HP(HP_GL, k) = gL;
        HP(HP_ENA, k) = ENa; HP(HP_EK, k) = EK; HP(HP_EL, k) = EL;
        HP(HP_LSNA, k) = lsna; HP(HP_LSK, k) = lsk; HP(HP_REST, k) = rest;
      }
      k++;
      crit = (2 * r_a * c_m * dX * dX) / 4;            /* src/init.cpp:141 */
    } else {
      /* src/init.cpp:180-198, inc/discretization.h:126-151 */
      if (myelin) {
        double temp = 0;
        for (int l = 1; l <= NRO_LAYERS_MY; l++)
          temp = temp + 1 / (d + th * 2 + 2 * (l - 1) * NRO_TH_MY);
        double c_my_T = NRO_TH_MY * temp / (NRO_PER_MY * NRO_PI);
        double c_my = 1 / c_my_T;
        double r_my = (NRO_RO_MY * NRO_TH_MY * temp) / NRO_PI;
        r_m = r_m + r_my;
        c_m = (c_m * c_my) / (c_my + c_m);
      }
      W = -1 / r_m;                                    /* src/discretization.cpp:63-68 */
      K = rest / r_m;
      crit = (2 * r_a * c_m * dX * dX) / (4 + (r_a * dX * dX) / r_m);  /* src/init.cpp:144 */
    }
    EP(EP_CM, i) = c_m; EP(EP_RA, i) = r_a; EP(EP_DX, i) = dX;
    EP(EP_W, i) = W; EP(EP_K, i) = K; EP(EP_CRIT, i) = crit;
  }
  /* src/init.cpp:165-174 */
  double t = EP(EP_CRIT, 1);
  for (int i = 2; i < n - 1; i++)
    if (t > EP(EP_CRIT, i)) t = EP(EP_CRIT, i);
  if (dT_crit_out) *dT_crit_out = t;
  if (num_hh_out) *num_hh_out = num_hh;
  return NRO_OK;
}

/* SolverExCPU::update gate loop (src/solverEx-cpu.cpp:106-127); also the implicit
 * variant (src/solverIm-cpu.cpp:326-349), which is the same arithmetic. */
static void hh_update(int num_hh, const int32_t *hh_elem, double *hparam, const double *Vprev,
                      double dT, double *W, double *K) {
  const double dt = dT * 1000;
  for (int i = 0; i < num_hh; i++) {
    rates_t a, b;
    int e = hh_elem[i];
    hh_rates(&a, &b, HP(HP_REST, i), Vprev[e], HP(HP_LSNA, i), HP(HP_LSK, i));
    double m0 = HP(HP_M, i), h0 = HP(HP_H, i), n0 = HP(HP_N, i);
    double m = m0 + dt * (a.m * (1 - m0) - b.m * m0);
    double h = h0 + dt * (a.h * (1 - h0) - b.h * h0);
    double nn = n0 + dt * (a.n * (1 - n0) - b.n * n0);
    double GNa = HP(HP_GNA, i) * m * m * m * h;
    double GK = HP(HP_GK, i) * nn * nn * nn * nn;
    double GL = HP(HP_GL, i);
    W[e] = -(GNa + GK + GL);                              /* src/discretization.cpp:99-101 */
    K[e] = GNa * HP(HP_ENA, i) + GK * HP(HP_EK, i) + GL * HP(HP_EL, i);  /* :102-104 */
    HP(HP_M, i) = m; HP(HP_H, i) = h; HP(HP_N, i) = nn;
  }
}

int nro_explicit_run(int n, const int32_t *ispec, const double *eparam, const double *input_on,
                     int num_term, const int32_t *terminals, int num_hh, const int32_t *hh_elem,
                     double *hparam, double dT, int i_begin, int i_end, double init_time,
                     double end_input, double *V, int record_every, int nprobe,
                     const int32_t *probes, double *trace, int *nrec_out) {
  if (n < 3 || num_term < 1) return NRO_EINVAL;
  double *W = malloc(sizeof(double) * n), *K = malloc(sizeof(double) * n);
  double *prevT = malloc(sizeof(double) * n), *currT = malloc(sizeof(double) * n);
  double *zero = calloc(n, sizeof(double));
  if (!W || !K || !prevT || !currT || !zero) {
    free(W); free(K); free(prevT); free(currT); free(zero);
    return NRO_ENOMEM;
  }
  memcpy(W, eparam + (size_t)EP_W * n, sizeof(double) * n);
  memcpy(K, eparam + (size_t)EP_K * n, sizeof(double) * n);
  memcpy(prevT, V, sizeof(double) * n);
  memcpy(currT, V, sizeof(double) * n);
  const double *c_m = eparam + (size_t)EP_CM * n, *r_a = eparam + (size_t)EP_RA * n;
  const double *dX = eparam + (size_t)EP_DX * n;
  int nrec = 0;
  for (int it = i_begin; it < i_end; it++) {
    double time_run = it * dT;
    const double *input = ((time_run >= init_time) && (time_run <= end_input)) ? input_on : zero;
    hh_update(num_hh, hh_elem, hparam, prevT, dT, W, K);
    /* src/solverEx-cpu.cpp:137-153 */
    for (int j = 1; j < n - 1; j++) {
      double Rp = prevT[j];
      int dl = ISPEC(IS_DL, j), dr = ISPEC(IS_DR, j), mo = ISPEC(IS_MOTHER, j);
      double br = ISPEC(IS_BRANCH, j) ? 1.0 : 0.0;
      currT[j] = Rp + (dT / (c_m[j] * dX[j])) *
                          (br * ((prevT[dl] - Rp) / (r_a[dl] * dX[dl])) +
                           (prevT[dr] - Rp) / (r_a[dr] * dX[dr]) +
                           (prevT[mo] - Rp) / (r_a[j] * dX[j]) + W[j] * dX[j] * Rp +
                           K[j] * dX[j] + input[j]);
    }
    /* src/solverEx-cpu.cpp:155-161 */
    currT[terminals[0]] = currT[terminals[0] + 1];
    for (int k = 1; k < num_term; k++) currT[terminals[k]] = currT[ISPEC(IS_MOTHER, terminals[k])];
    double *flip = currT; currT = prevT; prevT = flip;
    if (record_every > 0 && (it % record_every) == 0 && trace) {
      double *row = trace + (size_t)nrec * (nprobe + 1);
      row[0] = it;
      for (int p = 0; p < nprobe; p++) row[p + 1] = prevT[probes[p]];
      nrec++;
    }
  }
  memcpy(V, prevT, sizeof(double) * n);
  if (nrec_out) *nrec_out = nrec;
  free(W); free(K); free(prevT); free(currT); free(zero);
  return NRO_OK;
}

/* One matrix row of createMatrix: the alpha/beta/gamma/delta of src/solverIm-cpu.cpp:51-54
 * (identical at :102-105, :117-120, :149-152). */
typedef struct { double alpha, beta, gamma, delta; } rowc_t;
static rowc_t row_coeffs(int n, const int32_t *ispec, const double *c_m, const double *r_a,
                         const double *dX, const double *W, double dT, int j) {
  rowc_t r;
  int dl = ISPEC(IS_DL, j), dr = ISPEC(IS_DR, j);
  double br = ISPEC(IS_BRANCH, j) ? 1.0 : 0.0;
  r.gamma = -br / (r_a[dl] * dX[dl]);
  r.beta = (c_m[j] * dX[j]) / dT - W[j] * dX[j] + br / (r_a[dl] * dX[dl]) +
           1 / (r_a[dr] * dX[dr]) + 1 / (r_a[j] * dX[j]);
  r.alpha = -1 / (r_a[j] * dX[j]);
  r.delta = -1 / (r_a[dr] * dX[dr]);
  return r;
}

int nro_implicit_matrix(int n, const int32_t *ispec, const double *eparam, const double *W,
                        const double *K, const double *input, double dT, const double *Vprev,
                        int32_t *row_ptr, int32_t *col, double *val, double *rhs, int *nnz_out) {
  if (n < 4) return NRO_EINVAL;
  const double *c_m = eparam + (size_t)EP_CM * n, *r_a = eparam + (size_t)EP_RA * n;
  const double *dX = eparam + (size_t)EP_DX * n;
  int nnz = 1;
  val[0] = 1; col[0] = 0; row_ptr[0] = 0;
#define RHS(j) (c_m[j] * dX[j] * Vprev[j] / dT + K[j] * dX[j] + input[j])
  /* row 1, src/solverIm-cpu.cpp:50-83: the mother column folds into the diagonal */
  {
    int j = 1, dl = ISPEC(IS_DL, 1), dr = ISPEC(IS_DR, 1);
    rowc_t r = row_coeffs(n, ispec, c_m, r_a, dX, W, dT, j);
    r.beta = r.beta + r.alpha;
    val[nnz] = r.beta; col[nnz] = 1; row_ptr[1] = nnz; nnz++;
    if (dl == 0) {
      val[nnz] = r.delta; col[nnz] = dr; nnz++;
    } else if (dr < dl) {
      val[nnz] = r.delta; col[nnz] = dr; nnz++;
      val[nnz] = r.gamma; col[nnz] = dl; nnz++;
    } else {
      val[nnz] = r.gamma; col[nnz] = dl; nnz++;
      val[nnz] = r.delta; col[nnz] = dr; nnz++;
    }
    rhs[1] = RHS(1);
  }
  /* rows 2 .. n-3, src/solverIm-cpu.cpp:86-145 */
  int flag_salto = 0, j;
  for (j = 2; j < n - 2; j++) {
    if (flag_salto) {
      flag_salto = 0;
      val[nnz] = 1; col[nnz] = j; row_ptr[j] = nnz; nnz++;
      continue;
    }
    rowc_t r = row_coeffs(n, ispec, c_m, r_a, dX, W, dT, j);
    if (ISPEC(IS_DR, j + 1) == j + 1) {
      flag_salto = 1;
      val[nnz] = r.alpha; col[nnz] = ISPEC(IS_MOTHER, j); row_ptr[j] = nnz; nnz++;
      val[nnz] = r.beta + r.delta; col[nnz] = j; nnz++;
    } else {
      val[nnz] = r.alpha; col[nnz] = ISPEC(IS_MOTHER, j); row_ptr[j] = nnz; nnz++;
      val[nnz] = r.beta; col[nnz] = j; nnz++;
      val[nnz] = r.delta; col[nnz] = ISPEC(IS_DR, j); nnz++;
      if (ISPEC(IS_DL, j) != 0) { val[nnz] = r.gamma; col[nnz] = ISPEC(IS_DL, j); nnz++; }
    }
    rhs[j] = RHS(j);
  }
  /* row n-2, src/solverIm-cpu.cpp:147-170: the DR column folds into the diagonal */
  {
    rowc_t r = row_coeffs(n, ispec, c_m, r_a, dX, W, dT, n - 2);
    r.beta = r.beta + r.delta;
    val[nnz] = r.alpha; col[nnz] = ISPEC(IS_MOTHER, n - 2); row_ptr[n - 2] = nnz; nnz++;
    val[nnz] = r.beta; col[nnz] = j; nnz++;
    if (ISPEC(IS_DL, n - 2) != 0) { val[nnz] = r.gamma; col[nnz] = ISPEC(IS_DL, n - 2); nnz++; }
    rhs[n - 2] = RHS(n - 2);
  }
  /* row n-1, src/solverIm-cpu.cpp:172-177 */
  val[nnz] = 1; col[nnz] = n - 1; row_ptr[n - 1] = nnz; nnz++;
  row_ptr[n] = nnz;
#undef RHS
  if (nnz_out) *nnz_out = nnz;
  return NRO_OK;
}

int nro_tree_solve(int n, const int32_t *row_ptr, const int32_t *col, const double *val,
                   const double *b, double *x) {
  double *D = malloc(sizeof(double) * n), *y = malloc(sizeof(double) * n);
  double *aup = malloc(sizeof(double) * n), *adown = malloc(sizeof(double) * n);
  int32_t *up = malloc(sizeof(int32_t) * n);
  int rc = NRO_OK;
  if (!D || !y || !aup || !adown || !up) { rc = NRO_ENOMEM; goto out; }
  for (int j = 0; j < n; j++) {
    D[j] = 0; up[j] = -1; aup[j] = 0; adown[j] = 0; y[j] = b[j];
    for (int p = row_ptr[j]; p < row_ptr[j + 1]; p++) {
      int c = col[p];
      if (c == j) D[j] += val[p];
      else if (c < j) {
        if (up[j] >= 0 && up[j] != c) { rc = NRO_EINVAL; goto out; }
        up[j] = c;
        aup[j] += val[p];
      }
    }
  }
  /* every entry above the diagonal must be the transpose position of a child's up link */
  for (int j = 0; j < n; j++)
    for (int p = row_ptr[j]; p < row_ptr[j + 1]; p++) {
      int c = col[p];
      if (c > j) {
        if (up[c] != j) { rc = NRO_EINVAL; goto out; }
        adown[c] += val[p];
      }
    }
  for (int j = n - 1; j > 0; j--) {
    int u = up[j];
    if (u < 0 || adown[j] == 0) continue;
    double f = adown[j] / D[j];
    D[u] -= f * aup[j];
    y[u] -= f * y[j];
  }
  for (int j = 0; j < n; j++) {
    double s = y[j];
    if (up[j] >= 0) s -= aup[j] * x[up[j]];
    x[j] = s / D[j];
  }
out:
  free(D); free(y); free(aup); free(adown); free(up);
  return rc;
}

static void csr_mv(int n, const int32_t *row_ptr, const int32_t *col, const double *val,
                   const double *x, double *y) {
  for (int i = 0; i < n; i++) {
    double s = 0;
    for (int p = row_ptr[i]; p < row_ptr[i + 1]; p++) s += val[p] * x[col[p]];
    y[i] = s;
  }
}

int nro_gmres(int n, const int32_t *row_ptr, const int32_t *col, const double *val,
              const double *b, double *x, int restart, double tol, int max_it, int *iters_out) {
  int m = restart < n ? restart : n;
  double *Vb = malloc(sizeof(double) * (size_t)n * (m + 1));
  double *H = calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = malloc(sizeof(double) * m), *sn = malloc(sizeof(double) * m);
  double *g = malloc(sizeof(double) * (m + 1)), *yv = malloc(sizeof(double) * m);
  double *w = malloc(sizeof(double) * n);
  int it = 0, rc = NRO_ENOCONV;
  if (!Vb || !H || !cs || !sn || !g || !yv || !w) { rc = NRO_ENOMEM; goto out; }
  for (int i = 0; i < n; i++) x[i] = 0;  /* x0 = 0, src/solverIm-cpu.cpp:200 */
  for (;;) {
    csr_mv(n, row_ptr, col, val, x, w);
    double beta = 0;
    for (int i = 0; i < n; i++) { w[i] = b[i] - w[i]; beta += w[i] * w[i]; }
    beta = sqrt(beta);
    if (beta <= tol) { rc = NRO_OK; goto out; }
    for (int i = 0; i < n; i++) Vb[i] = w[i] / beta;
    memset(g, 0, sizeof(double) * (m + 1));
    g[0] = beta;
    int k, done = 0;
    for (k = 0; k < m; k++) {
      if (it >= max_it) goto out;
      it++;
      double *vk = Vb + (size_t)k * n, *vn = Vb + (size_t)(k + 1) * n;
      csr_mv(n, row_ptr, col, val, vk, vn);
      for (int i = 0; i <= k; i++) {                 /* modified Gram-Schmidt */
        double *vi = Vb + (size_t)i * n, h = 0;
        for (int r = 0; r < n; r++) h += vn[r] * vi[r];
        H[(size_t)i * m + k] = h;
        for (int r = 0; r < n; r++) vn[r] -= h * vi[r];
      }
      double hn = 0;
      for (int r = 0; r < n; r++) hn += vn[r] * vn[r];
      hn = sqrt(hn);
      H[(size_t)(k + 1) * m + k] = hn;
      if (hn != 0) for (int r = 0; r < n; r++) vn[r] /= hn;
      for (int i = 0; i < k; i++) {                   /* apply earlier rotations */
        double a = H[(size_t)i * m + k], c = H[(size_t)(i + 1) * m + k];
        H[(size_t)i * m + k] = cs[i] * a + sn[i] * c;
        H[(size_t)(i + 1) * m + k] = -sn[i] * a + cs[i] * c;
      }
      double a = H[(size_t)k * m + k], c = H[(size_t)(k + 1) * m + k];
      double den = sqrt(a * a + c * c);
      cs[k] = den == 0 ? 1 : a / den;
      sn[k] = den == 0 ? 0 : c / den;
      H[(size_t)k * m + k] = den;
      H[(size_t)(k + 1) * m + k] = 0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      if (fabs(g[k + 1]) <= tol || hn == 0) { k++; done = 1; break; }
    }
    for (int i = k - 1; i >= 0; i--) {               /* back substitution, x += V y */
      double s = g[i];
      for (int l = i + 1; l < k; l++) s -= H[(size_t)i * m + l] * yv[l];
      yv[i] = s / H[(size_t)i * m + i];
    }
    for (int i = 0; i < k; i++) {
      double *vi = Vb + (size_t)i * n;
      for (int r = 0; r < n; r++) x[r] += yv[i] * vi[r];
    }
    if (done) { rc = NRO_OK; goto out; }
  }
out:
  if (iters_out) *iters_out = it;
  free(Vb); free(H); free(cs); free(sn); free(g); free(yv); free(w);
  return rc;
}

/* Crank-Nicolson from the backward-Euler system (not in the reference, which is backward
 * Euler only).  With A = C/dT + L the reference's matrix (C/dT = c_m dX / dT on the
 * diagonal, L the membrane and coupling terms) and b = C/dT V^n + K dX + I its right-hand
 * side, the trapezoidal rule (C/dT + L/2) x = (C/dT - L/2) V^n + K dX + I, doubled, is
 *   (A + C/dT) x = 2 b + C/dT V^n - A V^n
 * on every row except the identity rows (a single unit entry), which stay as they are. */
static void cn_from_be(int n, const int32_t *row_ptr, const int32_t *col, double *val, double *rhs,
                       const double *Vn, const double *c_m, const double *dX, double dT) {
  for (int j = 0; j < n; j++) {
    if (row_ptr[j + 1] - row_ptr[j] == 1) continue;
    const double cdt = c_m[j] * dX[j] / dT;
    double av = 0;
    int kd = -1;
    for (int k = row_ptr[j]; k < row_ptr[j + 1]; k++) {
      av += val[k] * Vn[col[k]];
      if (col[k] == j) kd = k;
    }
    rhs[j] = 2 * rhs[j] + cdt * Vn[j] - av;
    val[kd] += cdt;
  }
}

int nro_implicit_run(int n, const int32_t *ispec, const double *eparam, const double *input_on,
                     int num_hh, const int32_t *hh_elem, double *hparam, double dT, int i_begin,
                     int i_end, double init_time, double end_input, double *V, double *Vother,
                     int linsolve, int record_every, int nprobe, const int32_t *probes,
                     double *trace, int *nrec_out, long long *krylov_iters_out, int scheme) {
  if (n < 4) return NRO_EINVAL;
  size_t cap = (size_t)4 * n + 2;
  double *W = malloc(sizeof(double) * n), *K = malloc(sizeof(double) * n);
  double *zero = calloc(n, sizeof(double)), *val = malloc(sizeof(double) * cap);
  double *bufA = malloc(sizeof(double) * n), *bufB = malloc(sizeof(double) * n);
  double *sol = malloc(sizeof(double) * n);
  int32_t *col = malloc(sizeof(int32_t) * cap), *row_ptr = malloc(sizeof(int32_t) * (n + 1));
  int rc = NRO_OK, nrec = 0;
  long long kit = 0;
  if (!W || !K || !zero || !val || !bufA || !bufB || !sol || !col || !row_ptr) {
    rc = NRO_ENOMEM;
    goto out;
  }
  memcpy(W, eparam + (size_t)EP_W * n, sizeof(double) * n);
  memcpy(K, eparam + (size_t)EP_K * n, sizeof(double) * n);
  double *prevT = bufA, *currT = bufB;
  memcpy(prevT, V, sizeof(double) * n);
  memcpy(currT, Vother, sizeof(double) * n);
  for (int it = i_begin; it < i_end; it++) {
    double time_run = it * dT;
    const double *input = ((time_run >= init_time) && (time_run <= end_input)) ? input_on : zero;
    hh_update(num_hh, hh_elem, hparam, prevT, dT, W, K);
    int nnz;
    rc = nro_implicit_matrix(n, ispec, eparam, W, K, input, dT, prevT, row_ptr, col, val, currT, &nnz);
    if (rc) goto out;
    if (scheme == 1)
      cn_from_be(n, row_ptr, col, val, currT, prevT, eparam + (size_t)EP_CM * n,
                 eparam + (size_t)EP_DX * n, dT);
    if (linsolve == 0) {
      rc = nro_tree_solve(n, row_ptr, col, val, currT, currT);
    } else {
      int its = 0;
      rc = nro_gmres(n, row_ptr, col, val, currT, sol, 150, 1e-14, n, &its);
      kit += its;
      if (rc == NRO_ENOCONV && linsolve == 2) rc = NRO_OK;
      memcpy(currT, sol, sizeof(double) * n);
    }
    if (rc) goto out;
    double *flip = currT; currT = prevT; prevT = flip;
    if (record_every > 0 && (it % record_every) == 0 && trace) {
      double *row = trace + (size_t)nrec * (nprobe + 1);
      row[0] = it;
      for (int p = 0; p < nprobe; p++) row[p + 1] = prevT[probes[p]];
      nrec++;
    }
  }
  memcpy(V, prevT, sizeof(double) * n);
  memcpy(Vother, currT, sizeof(double) * n);
out:
  if (nrec_out) *nrec_out = nrec;
  if (krylov_iters_out) *krylov_iters_out = kit;
  free(W); free(K); free(zero); free(val); free(bufA); free(bufB); free(sol); free(col); free(row_ptr);
  return rc;
}
