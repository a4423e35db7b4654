/*
 * boss_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * A plain-C restatement of theboss's permanent hot path, used only to check results
 * by tests/, by __graft_entry__.smoke() and by bench.py's CPU baseline leg.  The
 * product (theboss_gb300/) never links, imports or calls anything in this file.
 *
 * Two arithmetic flavours:
 *   - FP64 functions (oracle_*) follow the reference's Python loops operation by
 *     operation (same Guan-code order, same complex multiply formula, no FMA
 *     contraction: build with -ffp-contract=off), so they agree with the reference
 *     to a few ULP.  Every function names the reference file:line it follows.
 *   - double-double functions (oracle_dd_*) evaluate the same formulas in ~106-bit
 *     arithmetic (Knuth TwoSum, FMA-based TwoProd) and serve as the "true value"
 *     against which every FP64 implementation's error is stated.
 *
 * Matrices are complex128, row-major, U[out_mode][in_mode] (two doubles per entry),
 * exactly as theboss indexes them (ryser_permanent_calculator.py:62-64).
 * Occupations are int arrays of length `len` (len <= m).
 * Return codes: 0 ok, 1 size mismatch (the reference raises AttributeError,
 * bs_permanent_calculator_base.py:179-180), 2 size limit exceeded.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAX_MODES 256
#define ORACLE_MAX_PHOTONS 64

typedef struct { double re, im; } cpx;

static inline cpx c_make(double re, double im) { cpx z; z.re = re; z.im = im; return z; }
static inline cpx c_add(cpx a, cpx b) { return c_make(a.re + b.re, a.im + b.im); }
static inline cpx c_sub(cpx a, cpx b) { return c_make(a.re - b.re, a.im - b.im); }
/* numpy's complex128 multiply: (ar*br - ai*bi, ar*bi + ai*br). */
static inline cpx c_mul(cpx a, cpx b) {
  return c_make(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
/* A Python/numpy real scalar times a complex128 promotes the scalar to (s + 0j). */
static inline cpx c_rmul(double s, cpx z) { return c_mul(c_make(s, 0.0), z); }
static inline cpx c_mulr(cpx z, double s) { return c_mul(z, c_make(s, 0.0)); }
static inline cpx U_at(const double* U, int m, int row, int col) {
  return c_make(U[2 * ((size_t)row * m + col)], U[2 * ((size_t)row * m + col) + 1]);
}

/* numpy's complex power for a small non-negative integer exponent: special cases
 * 1, 2, 3, then binary exponentiation (numpy npymath npy_cpow). */
static cpx c_powi(cpx a, long n) {
  if (n == 1) return a;
  if (n == 2) return c_mul(a, a);
  if (n == 3) return c_mul(a, c_mul(a, a));
  cpx aa = c_make(1.0, 0.0), p = a;
  long mask = 1;
  for (;;) {
    if (n & mask) aa = c_mul(aa, p);
    mask <<= 1;
    if (n < mask || mask <= 0) break;
    p = c_mul(p, p);
  }
  return aa;
}

/* ---------------------------------------------------------------------------
 * Guan code (reflected mixed-radix Gray code) over r in prod_i [0, S_i].
 * Follows bs_permanent_calculator_base.py:115-149 (and the identical copy in
 * bs_submatrices_permanent_calculator_base.py:99-133).
 * ------------------------------------------------------------------------- */
typedef struct {
  int len;
  int r[ORACLE_MAX_MODES];
  int u[ORACLE_MAX_MODES];
  int lim[ORACLE_MAX_MODES];
  int idx;
  int last;
} guan_t;

static void guan_init(guan_t* g, const int* S, int len) {
  g->len = len;
  for (int i = 0; i < len; ++i) { g->r[i] = 0; g->u[i] = 1; g->lim[i] = S[i]; }
  g->idx = 0; g->last = 0;
}

/* Advances to the next code; returns 0 when the sequence is exhausted. */
static int guan_next(guan_t* g) {
  g->idx = 0;
  int k = g->r[0] + g->u[0];
  while (k > g->lim[g->idx] || k < 0) {
    g->u[g->idx] = -g->u[g->idx];
    g->idx += 1;
    if (g->idx == g->len) return 0;
    k = g->r[g->idx] + g->u[g->idx];
  }
  g->last = g->r[g->idx];
  g->r[g->idx] = k;
  return 1;
}

/* bs_permanent_calculator_base.py:151-164 */
static double guan_binom_update(const guan_t* g, const int* S, double binom) {
  int i = g->idx;
  if (g->r[i] > g->last) return binom * ((double)(S[i] - g->last) / (double)g->r[i]);
  return binom * ((double)g->last / (double)(S[i] - g->r[i]));
}

/* Exposed for tests: writes the whole Guan sequence of updated indices and the
 * r vectors (count x len) into caller buffers; returns the number of codes. */
long oracle_guan_sequence(const int* S, int len, int* idx_out, int* r_out, long cap) {
  if (len <= 0 || len > ORACLE_MAX_MODES) return -1;
  guan_t g; guan_init(&g, S, len);
  long c = 0;
  if (c < cap) { idx_out[c] = -1; memcpy(r_out + c * len, g.r, sizeof(int) * len); }
  ++c;
  while (guan_next(&g)) {
    if (c < cap) { idx_out[c] = g.idx; memcpy(r_out + c * len, g.r, sizeof(int) * len); }
    ++c;
  }
  return c;
}

static int sum_int(const int* v, int len) { int s = 0; for (int i = 0; i < len; ++i) s += v[i]; return s; }

/* bs_permanent_calculator_base.py:61-72 */
static int check_sizes(int m, int len_in, int len_out) {
  return (len_in == len_out && len_out <= m) ? 0 : 1;
}

/* bs_permanent_calculator_base.py:200-209: permanent += (mult*binom) * prod_j sums_j^T_j */
static cpx addend(double init, const cpx* sums, const int* cols, int ncols, const int* T) {
  cpx acc = c_make(init, 0.0);
  for (int c = 0; c < ncols; ++c) acc = c_mul(acc, c_powi(sums[c], T[cols[c]]));
  return acc;
}

/* ---------------------------------------------------------------------------
 * Ryser with Guan codes: ryser_permanent_calculator.py:45-64 driven by
 * bs_permanent_calculator_base.py:103-113,166-209.
 * ------------------------------------------------------------------------- */
int oracle_perm_ryser(const double* U, int m, const int* S, const int* T, int len, double* out) {
  if (check_sizes(m, len, len)) return 1;
  if (len <= 0 || len > ORACLE_MAX_MODES) return 2;
  int cols[ORACLE_MAX_MODES], ncols = 0;
  for (int j = 0; j < len; ++j) if (T[j] != 0) cols[ncols++] = j;
  cpx sums[ORACLE_MAX_MODES];
  for (int c = 0; c < ncols; ++c) sums[c] = c_make(0.0, 0.0);
  double mult = (sum_int(S, len) % 2) ? -1.0 : 1.0;
  double binom = 1.0;
  guan_t g; guan_init(&g, S, len);
  cpx perm = addend(mult * binom, sums, cols, ncols, T);
  while (guan_next(&g)) {
    mult = -mult;
    int d = g.r[g.idx] - g.last;
    for (int c = 0; c < ncols; ++c) sums[c] = c_add(sums[c], c_rmul((double)d, U_at(U, m, cols[c], g.idx)));
    binom = guan_binom_update(&g, S, binom);
    perm = c_add(perm, addend(mult * binom, sums, cols, ncols, T));
  }
  out[0] = perm.re; out[1] = perm.im;
  return 0;
}

/* ---------------------------------------------------------------------------
 * Chin-Huh with Guan codes: chin_huh_permanent_calculator.py:38-59 driven by
 * bs_permanent_calculator_base.py:166-209.
 * ------------------------------------------------------------------------- */
int oracle_perm_chin_huh(const double* U, int m, const int* S, const int* T, int len, double* out) {
  if (check_sizes(m, len, len)) return 1;
  if (len <= 0 || len > ORACLE_MAX_MODES) return 2;
  int cols[ORACLE_MAX_MODES], ncols = 0;
  for (int j = 0; j < len; ++j) if (T[j] != 0) cols[ncols++] = j;
  cpx sums[ORACLE_MAX_MODES];
  for (int c = 0; c < ncols; ++c) {
    sums[c] = c_make(0.0, 0.0);
    for (int j = 0; j < len; ++j) sums[c] = c_add(sums[c], c_rmul((double)S[j], U_at(U, m, cols[c], j)));
  }
  double mult = 1.0 / pow(2.0, (double)sum_int(S, len));
  double binom = 1.0;
  guan_t g; guan_init(&g, S, len);
  cpx perm = addend(mult * binom, sums, cols, ncols, T);
  while (guan_next(&g)) {
    mult = -mult;
    int d = g.r[g.idx] - g.last;
    for (int c = 0; c < ncols; ++c)
      sums[c] = c_sub(sums[c], c_rmul((double)(2 * d), U_at(U, m, cols[c], g.idx)));
    binom = guan_binom_update(&g, S, binom);
    perm = c_add(perm, addend(mult * binom, sums, cols, ncols, T));
  }
  out[0] = perm.re; out[1] = perm.im;
  return 0;
}

/* Effective scattering matrix: boson_sampling_utilities.py:595-626.  Column i of U
 * repeated S_i times, then row j repeated T_j times.  Returns rows (=sum T); cols
 * = sum S written to *ncols_out. */
static int effective_matrix(const double* U, int m, const int* S, const int* T, int len, cpx* M,
                            int* ncols_out) {
  int colmode[ORACLE_MAX_PHOTONS], nc = 0, rowmode[ORACLE_MAX_PHOTONS], nr = 0;
  for (int i = 0; i < len; ++i)
    for (int k = 0; k < S[i]; ++k) { if (nc >= ORACLE_MAX_PHOTONS) return -1; colmode[nc++] = i; }
  for (int j = 0; j < len; ++j)
    for (int k = 0; k < T[j]; ++k) { if (nr >= ORACLE_MAX_PHOTONS) return -1; rowmode[nr++] = j; }
  for (int a = 0; a < nr; ++a)
    for (int b = 0; b < nc; ++b) M[a * nc + b] = U_at(U, m, rowmode[a], colmode[b]);
  *ncols_out = nc;
  return nr;
}

/* ---------------------------------------------------------------------------
 * Glynn with Gray codes: glynn_gray_permanent_calculator.py:41-84.  The flip
 * sequence is the binary-reflected Gray code over n-1 rows (step t flips bit
 * ctz(t)); the guancodes package that supplies the reference's sequence is not
 * available, so only the value (not the summation order) is pinned.
 * Rows must equal columns (sum S == sum T); returns 1 otherwise.
 * ------------------------------------------------------------------------- */
int oracle_perm_glynn(const double* U, int m, const int* S, const int* T, int len, double* out) {
  if (len > m) return 1;
  int sS = sum_int(S, len), sT = sum_int(T, len);
  if (sS == 0 || sT == 0) { out[0] = 1.0; out[1] = 0.0; return 0; }
  if (sS != sT) return 1;
  if (sS > ORACLE_MAX_PHOTONS) return 2;
  static __thread cpx M[ORACLE_MAX_PHOTONS * ORACLE_MAX_PHOTONS];
  int nc;
  int n = effective_matrix(U, m, S, T, len, M, &nc);
  if (n < 0) return 2;
  int delta[ORACLE_MAX_PHOTONS];
  cpx sums[ORACLE_MAX_PHOTONS];
  for (int i = 0; i < n; ++i) delta[i] = 1;
  for (int j = 0; j < n; ++j) {
    sums[j] = c_make(0.0, 0.0);
    for (int i = 0; i < n; ++i) sums[j] = c_add(sums[j], c_rmul((double)delta[i], M[i * n + j]));
  }
  double mult = 1.0;
  cpx prod = c_make(1.0, 0.0);
  for (int j = 0; j < n; ++j) prod = c_mul(prod, sums[j]);
  cpx perm = c_rmul(mult, prod);
  uint64_t steps = (n >= 1) ? ((uint64_t)1 << (n - 1)) : 1;
  for (uint64_t t = 1; t < steps; ++t) {
    int i = __builtin_ctzll(t);
    mult = -mult;
    delta[i] = -delta[i];
    for (int j = 0; j < n; ++j) sums[j] = c_add(sums[j], c_rmul((double)(2 * delta[i]), M[i * n + j]));
    prod = c_make(1.0, 0.0);
    for (int j = 0; j < n; ++j) prod = c_mul(prod, sums[j]);
    perm = c_add(perm, c_rmul(mult, prod));
  }
  double scale = ldexp(1.0, n - 1);
  out[0] = perm.re / scale; out[1] = perm.im / scale;
  return 0;
}

/* Brute-force row expansion: classic_permanent_calculator.py:27-67 (tiny n only). */
static cpx classic_rec(const cpx* M, int n, int col, uint64_t used, cpx prod) {
  if (col == n) return prod;
  cpx res = c_make(0.0, 0.0);
  for (int row = 0; row < n; ++row)
    if (!(used & ((uint64_t)1 << row)))
      res = c_add(res, classic_rec(M, n, col + 1, used | ((uint64_t)1 << row), c_mul(prod, M[row * n + col])));
  return res;
}
int oracle_perm_classic(const double* U, int m, const int* S, const int* T, int len, double* out) {
  if (len > m) return 1;
  int sS = sum_int(S, len), sT = sum_int(T, len);
  if (sS == 0) { out[0] = (sT == 0) ? 1.0 : 0.0; out[1] = 0.0; return 0; }
  if (sS != sT) return 1;
  if (sS > 12) return 2;
  cpx M[144];
  int nc;
  int n = effective_matrix(U, m, S, T, len, M, &nc);
  cpx r = classic_rec(M, n, 0, 0, c_make(1.0, 0.0));
  out[0] = r.re; out[1] = r.im;
  return 0;
}

/* ---------------------------------------------------------------------------
 * A batch of permanents: row k of S and of T (len modes each) with the
 * calculator named by variant (0 Ryser, 1 Chin-Huh, 2 Glynn, 3 classic), the
 * values of the functions above, one call for a whole sampler stream.
 * ------------------------------------------------------------------------- */
int oracle_perm_batch(const double* U, int m, const int* S, const int* T, int len, int count, int variant,
                      double* out) {
  for (int k = 0; k < count; ++k) {
    const int* s = S + (size_t)k * len;
    const int* t = T + (size_t)k * len;
    double* o = out + 2 * (size_t)k;
    int rc;
    switch (variant) {
      case 0: rc = oracle_perm_ryser(U, m, s, t, len, o); break;
      case 1: rc = oracle_perm_chin_huh(U, m, s, t, len, o); break;
      case 2: rc = oracle_perm_glynn(U, m, s, t, len, o); break;
      case 3: rc = oracle_perm_classic(U, m, s, t, len, o); break;
      default: return 4;
    }
    if (rc) return rc;
  }
  return 0;
}

/* ---------------------------------------------------------------------------
 * All-minors ("submatrices") permanents, Ryser flavour:
 * bs_cc_ryser_submatrices_permanent_calculator.py:73-119 driven by
 * bs_submatrices_permanent_calculator_base.py:150-189.
 * out: len complex values (2*len doubles).
 * ------------------------------------------------------------------------- */
int oracle_submatrices_ryser(const double* U, int m, const int* S, const int* T, int len, double* out) {
  if (len <= 0 || len > ORACLE_MAX_MODES || len > m) return 2;
  int sS = sum_int(S, len);
  if (sS == 1) {  /* bs_submatrices_permanent_calculator_base.py:157-158 */
    for (int i = 0; i < len; ++i) { out[2 * i] = (double)S[i]; out[2 * i + 1] = 0.0; }
    return 0;
  }
  cpx perms[ORACLE_MAX_MODES];
  for (int i = 0; i < len; ++i) perms[i] = c_make(0.0, 0.0);
  int cols[ORACLE_MAX_MODES], ncols = 0;
  for (int j = 0; j < len; ++j) if (T[j] != 0) cols[ncols++] = j;
  cpx sums[ORACLE_MAX_MODES];
  for (int c = 0; c < ncols; ++c) sums[c] = c_make(0.0, 0.0);
  double mult = (sum_int(T, len) % 2) ? -1.0 : 1.0;
  double binom = 1.0;
  guan_t g; guan_init(&g, S, len);
  while (guan_next(&g)) {
    mult = -mult;
    binom = guan_binom_update(&g, S, binom);
    int d = g.r[g.idx] - g.last;
    cpx prod = c_make(1.0, 0.0);
    for (int c = 0; c < ncols; ++c) {
      sums[c] = c_add(sums[c], c_rmul((double)d, U_at(U, m, cols[c], g.idx)));
      prod = c_mul(prod, c_powi(sums[c], T[cols[c]]));
    }
    prod = c_mulr(prod, mult);
    for (int i = 0; i < len; ++i) {
      if (S[i] == 0 || g.r[i] == S[i]) continue;
      double ub = binom;
      ub /= ((double)S[i] / (double)(S[i] - g.r[i]));
      perms[i] = c_add(perms[i], c_mulr(prod, ub));
    }
  }
  for (int i = 0; i < len; ++i) { out[2 * i] = perms[i].re; out[2 * i + 1] = perms[i].im; }
  return 0;
}

/* All-minors, Chin-Huh flavour: bs_cc_ch_submatrices_permanent_calculator.py:51-105. */
static void ch_sub_update(const double* U, int m, const int* S, const int* T, int len, const guan_t* g,
                          const cpx* sums, const int* cols, int ncols, double mult, double binom, cpx* perms) {
  for (int i = 0; i < len; ++i) {
    if (S[i] == 0 || S[i] == g->r[i]) continue;
    cpx upd[ORACLE_MAX_MODES];
    for (int c = 0; c < ncols; ++c) upd[c] = c_sub(sums[c], U_at(U, m, cols[c], i));
    double ub = binom / ((double)S[i] / (double)(S[i] - g->r[i]));
    perms[i] = c_add(perms[i], addend(mult * ub, upd, cols, ncols, T));
  }
}
int oracle_submatrices_chin_huh(const double* U, int m, const int* S, const int* T, int len, double* out) {
  if (len <= 0 || len > ORACLE_MAX_MODES || len > m) return 2;
  int sS = sum_int(S, len);
  if (sS == 1) {
    for (int i = 0; i < len; ++i) { out[2 * i] = (double)S[i]; out[2 * i + 1] = 0.0; }
    return 0;
  }
  cpx perms[ORACLE_MAX_MODES];
  for (int i = 0; i < len; ++i) perms[i] = c_make(0.0, 0.0);
  int cols[ORACLE_MAX_MODES], ncols = 0;
  for (int j = 0; j < len; ++j) if (T[j] != 0) cols[ncols++] = j;
  double mult = 1.0 / pow(2.0, (double)(sS - 1));
  double binom = 1.0;
  cpx sums[ORACLE_MAX_MODES];
  for (int c = 0; c < ncols; ++c) {
    sums[c] = c_make(0.0, 0.0);
    for (int j = 0; j < len; ++j) sums[c] = c_add(sums[c], c_rmul((double)S[j], U_at(U, m, cols[c], j)));
  }
  guan_t g; guan_init(&g, S, len);
  ch_sub_update(U, m, S, T, len, &g, sums, cols, ncols, mult, binom, perms);
  while (guan_next(&g)) {
    mult = -mult;
    binom = guan_binom_update(&g, S, binom);
    int d = g.r[g.idx] - g.last;
    for (int c = 0; c < ncols; ++c)
      sums[c] = c_sub(sums[c], c_rmul((double)(2 * d), U_at(U, m, cols[c], g.idx)));
    ch_sub_update(U, m, S, T, len, &g, sums, cols, ncols, mult, binom, perms);
  }
  for (int i = 0; i < len; ++i) { out[2 * i] = perms[i].re; out[2 * i + 1] = perms[i].im; }
  return 0;
}

/* ---------------------------------------------------------------------------
 * One C&C-B step: generalized_cliffords_b_simulation_strategy.py:69-92 (the
 * Laplace expansion over the all-minors, |.|^2, normalisation by Python's
 * sequential sum) followed by numpy.random.choice's cdf/searchsorted rule
 * (cumsum, divide by the last entry, first index whose cdf exceeds u).
 * S, T: length m.  pmf_out: m doubles (normalised).  Returns the sampled mode,
 * or -1 when the pmf cannot be normalised (the reference raises ValueError).
 * ------------------------------------------------------------------------- */
int oracle_gccb_step(const double* U, int m, const int* S, const int* T, double u, double* pmf_out) {
  double sub[2 * ORACLE_MAX_MODES];
  if (oracle_submatrices_ryser(U, m, S, T, m, sub)) return -2;
  double total = 0.0;
  for (int j = 0; j < m; ++j) {
    cpx p = c_make(0.0, 0.0);
    for (int i = 0; i < m; ++i) {
      cpx pa = c_rmul((double)S[i], c_make(sub[2 * i], sub[2 * i + 1]));
      pa = c_mul(pa, U_at(U, m, j, i));
      p = c_add(p, pa);
    }
    double h = hypot(p.re, p.im);
    pmf_out[j] = pow(h, 2.0);
    total += pmf_out[j];
  }
  if (!(total > 0.0) || !isfinite(total)) return -1;
  for (int j = 0; j < m; ++j) pmf_out[j] = pmf_out[j] / total;
  double cdf[ORACLE_MAX_MODES];
  double acc = 0.0;
  for (int j = 0; j < m; ++j) { acc += pmf_out[j]; cdf[j] = acc; }
  double last = cdf[m - 1];
  int idx = 0;
  for (int j = 0; j < m; ++j) { cdf[j] /= last; if (cdf[j] <= u) idx = j + 1; }
  if (idx > m - 1) idx = m - 1;
  return idx;
}

/* Threads of the OpenMP loops below (n >= 1), whatever OMP_NUM_THREADS the process
 * inherited; returns the count now in force (1 without OpenMP). */
int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n >= 1) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

/* A whole batch of GCC-B samples from a pre-drawn random stream.  For sample s,
 * steps k = 0..L[s]-1: add_mode[s*maxL+k] is the input mode whose particle the
 * reference's randint pops (generalized_cliffords_b_simulation_strategy.py:102-105)
 * and uniform[s*maxL+k] the random_sample() numpy.random.choice consumes (:107-110).
 * samples_out: n_samples x m output occupations.  Samples are independent, so the
 * loop over samples runs on all OpenMP threads.  Returns 0, or -1 if any pmf failed. */
int oracle_gccb_run(const double* U, int m, int n_samples, int maxL, const int* L, const int* add_mode,
                    const double* uniform, int64_t* samples_out) {
  if (m > ORACLE_MAX_MODES) return 2;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
  for (int s = 0; s < n_samples; ++s) {
    int S[ORACLE_MAX_MODES], T[ORACLE_MAX_MODES];
    double pmf[ORACLE_MAX_MODES];
    for (int j = 0; j < m; ++j) { S[j] = 0; T[j] = 0; }
    for (int k = 0; k < L[s]; ++k) {
      S[add_mode[(size_t)s * maxL + k]] += 1;
      int o = oracle_gccb_step(U, m, S, T, uniform[(size_t)s * maxL + k], pmf);
      if (o < 0) { bad = 1; break; }
      T[o] += 1;
    }
    for (int j = 0; j < m; ++j) samples_out[(size_t)s * m + j] = T[j];
  }
  return bad ? -1 : 0;
}

/* ===========================================================================
 * double-double arithmetic (Dekker/Knuth error-free transforms; Bailey's
 * double-double add/mul).  Used for the high-precision oracle only.
 * ========================================================================= */
typedef struct { double hi, lo; } dd;
static inline dd dd_make(double h, double l) { dd r; r.hi = h; r.lo = l; return r; }
static inline dd two_sum(double a, double b) {
  double s = a + b, bb = s - a, e = (a - (s - bb)) + (b - bb);
  return dd_make(s, e);
}
static inline dd quick_two_sum(double a, double b) { double s = a + b; return dd_make(s, b - (s - a)); }
static inline dd two_prod(double a, double b) { double p = a * b; return dd_make(p, fma(a, b, -p)); }
static inline dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
  s.lo += t.hi; s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo; return quick_two_sum(s.hi, s.lo);
}
static inline dd dd_neg(dd a) { return dd_make(-a.hi, -a.lo); }
static inline dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}
static inline dd dd_muld(dd a, double b) {
  dd p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return quick_two_sum(p.hi, p.lo);
}
typedef struct { dd re, im; } cdd;
static inline cdd cdd_add(cdd a, cdd b) { cdd r; r.re = dd_add(a.re, b.re); r.im = dd_add(a.im, b.im); return r; }
static inline cdd cdd_mul(cdd a, cdd b) {
  cdd r;
  r.re = dd_add(dd_mul(a.re, b.re), dd_neg(dd_mul(a.im, b.im)));
  r.im = dd_add(dd_mul(a.re, b.im), dd_mul(a.im, b.re));
  return r;
}
static inline cdd cdd_muld(cdd a, double s) { cdd r; r.re = dd_muld(a.re, s); r.im = dd_muld(a.im, s); return r; }
static inline cdd cdd_from(double re, double im) { cdd r; r.re = dd_make(re, 0.0); r.im = dd_make(im, 0.0); return r; }
static inline cdd cdd_zero(void) { return cdd_from(0.0, 0.0); }

static double binom_exact(int n, int k) {
  if (k < 0 || k > n) return 0.0;
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (double)(n - k + i) / (double)i;
  return nearbyint(r);
}

/* Mixed-radix reflected Gray code decoded in closed form: digit i of code number t
 * (bases b_i = S_i + 1, digit 0 fastest) is d_i when the number of completed cycles
 * of digits 0..i is even, S_i - d_i otherwise. */
static void guan_decode(uint64_t t, const int* S, int len, int* r) {
  for (int i = 0; i < len; ++i) {
    uint64_t b = (uint64_t)S[i] + 1;
    uint64_t d = t % b, q = t / b;
    r[i] = (q & 1) ? (int)(S[i] - d) : (int)d;
    t = q;
  }
}

/* Glynn / Chin-Huh value in double-double:
 *   perm = 2^-n sum_{r<=S} (-1)^|r| prod_i C(S_i,r_i) prod_j (sum_i (S_i-2r_i) U[j][i])^T_j
 * (chin_huh_permanent_calculator.py:38-59 formula), chunked over code ranges so it
 * parallelises with OpenMP.  Each chunk recomputes its sums from the decoded code. */
int oracle_dd_perm(const double* U, int m, const int* S, const int* T, int len, double* out_hi_lo) {
  if (len <= 0 || len > m || len > ORACLE_MAX_MODES) return 1;
  int sS = sum_int(S, len), sT = sum_int(T, len);
  if (sS == 0) { out_hi_lo[0] = (sT == 0) ? 1.0 : 0.0; out_hi_lo[1] = out_hi_lo[2] = out_hi_lo[3] = 0.0; return 0; }
  if (sS != sT) return 1;
  int dig[ORACLE_MAX_MODES], nd = 0, cols[ORACLE_MAX_MODES], nc = 0;
  for (int i = 0; i < len; ++i) if (S[i] > 0) dig[nd++] = i;
  for (int j = 0; j < len; ++j) if (T[j] > 0) cols[nc++] = j;
  int Sd[ORACLE_MAX_MODES];
  uint64_t total = 1;
  for (int a = 0; a < nd; ++a) { Sd[a] = S[dig[a]]; total *= (uint64_t)(Sd[a] + 1); }
  uint64_t chunk = 1 << 12;
  uint64_t nchunks = (total + chunk - 1) / chunk;
  dd acc_re = dd_make(0, 0), acc_im = dd_make(0, 0);
#pragma omp parallel
  {
    dd lre = dd_make(0, 0), lim = dd_make(0, 0);
#pragma omp for schedule(dynamic, 1)
    for (uint64_t c = 0; c < nchunks; ++c) {
      uint64_t t0 = c * chunk, t1 = t0 + chunk; if (t1 > total) t1 = total;
      int r[ORACLE_MAX_MODES];
      cdd sums[ORACLE_MAX_MODES];
      for (uint64_t t = t0; t < t1; ++t) {
        guan_decode(t, Sd, nd, r);
        double w = 1.0; int parity = 0;
        for (int a = 0; a < nd; ++a) { w *= binom_exact(Sd[a], r[a]); parity += r[a]; }
        for (int c2 = 0; c2 < nc; ++c2) {
          sums[c2] = cdd_zero();
          for (int a = 0; a < nd; ++a) {
            cpx z = U_at(U, m, cols[c2], dig[a]);
            sums[c2] = cdd_add(sums[c2], cdd_muld(cdd_from(z.re, z.im), (double)(Sd[a] - 2 * r[a])));
          }
        }
        cdd prod = cdd_from(w * ((parity & 1) ? -1.0 : 1.0), 0.0);
        for (int c2 = 0; c2 < nc; ++c2)
          for (int p = 0; p < T[cols[c2]]; ++p) prod = cdd_mul(prod, sums[c2]);
        lre = dd_add(lre, prod.re); lim = dd_add(lim, prod.im);
      }
    }
#pragma omp critical
    { acc_re = dd_add(acc_re, lre); acc_im = dd_add(acc_im, lim); }
  }
  double sc = ldexp(1.0, -sS);
  out_hi_lo[0] = acc_re.hi * sc; out_hi_lo[1] = acc_re.lo * sc;
  out_hi_lo[2] = acc_im.hi * sc; out_hi_lo[3] = acc_im.lo * sc;
  return 0;
}

/* All-minors in double-double: minor i = perm(U[T, S - e_i]) (0 where S_i = 0).
 * out: len complex (hi parts then lo parts: out[4i..4i+3] = re.hi, re.lo, im.hi, im.lo). */
int oracle_dd_submatrices(const double* U, int m, const int* S, const int* T, int len, double* out) {
  int Sm[ORACLE_MAX_MODES];
  if (len <= 0 || len > ORACLE_MAX_MODES) return 1;
  for (int i = 0; i < len; ++i) Sm[i] = S[i];
  for (int i = 0; i < len; ++i) {
    if (S[i] == 0) { out[4 * i] = out[4 * i + 1] = out[4 * i + 2] = out[4 * i + 3] = 0.0; continue; }
    Sm[i] -= 1;
    int rc = oracle_dd_perm(U, m, Sm, T, len, out + 4 * i);
    Sm[i] += 1;
    if (rc) return rc;
  }
  return 0;
}
