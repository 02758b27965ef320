/*
 * CPU oracle: FP64 Felsenstein pruning arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY. This file restates, from the published method, the
 * libpll arithmetic that NetRAX calls but does not vendor (the libs/raxml-ng
 * submodule is empty in the reference tree):
 *
 *  - pll_update_partials_single, called at
 *    src/likelihood/ImprovedLoglikelihood.cpp:145 and :185:
 *      parent[n][r][i] = (sum_j Pl[r][i][j] L[n][r][j]) * (sum_j Pr[r][i][j] R[n][r][j])
 *    with per-site scaling: when every entry of a site (all rates, all states)
 *    is below 2^-256 the site is multiplied by 2^256 and its scale counter,
 *    which starts as left + right counters, is incremented.
 *    A missing right child is the all-ones "fake" CLV with the zero-length
 *    (identity) P-matrix (src/likelihood/Operation.cpp:19-33,
 *    src/RaxmlWrapper.cpp:156-187), so its factor is exactly 1.
 *  - pll_compute_root_loglikelihood, called at ImprovedLoglikelihood.cpp:450:
 *      logl = sum_n w_n [ log(sum_r rw_r sum_i pi_i clv[n][r][i])
 *                         + scaler_n * log(2^-256) ]
 *    (with invariant sites the site likelihood is (1 - pinv) times that
 *    mixture plus pinv times the invariant state's frequency)
 *
 * The same code is the timed CPU baseline (OpenMP over sites).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#define ORACLE_SCALE_THRESHOLD 0x1p-256
#define ORACLE_SCALE_FACTOR 0x1p+256

/* left / right: CLV [n][R][S] or NULL; a NULL right is the fake all-ones child.
 * left_scaler / right_scaler: [n] or NULL (tips have none).
 * pl / pr: [R][S][S] row-major P-matrices. */
void oracle_update_partial(int64_t n, int R, int S, double *parent,
                           uint32_t *parent_scaler, const double *left,
                           const uint32_t *left_scaler, const double *pl,
                           const double *right, const uint32_t *right_scaler,
                           const double *pr) {
  const int64_t span = (int64_t)R * S;
#pragma omp parallel for schedule(static) if (n > 4096)
  for (int64_t s = 0; s < n; ++s) {
    double *pc = parent + s * span;
    const double *lc = left + s * span;
    const double *rc = right ? right + s * span : NULL;
    int all_small = 1;
    for (int r = 0; r < R; ++r) {
      const double *lm = pl + (int64_t)r * S * S;
      const double *rm = pr ? pr + (int64_t)r * S * S : NULL;
      for (int i = 0; i < S; ++i) {
        double ta = 0.0, tb = 1.0;
        for (int j = 0; j < S; ++j) ta += lm[i * S + j] * lc[r * S + j];
        if (rc) {
          tb = 0.0;
          for (int j = 0; j < S; ++j) tb += rm[i * S + j] * rc[r * S + j];
        }
        const double v = ta * tb;
        pc[r * S + i] = v;
        all_small = all_small && (v < ORACLE_SCALE_THRESHOLD);
      }
    }
    uint32_t sc = (left_scaler ? left_scaler[s] : 0) +
                  (right_scaler ? right_scaler[s] : 0);
    if (all_small) {
      for (int64_t k = 0; k < span; ++k) pc[k] *= ORACLE_SCALE_FACTOR;
      sc += 1;
    }
    if (parent_scaler) parent_scaler[s] = sc;
  }
}

/* Returns the weighted root log-likelihood; persite (optional) receives the
 * unweighted per-site values. With invariant sites (+I) the site likelihood
 * is gamma_frac * (the Gamma mixture above) + inv_term[s]; inv_term NULL
 * (and gamma_frac 1) without. */
double oracle_root_logl(int64_t n, int R, int S, const double *clv,
                        const uint32_t *scaler, const double *freqs,
                        const double *rate_weights, const double *weights,
                        double *persite, double gamma_frac, const double *inv_term) {
  const int64_t span = (int64_t)R * S;
  const double log_thr = log(ORACLE_SCALE_THRESHOLD);
  double total = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : total) if (n > 4096)
  for (int64_t s = 0; s < n; ++s) {
    const double *c = clv + s * span;
    double site = 0.0;
    for (int r = 0; r < R; ++r) {
      double t = 0.0;
      for (int i = 0; i < S; ++i) t += freqs[i] * c[r * S + i];
      site += rate_weights[r] * t;
    }
    double l = log(gamma_frac * site);
    if (scaler) l += (double)scaler[s] * log_thr;
    if (inv_term && inv_term[s] > 0.0) { /* log(exp(l) + inv), without overflow */
      const double b = log(inv_term[s]);
      l = l > b ? l + log1p(exp(b - l)) : b + log1p(exp(l - b));
    }
    if (persite) persite[s] = l;
    total += weights[s] * l;
  }
  return total;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
