// Substitution-model math on the host (FP64): GTR eigensystem and discrete
// Gamma rates. These replace the libpll routines the reference reaches through
// pllmod_treeinfo_update_prob_matrices (src/likelihood/ImprovedLoglikelihood.cpp:661)
// and the mean-Gamma category setup (src/RaxmlWrapper.cpp:621).
//  - Q_ij = exch_ij * pi_j, rows sum to zero, scaled to one expected
//    substitution per unit time; eigensystem of the symmetric
//    Pi^1/2 Q Pi^-1/2 by cyclic Jacobi rotations (Golub & Van Loan, 8.5).
//  - Yang (1994) mean rates of equal-probability Gamma categories, with the
//    regularized incomplete gamma function by its power series / Legendre
//    continued fraction (Abramowitz & Stegun 6.5.29, 6.5.31) and quantiles by
//    safeguarded Newton iteration.
#include <cmath>

#include "../../include/netlk.h"
#include "internal.hpp"

namespace netlk {

static void jacobi_eigen(int n, std::vector<double> &A, std::vector<double> &V, std::vector<double> &d) {
  V.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        double app = A[p * n + p], aqq = A[q * n + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- A J
          double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // A <- J^T A
          double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
    }
  }
  d.resize(n);
  for (int i = 0; i < n; ++i) d[i] = A[i * n + i];
}

Eigen gtr_eigen(int S, const double *freqs, const double *exch) {
  Eigen e;
  e.S = S;
  std::vector<double> Q(S * S, 0.0);
  int k = 0;
  for (int i = 0; i < S; ++i)
    for (int j = i + 1; j < S; ++j, ++k) {
      if (!(exch[k] >= 0.0) || !std::isfinite(exch[k]))
        throw Error(NETLK_ERR_INVALID_ARGUMENT, "exchangeabilities must be finite and >= 0");
      Q[i * S + j] = exch[k] * freqs[j];
      Q[j * S + i] = exch[k] * freqs[i];
    }
  for (int i = 0; i < S; ++i) {
    if (!(freqs[i] > 0.0)) throw Error(NETLK_ERR_INVALID_ARGUMENT, "frequencies must be > 0");
    double s = 0.0;
    for (int j = 0; j < S; ++j)
      if (j != i) s += Q[i * S + j];
    Q[i * S + i] = -s;
  }
  double mu = 0.0;
  for (int i = 0; i < S; ++i) mu -= freqs[i] * Q[i * S + i];
  if (!(mu > 0.0)) throw Error(NETLK_ERR_INVALID_ARGUMENT, "degenerate rate matrix");
  for (double &q : Q) q /= mu;
  std::vector<double> sq(S), B(S * S);
  for (int i = 0; i < S; ++i) sq[i] = std::sqrt(freqs[i]);
  for (int i = 0; i < S; ++i)
    for (int j = 0; j < S; ++j) B[i * S + j] = sq[i] * Q[i * S + j] / sq[j];
  for (int i = 0; i < S; ++i)
    for (int j = i + 1; j < S; ++j) B[i * S + j] = B[j * S + i] = 0.5 * (B[i * S + j] + B[j * S + i]);
  std::vector<double> V, d;
  jacobi_eigen(S, B, V, d);
  e.lambda = d;
  e.U.assign(S * S, 0.0);
  e.Uinv.assign(S * S, 0.0);
  for (int i = 0; i < S; ++i)
    for (int j = 0; j < S; ++j) {
      e.U[i * S + j] = V[i * S + j] / sq[i];     // U = Pi^-1/2 V
      e.Uinv[j * S + i] = V[i * S + j] * sq[i];  // U^-1 = V^T Pi^1/2
    }
  e.Q = Q;
  return e;
}

// Regularized lower incomplete gamma P(a, x).
static double gammp(double a, double x) {
  if (x <= 0.0) return 0.0;
  const double lg = std::lgamma(a);
  if (x < a + 1.0) {
    double ap = a, sum = 1.0 / a, del = sum;
    for (int n = 0; n < 100000; ++n) {
      ap += 1.0;
      del *= x / ap;
      sum += del;
      if (std::fabs(del) < std::fabs(sum) * 1e-17) break;
    }
    return sum * std::exp(-x + a * std::log(x) - lg);
  }
  // Legendre continued fraction for Q(a, x), modified Lentz.
  const double tiny = 1e-300;
  double b = x + 1.0 - a, c = 1.0 / tiny, dd = 1.0 / b, h = dd;
  for (int i = 1; i < 100000; ++i) {
    double an = -i * (i - a);
    b += 2.0;
    dd = an * dd + b;
    if (std::fabs(dd) < tiny) dd = tiny;
    c = b + an / c;
    if (std::fabs(c) < tiny) c = tiny;
    dd = 1.0 / dd;
    double del = dd * c;
    h *= del;
    if (std::fabs(del - 1.0) < 1e-17) break;
  }
  return 1.0 - std::exp(-x + a * std::log(x) - lg) * h;
}

// x with P(a, x) = q.
static double gamma_quantile(double a, double q) {
  double lo = 0.0, hi = std::max(1.0, a);
  while (gammp(a, hi) < q) hi *= 2.0;
  double x = 0.5 * (lo + hi);
  const double lg = std::lgamma(a);
  for (int it = 0; it < 200; ++it) {
    double f = gammp(a, x) - q;
    if (f < 0) lo = x; else hi = x;
    double pdf = std::exp((a - 1.0) * std::log(x) - x - lg);
    double xn = (pdf > 0) ? x - f / pdf : 0.5 * (lo + hi);
    if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
    if (std::fabs(xn - x) <= 1e-16 * x) {
      x = xn;
      break;
    }
    x = xn;
  }
  return x;
}

std::vector<double> gamma_mean_rates(double alpha, int ncat) {
  if (!(alpha > 0.0) || !std::isfinite(alpha)) throw Error(NETLK_ERR_INVALID_ARGUMENT, "alpha must be > 0");
  std::vector<double> rates(ncat, 1.0);
  if (ncat == 1) return rates;
  std::vector<double> cdf(ncat + 1, 0.0);
  cdf[ncat] = 1.0;
  for (int k = 1; k < ncat; ++k) {
    double x = gamma_quantile(alpha, (double)k / ncat);  // quantile of Gamma(alpha, 1)
    cdf[k] = gammp(alpha + 1.0, x);
  }
  for (int k = 0; k < ncat; ++k) rates[k] = ncat * (cdf[k + 1] - cdf[k]);
  return rates;
}

}  // namespace netlk
