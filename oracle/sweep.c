/*
 * CPU oracle: whole-DAG FP64 sweeps (forward pruning + adjoint gradient).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU library at full workload
 * sizes and the timed CPU baseline. Nothing in the product links it.
 *
 * Forward: the reference's schedule, processPartitionsImproved
 * (src/likelihood/ImprovedLoglikelihood.cpp:488-519), as a flat list of
 * displayed-tree variants in post-order; each op is the
 * pll_update_partials_single call of :125-150 / :164-190 (same arithmetic and
 * libpll 2^-256 / 2^256 per-site scaling as clv.c, restated from the
 * published method), then pll_compute_root_loglikelihood (:450) per
 * displayed-tree root variant and partition.
 *
 * Threads play the reference's MPI ranks: each thread owns a contiguous
 * pattern slice of every partition and runs the whole schedule over it
 * (every rank of the reference holds its site slice of every partition and
 * runs the same schedule, ImprovedLoglikelihood.cpp:473-483). Per-thread
 * partial sums are added in thread order, so results depend only on the
 * thread count.
 *
 * With invariant sites (+I) the site likelihood is gamma_frac times the
 * root mixture plus inv_term[s] (in unscaled units).
 *
 * Adjoint (no counterpart in the reference, which differentiates one edge at
 * a time through sumtables, LikelihoodDerivatives.cpp:190-344): reverse-mode
 * differentiation of the same pruning. For op x with
 * X = 2^(256 k) (Pa a) * (Pb b) (k = 1 where the op rescaled the site),
 * u_a = 2^(256 k) adj_x * (Pb b), d logL / d t_a += sum u_a * (dPa/dt a),
 * adj_a += Pa^T u_a, symmetrically for b. Seeds at a displayed-tree root:
 * adj = w_tree * weight_s * rw_r * pi_i / L_s with L_s the scaled site
 * likelihood and w_tree the tree's posterior weight in the mixture.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define SCALE_THRESHOLD 0x1p-256
#define SCALE_FACTOR 0x1p+256
#define LOG_SCALE_THRESHOLD (-256.0 * 0.69314718055994530942)
#define FAKE_CHILD INT32_MIN

typedef struct {
  int32_t out;    /* variant id computed */
  int32_t a, b;   /* child: variant id >= 0, -1 - tip, or FAKE_CHILD (b only) */
  int32_t ea, eb; /* edge ids (-1 with the fake child) */
  int32_t first;  /* adjoint: bit 0 / bit 1 set where this op's message is the
                     first one child a / b receives (it stores instead of adds) */
} oracle_op;

typedef struct {
  int32_t R, S;
  int64_t n;                  /* patterns */
  const uint32_t *tips;       /* [n_tips][n] state masks */
  const double *weights;      /* [n] */
  const double *freqs;        /* [S] */
  const double *rate_weights; /* [R] */
  const double *pmat;         /* [n_edges][R][S][S] */
  const double *dpmat;        /* [n_edges][R][S][S] d/dt (adjoint only) */
  double *clv;                /* [n_var][n][R][S] */
  uint32_t *scaler;           /* [n_var][n] */
  double *adj;                /* [n_var][n][R][S] (adjoint only) */
  double gamma_frac;          /* 1 - pinv */
  const double *inv_term;     /* [n] pinv * pi(invariant state), or NULL without +I */
} oracle_part;

static int n_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static int thread_id(void) {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

/* y[r][i] = sum_j M[r][i][j] x[r][j] for one site; a tip child is its 0/1
 * state mask, the fake child is all ones with the identity matrix. Inlined
 * with constant R and S where the caller passes them. */
static inline __attribute__((always_inline)) void child_product(const oracle_part *pp, int32_t c, int64_t s,
                                                                const double *M, double *y, const int R,
                                                                const int S) {
  if (c == FAKE_CHILD) {
    for (int k = 0; k < R * S; ++k) y[k] = 1.0;
    return;
  }
  if (c < 0) {
    const uint32_t code = pp->tips[(int64_t)(-1 - c) * pp->n + s];
    for (int r = 0; r < R; ++r)
      for (int i = 0; i < S; ++i) {
        const double *m = M + ((int64_t)r * S + i) * S;
        double t = 0.0;
        for (int j = 0; j < S; ++j) t += ((code >> j) & 1u) ? m[j] : 0.0;
        y[r * S + i] = t;
      }
    return;
  }
  const double *x = pp->clv + ((int64_t)c * pp->n + s) * R * S;
  for (int r = 0; r < R; ++r)
    for (int i = 0; i < S; ++i) {
      const double *m = M + ((int64_t)r * S + i) * S;
      double t = 0.0;
      for (int j = 0; j < S; ++j) t += m[j] * x[r * S + j];
      y[r * S + i] = t;
    }
}

/* y[r][j] (=|+=) sum_i M[r][i][j] u[r][i] */
static inline __attribute__((always_inline)) void transposed_product(const double *M, const double *u, double *y,
                                                                     int add, const int R, const int S) {
  for (int r = 0; r < R; ++r)
    for (int j = 0; j < S; ++j) {
      double acc = 0.0;
      for (int i = 0; i < S; ++i) acc += M[((int64_t)r * S + i) * S + j] * u[r * S + i];
      y[r * S + j] = add ? y[r * S + j] + acc : acc;
    }
}

static inline uint32_t child_scaler(const oracle_part *pp, int32_t c, int64_t s) {
  return c >= 0 ? pp->scaler[(int64_t)c * pp->n + s] : 0u;
}

static inline const double *edge_mat(const double *base, int32_t e, int R, int S) {
  return base + (int64_t)e * R * S * S;
}

/* One forward op over the sites [lo, hi) of one partition. */
static inline __attribute__((always_inline)) void forward_op(const oracle_part *pp, const oracle_op *op, int64_t lo,
                                                             int64_t hi, const int R, const int S) {
  const int RS = R * S;
  double ya[8 * 20], yb[8 * 20];
  const double *Ma = edge_mat(pp->pmat, op->ea, R, S);
  const double *Mb = op->b == FAKE_CHILD ? NULL : edge_mat(pp->pmat, op->eb, R, S);
  for (int64_t s = lo; s < hi; ++s) {
    child_product(pp, op->a, s, Ma, ya, R, S);
    child_product(pp, op->b, s, Mb, yb, R, S);
    double *x = pp->clv + ((int64_t)op->out * pp->n + s) * RS;
    int small = 1;
    for (int k = 0; k < RS; ++k) {
      x[k] = ya[k] * yb[k];
      small &= x[k] < SCALE_THRESHOLD;
    }
    uint32_t sc = child_scaler(pp, op->a, s) + child_scaler(pp, op->b, s);
    if (small) {
      for (int k = 0; k < RS; ++k) x[k] *= SCALE_FACTOR;
      sc += 1;
    }
    pp->scaler[(int64_t)op->out * pp->n + s] = sc;
  }
}

/* One adjoint op over the sites [lo, hi); returns the two edge terms. */
static inline __attribute__((always_inline)) void adjoint_op(const oracle_part *pp, const oracle_op *op, int64_t lo,
                                                             int64_t hi, double *ga_out, double *gb_out,
                                                             const int R, const int S) {
  const int RS = R * S;
  double ya[8 * 20], yb[8 * 20], da[8 * 20], db[8 * 20], ua[8 * 20], ub[8 * 20];
  const int fake = op->b == FAKE_CHILD;
  const double *Ma = edge_mat(pp->pmat, op->ea, R, S);
  const double *Da = edge_mat(pp->dpmat, op->ea, R, S);
  const double *Mb = fake ? NULL : edge_mat(pp->pmat, op->eb, R, S);
  const double *Db = fake ? NULL : edge_mat(pp->dpmat, op->eb, R, S);
  double ga = 0.0, gb = 0.0;
  for (int64_t s = lo; s < hi; ++s) {
    const double *ax = pp->adj + ((int64_t)op->out * pp->n + s) * RS;
    child_product(pp, op->a, s, Ma, ya, R, S);
    child_product(pp, op->b, s, Mb, yb, R, S);
    child_product(pp, op->a, s, Da, da, R, S);
    if (!fake) child_product(pp, op->b, s, Db, db, R, S);
    const uint32_t k = pp->scaler[(int64_t)op->out * pp->n + s] - child_scaler(pp, op->a, s) -
                       child_scaler(pp, op->b, s);
    const double f = k ? SCALE_FACTOR : 1.0;
    for (int q = 0; q < RS; ++q) {
      ua[q] = f * (ax[q] * yb[q]);
      ga += ua[q] * da[q];
    }
    if (!fake)
      for (int q = 0; q < RS; ++q) {
        ub[q] = f * (ax[q] * ya[q]);
        gb += ub[q] * db[q];
      }
    if (op->a >= 0)
      transposed_product(Ma, ua, pp->adj + ((int64_t)op->a * pp->n + s) * RS, !(op->first & 1), R, S);
    if (!fake && op->b >= 0)
      transposed_product(Mb, ub, pp->adj + ((int64_t)op->b * pp->n + s) * RS, !(op->first & 2), R, S);
  }
  *ga_out += ga;
  *gb_out += gb;
}

static double root_site(const oracle_part *pp, const double *x, int R, int S) {
  double site = 0.0;
  for (int r = 0; r < R; ++r) {
    double q = 0.0;
    for (int i = 0; i < S; ++i) q += pp->freqs[i] * x[r * S + i];
    site += pp->rate_weights[r] * q;
  }
  return site;
}

/* Forward sweep + per-slot root log-likelihoods.
 * slot_variant [n_slots]: the variant holding each displayed tree's root CLV;
 * slot_logl [n_slots][n_parts] receives sum_s w_s log L_s (scaled back). */
int oracle_sweep_forward(int32_t n_ops, const oracle_op *ops, int32_t n_parts, const oracle_part *parts,
                         int32_t n_slots, const int32_t *slot_variant, double *slot_logl) {
  const int T = n_threads();
  double *partial = (double *)calloc((size_t)T * n_slots * n_parts, sizeof(double));
  if (!partial) return 1;
#pragma omp parallel
  {
    const int t = thread_id();
    for (int p = 0; p < n_parts; ++p) {
      const oracle_part *pp = &parts[p];
      const int R = pp->R, S = pp->S, RS = R * S;
      const int64_t lo = pp->n * t / T, hi = pp->n * (t + 1) / T;
      for (int o = 0; o < n_ops; ++o) {
        if (R == 4 && S == 4)
          forward_op(pp, &ops[o], lo, hi, 4, 4);
        else if (R == 4 && S == 20)
          forward_op(pp, &ops[o], lo, hi, 4, 20);
        else
          forward_op(pp, &ops[o], lo, hi, R, S);
      }
      for (int d = 0; d < n_slots; ++d) {
        const int32_t v = slot_variant[d];
        double acc = 0.0;
        for (int64_t s = lo; s < hi; ++s) {
          const double site = root_site(pp, pp->clv + ((int64_t)v * pp->n + s) * RS, R, S);
          double l = log(pp->gamma_frac * site) + (double)pp->scaler[(int64_t)v * pp->n + s] * LOG_SCALE_THRESHOLD;
          if (pp->inv_term && pp->inv_term[s] > 0.0) {  /* + pinv * pi(state), in log space */
            const double b = log(pp->inv_term[s]);
            l = l > b ? l + log1p(exp(b - l)) : b + log1p(exp(l - b));
          }
          acc += pp->weights[s] * l;
        }
        partial[((size_t)t * n_slots + d) * n_parts + p] = acc;
      }
    }
  }
  for (int d = 0; d < n_slots; ++d)
    for (int p = 0; p < n_parts; ++p) {
      double acc = 0.0;
      for (int t = 0; t < T; ++t) acc += partial[((size_t)t * n_slots + d) * n_parts + p];
      slot_logl[(size_t)d * n_parts + p] = acc;
    }
  free(partial);
  return 0;
}

/* Adjoint sweep after oracle_sweep_forward. bwd_ops: the ops whose variant
 * is reachable from a used displayed-tree root, parents before children,
 * with their `first` flags set. Every root slot's variant is seeded (stored,
 * not added) before the ops run; slot_weight [n_slots][n_parts] is each
 * slot's posterior weight in its partition's mixture. grad [n_parts][n_edges]
 * receives d logL / d t_e per partition (the partition's own lengths). */
int oracle_sweep_adjoint(int32_t n_ops, const oracle_op *bwd_ops, int32_t n_var, int32_t n_parts,
                         const oracle_part *parts, int32_t n_slots, const int32_t *slot_variant,
                         const double *slot_weight, int32_t n_edges, double *grad) {
  (void)n_var;
  const int T = n_threads();
  double *partial = (double *)calloc((size_t)T * n_parts * n_edges, sizeof(double));
  if (!partial) return 1;
#pragma omp parallel
  {
    const int t = thread_id();
    for (int p = 0; p < n_parts; ++p) {
      double *g = partial + ((size_t)t * n_parts + p) * n_edges;
      const oracle_part *pp = &parts[p];
      const int R = pp->R, S = pp->S, RS = R * S;
      const int64_t lo = pp->n * t / T, hi = pp->n * (t + 1) / T;
      for (int d = 0; d < n_slots; ++d) {
        const double w = slot_weight[(size_t)d * n_parts + p];
        const int32_t v = slot_variant[d];
        for (int64_t s = lo; s < hi; ++s) {
          const double *x = pp->clv + ((int64_t)v * pp->n + s) * RS;
          double *ad = pp->adj + ((int64_t)v * pp->n + s) * RS;
          /* d log L_s / d X[r][i] = gamma_frac rw_r pi_i / L_s, L_s in X's scaled units */
          double den = pp->gamma_frac * root_site(pp, x, R, S);
          if (pp->inv_term && pp->inv_term[s] > 0.0)
            den += ldexp(pp->inv_term[s], 256 * (int)pp->scaler[(int64_t)v * pp->n + s]);
          const double c = w * pp->weights[s] * pp->gamma_frac / den;
          for (int r = 0; r < R; ++r)
            for (int i = 0; i < S; ++i) ad[r * S + i] = c * pp->rate_weights[r] * pp->freqs[i];
        }
      }
      for (int o = 0; o < n_ops; ++o) {
        const oracle_op *op = &bwd_ops[o];
        double ga = 0.0, gb = 0.0;
        if (R == 4 && S == 4)
          adjoint_op(pp, op, lo, hi, &ga, &gb, 4, 4);
        else if (R == 4 && S == 20)
          adjoint_op(pp, op, lo, hi, &ga, &gb, 4, 20);
        else
          adjoint_op(pp, op, lo, hi, &ga, &gb, R, S);
        g[op->ea] += ga;
        if (op->b != FAKE_CHILD) g[op->eb] += gb;
      }
    }
  }
  for (int p = 0; p < n_parts; ++p)
    for (int e = 0; e < n_edges; ++e) {
      double acc = 0.0;
      for (int t = 0; t < T; ++t) acc += partial[((size_t)t * n_parts + p) * n_edges + e];
      grad[(size_t)p * n_edges + e] = acc;
    }
  free(partial);
  return 0;
}

int oracle_sweep_threads(void) { return n_threads(); }
