"""The reference's branch-length and reticulation-probability optimizer loops,
restated for the tests that drive them through the library and through the
oracle (test harness; not a test module itself).

* Branch lengths, one pass of ``optimize_branches_internal``
  (src/optimization/BranchLengthOptimization.cpp:422-477) over every edge,
  with ``optimize_branch`` (:284-339): the edge's log-likelihood before, a
  bounded Newton-Raphson search on the derivative callback
  (``network_derivative_func_multi``, :171-200, minimised in the reference by
  pll-modules' ``pllmod_opt_minimize_newton_multi``, not vendored) with bounds
  [brlen_min, brlen_max] and tolerance brlen_min / 10 (:218-236), and the old
  length restored if the log-likelihood got worse (:317-330).
* Branch lengths by Brent (the reference's BRENT_REROOT / BRENT_NORMAL
  methods), ``optimize_branch_brent`` (BranchLengthOptimization.cpp:112-160)
  per edge on the edge log-likelihood.
* Reticulation probabilities, ``optimize_reticulations``
  (src/optimization/ReticulationOptimization.cpp:104-118): per reticulation a
  Brent minimisation of -logL over [brprob_min, brprob_max]
  (``optimize_reticulation``, :75-102; pll-modules' ``pllmod_opt_minimize_brent``,
  not vendored), repeated until a pass leaves the log-likelihood unchanged.

* Model parameters, the one-dimensional part of ``optimize_params``
  (src/optimization/ModelOptimization.cpp:25-97): per partition a Brent
  search of the Gamma shape (pll-modules' ``pllmod_algo_opt_onedim_treeinfo``
  with PLLMOD_OPT_PARAM_ALPHA, bounds 0.02 and 1000), then each
  exchangeability (the last one, GT, fixed at its value) by Brent on its
  logarithm within [1e-3, 1e3] - a coordinate search standing in for
  pll-modules' BFGS over the rates - each evaluation through the
  log-likelihood callback (``likelihood_target_function``).

The Newton and Brent searches follow the published methods: Newton's step
-f'/f'' toward a maximum, clamped to the bounds, with a halving / doubling step
where the curvature is not negative; Brent (1973) golden-section search with
parabolic interpolation.
"""
import math

import numpy as np

BRLEN_MIN, BRLEN_MAX = 1e-6, 100.0           # RAXML_BRLEN_MIN / MAX
BRPROB_MIN, BRPROB_MAX = 1e-6, 1.0 - 1e-6    # NetraxOptions.hpp:102-103
NR_TOLERANCE = BRLEN_MIN / 10.0              # BranchLengthOptimization.cpp:218-220


def newton_maximize(derivs, x0, lo, hi, tol, max_iters):
    """Bounded Newton-Raphson on a log-likelihood with derivatives
    ``derivs(x) -> (d1, d2)``; returns the last iterate."""
    x = x0
    for _ in range(max_iters):
        d1, d2 = derivs(x)
        if d2 < 0.0:
            x_new = x - d1 / d2
        elif d1 > 0.0:
            x_new = 2.0 * x
        else:
            x_new = 0.5 * x
        x_new = min(max(x_new, lo), hi)
        if abs(x_new - x) < tol:
            return x_new
        x = x_new
    return x


def brent_minimize(f, a, b, x0, tol, max_iters=200):
    """Brent's method for min f on [a, b] from x0; returns (x, f(x))."""
    cgold = 0.5 * (3.0 - math.sqrt(5.0))
    x = w = v = min(max(x0, a), b)
    fx = fw = fv = f(x)
    d = e = 0.0
    for _ in range(max_iters):
        m = 0.5 * (a + b)
        tol1 = tol * abs(x) + 1e-12
        tol2 = 2.0 * tol1
        if abs(x - m) <= tol2 - 0.5 * (b - a):
            break
        parabolic = False
        if abs(e) > tol1:
            r = (x - w) * (fx - fv)
            q = (x - v) * (fx - fw)
            p = (x - v) * q - (x - w) * r
            q = 2.0 * (q - r)
            if q > 0.0:
                p = -p
            q = abs(q)
            if abs(p) < abs(0.5 * q * e) and q * (a - x) < p < q * (b - x):
                e, d = d, p / q
                u = x + d
                if u - a < tol2 or b - u < tol2:
                    d = tol1 if x < m else -tol1
                parabolic = True
        if not parabolic:
            e = (b - x) if x < m else (a - x)
            d = cgold * e
        u = x + d if abs(d) >= tol1 else x + (tol1 if d > 0 else -tol1)
        fu = f(u)
        if fu <= fx:
            if u < x:
                b = x
            else:
                a = x
            v, fv, w, fw, x, fx = w, fw, x, fx, u, fu
        else:
            if u < x:
                a = u
            else:
                b = u
            if fu <= fw or w == x:
                v, fv, w, fw = w, fw, u, fu
            elif fu <= fv or v == x or v == w:
                v, fv = u, fu
    return x, fx


def optimize_branches(edge_logl, edge_derivs, lengths, max_iters=30, derivs_at=None):
    """One pass over every edge. edge_logl(e, t): logL with edge e at length
    t (kept); edge_derivs(e): (d1, d2) at the current lengths; or
    derivs_at(e, t): (d1, d2) with edge e at t, nothing kept (the
    reference's callback on sumtables, which only invalidates the edge's
    P-matrix). Returns the final lengths and logL, and whether any step
    lowered the logL."""
    lengths = list(lengths)
    logl = None
    worse = False
    for e in range(len(lengths)):
        t0 = lengths[e]
        start = edge_logl(e, t0)

        def derivs(t, e=e):
            if derivs_at is not None:
                return derivs_at(e, t)
            edge_logl(e, t)
            return edge_derivs(e)

        t = newton_maximize(derivs, t0, BRLEN_MIN, BRLEN_MAX, NR_TOLERANCE, max_iters)
        new = edge_logl(e, t)
        if new < start:  # the reference reloads the old length
            t = t0
            new = edge_logl(e, t0)
        lengths[e] = t
        worse = worse or (logl is not None and new < logl - 1e-6 * abs(logl))
        logl = new
    return lengths, logl, worse


def optimize_branches_brent(logl_at, set_length, lengths, tol):
    """One pass of optimize_branch_brent (BranchLengthOptimization.cpp:112-160)
    over every edge: Brent on -logL within [brlen_min, brlen_max] from the
    current length. logl_at(e, t): logL with edge e at t (nothing kept - the
    reference's BRENT_REROOT evaluates computeLoglikelihoodBrlenOpt);
    set_length(e, t): keep t and return the logL. Returns the final lengths
    and logL."""
    lengths = list(lengths)
    logl = None
    for e in range(len(lengths)):
        x, fx = brent_minimize(lambda t, e=e: -logl_at(e, t), BRLEN_MIN, BRLEN_MAX, lengths[e], tol)
        lengths[e] = x
        logl = set_length(e, x)
    return lengths, logl


def optimize_reticulations(logl_at, probs, tol, max_passes=10):
    """Brent per reticulation until a pass changes nothing. logl_at(probs):
    the network logL at these first-parent probabilities. Returns the final
    probabilities and logL."""
    probs = list(probs)
    act = logl_at(probs)
    for _ in range(max_passes):
        loop = act
        for k in range(len(probs)):
            def f(x, k=k):
                q = list(probs)
                q[k] = x
                return -logl_at(q)

            x, fx = brent_minimize(f, BRPROB_MIN, BRPROB_MAX, probs[k], tol)
            probs[k] = x  # Brent's best point, never worse than its start
            loop = -fx
        if loop == act:
            break
        act = loop
    return probs, logl_at(probs)


ALPHA_MIN, ALPHA_MAX = 0.02, 1000.0     # PLLMOD_OPT_MIN_ALPHA / MAX_ALPHA
SUBST_MIN, SUBST_MAX = 1e-3, 1e3        # PLLMOD_OPT_MIN_SUBST_RATE / MAX


def optimize_model(logl_at, models, tol=1e-6, exchangeabilities=True):
    """models: per partition (freqs, exch, alpha). logl_at(models) -> logL.
    Brent on each alpha, then each exchangeability but the last on a log
    scale; returns the final models and logL."""
    models = [(np.asarray(f, float).copy(), np.asarray(x, float).copy(), float(a)) for f, x, a in models]

    def with_param(p, alpha=None, k=None, value=None):
        out = [(f, x.copy(), a) for f, x, a in models]
        f, x, a = out[p]
        if alpha is not None:
            a = alpha
        if k is not None:
            x[k] = value
        out[p] = (f, x, a)
        return out

    for p in range(len(models)):
        la, _ = brent_minimize(lambda u: -logl_at(with_param(p, alpha=math.exp(u))),
                               math.log(ALPHA_MIN), math.log(ALPHA_MAX), math.log(models[p][2]), tol)
        models = with_param(p, alpha=math.exp(la))
        if exchangeabilities:
            for k in range(len(models[p][1]) - 1):
                lx, _ = brent_minimize(lambda u: -logl_at(with_param(p, k=k, value=math.exp(u))),
                                       math.log(SUBST_MIN), math.log(SUBST_MAX), math.log(models[p][1][k]), tol)
                models = with_param(p, k=k, value=math.exp(lx))
    return models, logl_at(models)
