"""GPU: gradients and edge derivatives against the oracle's analytic derivatives.

``tests/golden/derivative_cases.json`` holds, per golden case, the derivatives
that ``oracle/derivatives.py`` computes the reference's way (per-tree sumtable
derivatives at the edge, combined by ``LikelihoodDerivatives.cpp``'s
formulas; pinned on CPU against finite differences in
``test_oracle_derivatives.py``). Through the C ABI:

* the adjoint gradient (``netlk_loglikelihood_gradient``): FP64 within 1e-8
  relative (plus 1e-9 of the largest entry), FP32 within 1e-4 relative (plus
  1e-4 of the largest entry), for every branch length and reticulation
  probability;
* ``netlk_edge_derivatives`` mode 0 (true derivative) and mode 1 (the
  reference's formula), on the edge sumtables (default) and on the tangent
  sweep (``sumtables = 0``), FP64: d1 within 1e-8 relative on every edge; d2 - a
  central difference of d1 over +-1e-6 - within 1e-4 relative where the
  length is at least 1e-3 (nearer the 1e-6 clamp the difference is one-sided);
* the same in FP32: d1 within 1e-4 relative (plus 1e-4 of the largest entry),
  d2 - a central difference over a step that grows with the length - within
  4e-3 of max(1, |d2|) on every edge longer than 2e-5 (measured worst: 1.8e-3).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, GoldenPartition, golden_cases

pytestmark = pytest.mark.gpu

CASES = {c["name"]: c for c in golden_cases()}
with open(os.path.join(GOLDEN, "derivative_cases.json")) as _f:
    DERIVS = {c["name"]: c for c in json.load(_f)["cases"]}
NAMES = sorted(DERIVS)


def _lik(name, variant, precision, **kw):
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    case = CASES[name]
    net = parse_extended_newick(case["newick"])
    parts = [GoldenPartition(d) for d in case["partitions"]]
    return NetworkLikelihood(net, parts, variant=variant, precision=precision, **kw)


def _close(got, want, rel, abs_frac):
    got, want = np.asarray(got, float), np.asarray(want, float)
    scale = max(1.0, float(np.abs(want).max())) if want.size else 1.0
    err = np.abs(got - want)
    ok = err <= rel * np.abs(want) + abs_frac * scale
    return bool(ok.all()), float((err / np.maximum(np.abs(want), scale * 1e-3)).max()) if want.size else 0.0


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gradient_matches_analytic_oracle(name, variant, precision):
    want = DERIVS[name][variant]
    rel, absf = (1e-8, 1e-9) if precision == "fp64" else (1e-4, 1e-4)
    with _lik(name, variant, precision) as lik:
        _, gb, gr = lik.loglikelihood_gradient()
    ok, worst = _close(gb, want["grad_brlen"], rel, absf)
    print("%s %s %s brlen worst relative error %.2e" % (name, variant, precision, worst))
    assert ok, worst
    if len(want["grad_retprob"]):
        ok, worst = _close(gr, want["grad_retprob"], rel, absf)
        print("%s %s %s retprob worst relative error %.2e" % (name, variant, precision, worst))
        assert ok, worst


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("sumtables", [True, False])
def test_edge_derivatives_match_analytic_oracle(name, variant, mode, sumtables):
    want = DERIVS[name][variant]
    key = "true" if mode == 0 else "reference"
    w1 = np.array(want["d1_" + key])
    w2 = np.array(want["d2_" + key])
    with _lik(name, variant, "fp64", sumtables=sumtables) as lik:
        lengths = lik.branch_lengths.copy()
        got1, got2 = [], []
        for e in range(lik.n_edges):
            d1, d2 = lik.edge_derivatives(e, second=True, mode=mode)
            got1.append(d1)
            got2.append(d2)
        # the context is left evaluating the network at its own lengths
        assert lik.loglikelihood() == pytest.approx(CASES[name][variant]["logl"], rel=1e-9)
    ok, worst = _close(got1, w1, 1e-8, 1e-9)
    print("%s %s mode %d d1 worst relative error %.2e" % (name, variant, mode, worst))
    assert ok, worst
    # d2 is analytic (tangent sweep): every edge, clamped lengths included
    ok, worst = _close(np.array(got2), w2, 1e-8, 1e-8)
    print("%s %s mode %d d2 worst relative error %.2e" % (name, variant, mode, worst))
    assert ok, worst


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("sumtables", [True, False])
def test_fp32_edge_derivatives_match_analytic_oracle(name, variant, mode, sumtables):
    want = DERIVS[name][variant]
    key = "true" if mode == 0 else "reference"
    w1 = np.array(want["d1_" + key])
    w2 = np.array(want["d2_" + key])
    with _lik(name, variant, "fp32", sumtables=sumtables) as lik:
        lengths = lik.branch_lengths.copy()
        got = np.array([lik.edge_derivatives(e, second=True, mode=mode) for e in range(lik.n_edges)])
    ok, worst = _close(got[:, 0], w1, 1e-4, 1e-4)
    print("%s %s fp32 mode %d d1 worst relative error %.2e" % (name, variant, mode, worst))
    assert ok, worst
    # analytic d2 from FP32 tangents: every edge, clamped lengths included
    err = np.abs(got[:, 1] - w2) / np.maximum(1.0, np.abs(w2))
    print("%s %s fp32 mode %d d2 worst error %.2e" % (name, variant, mode, err.max()))
    assert err.max() <= 1e-4, err.max()


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_random_networks_match_oracle(seed, precision):
    """Random networks with arcs on any edge (reticulations below
    reticulations, nodes that die in some configurations; the generator of
    test_dag_random.py), 40 simulated-free random patterns: logL against the
    DAG oracle (FP64 1e-9, FP32 1e-6) and the adjoint gradient against the
    analytic derivative oracle (FP64 1e-8, FP32 1e-4 plus 1e-4 of the largest
    entry), AVERAGE and BEST; edge sumtables at a proposed length on three
    edges against the oracle at that length (logL as above, d1 and d2 FP64
    1e-8, FP32 d1 1e-4 and d2 5e-4 of the gradient scale)."""
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    from oracle import derivatives, improved, newick as onewick, pllmath
    from test_dag_random import nasty_network
    rng = np.random.default_rng(7000 + seed)
    n_taxa = int(rng.integers(4, 16))
    n_ret = int(rng.integers(1, 6))
    text = nasty_network(rng, n_taxa, n_ret)
    freqs = rng.dirichlet(np.ones(4))
    part = GoldenPartition({"tip_states": rng.integers(1, 16, size=(n_taxa, 40)).tolist(),
                            "weights": rng.integers(1, 4, size=40).astype(float).tolist(),
                            "freqs": (freqs / freqs.sum()).tolist(),
                            "exch": (rng.dirichlet(np.ones(6)) * 6).tolist(), "alpha": 0.7})
    onet = onewick.parse_newick(text)
    net = parse_extended_newick(text)
    rel, absf = (1e-8, 1e-9) if precision == "fp64" else (1e-4, 1e-4)
    for variant in ("AVERAGE", "BEST"):
        opart = improved.Partition(part.tip_states, part.weights, part.freqs, part.exch,
                                   pllmath.gamma_rates_mean(part.alpha, 4))
        orc = improved.ImprovedOracle(onet, [opart], variant=variant)
        want_logl = orc.loglikelihood()
        g, gr = derivatives.EdgeDerivativeOracle(orc).gradient()
        # edge sumtables at a proposed length (three edges) against the
        # oracle with that length: logL, d1, d2
        edges = rng.choice(net.n_edges, size=min(3, net.n_edges), replace=False)
        stab = {}
        with NetworkLikelihood(net, [part], variant=variant, precision=precision) as lik:
            total, gb, gbr = lik.loglikelihood_gradient()
            for e in edges:
                stab[int(e)] = lik.edge_sumtable_derivatives(int(e), 0.37 * lik.branch_lengths[e] + 0.01)
        assert total == pytest.approx(want_logl, rel=1e-9 if precision == "fp64" else 1e-6), text
        ok, worst = _close(gb, g, rel, absf)
        assert ok, (variant, worst, text)
        ok, worst = _close(gbr, gr, rel, absf)
        assert ok, (variant, worst, text)
        for e, (l, d1, d2) in stab.items():
            t0 = orc.brlen[e]
            orc.brlen[e] = 0.37 * t0 + 0.01
            wl = orc.loglikelihood()
            w1, w2 = derivatives.EdgeDerivativeOracle(orc).edge(e)
            orc.brlen[e] = t0
            orc.loglikelihood()
            assert l == pytest.approx(wl, rel=1e-9 if precision == "fp64" else 1e-6), (variant, e, text)
            scale = max(1.0, float(np.abs(g).max()))
            # FP32 d2: per-site L''/L - (L'/L)^2 cancels in FP32 (measured worst
            # on these networks 1.1e-4 of the scale)
            tol1, tol2 = (1e-8, 1e-8) if precision == "fp64" else (1e-4, 5e-4)
            assert abs(d1 - w1) <= tol1 * max(scale, abs(w1)), (variant, e, d1, w1, text)
            assert abs(d2 - w2) <= tol2 * max(scale, abs(w2)), (variant, e, d2, w2, text)
