"""CPU: the oracle's analytic branch-length derivatives (``oracle/derivatives.py``).

The restatement of the reference's per-edge sumtable derivatives is pinned
three ways before the GPU tests use it: its per-tree log-likelihoods equal the
displayed-tree DAG oracle's, its gradient equals the central differences
stored in the likelihood fixtures, and its second derivatives equal central
differences of its first. ``derivative_cases.json`` is checked against a fresh
run of the oracle.
"""
import json
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases

sys.path.insert(0, GOLDEN)
import make_derivative_golden as mdg  # noqa: E402

CASES = {c["name"]: c for c in golden_cases()}


def _derivs():
    with open(os.path.join(GOLDEN, "derivative_cases.json")) as f:
        return {c["name"]: c for c in json.load(f)["cases"]}


DERIVS = _derivs()


def _oracle(name, variant):
    from oracle import derivatives
    orc = mdg.oracle_for(CASES[name], variant)
    return orc, derivatives.EdgeDerivativeOracle(orc)


SMALL = ["tinyNetwork", "smallNetwork", "twoReticulations", "threeReticulations", "interleavedReticulations",
         "reticulationInReticulation", "synthetic_12taxa_3ret_2parts", "protein_8taxa_2ret"]


@pytest.mark.parametrize("name", SMALL)
def test_tree_loglikelihoods_match_the_dag_oracle(name):
    orc, d = _oracle(name, "AVERAGE")
    for t, tr in zip(orc.root_trees(), d.trees):
        if t.logl_valid:
            assert np.allclose(t.partition_logl, tr["logl"], rtol=1e-11, atol=1e-9)


@pytest.mark.parametrize("name", [n for n in DERIVS if "fd_grad_brlen" in CASES[n]["AVERAGE"]])
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_gradient_matches_finite_differences(name, variant):
    want = CASES[name][variant]
    got = DERIVS[name][variant]
    fd = np.array(want["fd_grad_brlen"])
    g = np.array(got["grad_brlen"])
    from oracle import newick
    lengths = np.array(newick.parse_newick(CASES[name]["newick"]).edge_length)
    free = lengths > 2e-5  # clamped edges only have a one-sided difference
    assert np.all(np.abs(g - fd)[free] <= 1e-5 * np.maximum(1.0, np.abs(fd[free])))
    fdr = np.array(want["fd_grad_retprob"])
    assert np.allclose(got["grad_retprob"], fdr, rtol=1e-5, atol=1e-6)
    # the gradient is the mode-0 first derivative, edge by edge
    assert np.allclose(got["d1_true"], g, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("name", ["smallNetwork", "synthetic_12taxa_3ret_2parts", "protein_8taxa_2ret"])
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_second_derivative_is_the_derivative_of_the_first(name, variant):
    """Every reticulation edge and the first four other free edges, both modes."""
    orc, d = _oracle(name, variant)
    from oracle import derivatives
    base = list(orc.brlen)
    ret = set(orc.net.ret_first_edge) | set(orc.net.ret_second_edge)
    free = [e for e in range(orc.net.n_edges) if base[e] >= 1e-4]
    edges = [e for e in free if e in ret] + [e for e in free if e not in ret][:4]
    h = 1e-5
    for e in edges:
        shifted = []
        for sgn in (1, -1):
            orc.brlen = list(base)
            orc.brlen[e] = base[e] + sgn * h
            orc.loglikelihood()
            shifted.append(derivatives.EdgeDerivativeOracle(orc))
        orc.brlen = list(base)
        for mode in ("true", "reference"):
            want = (shifted[0].edge(e, mode)[0] - shifted[1].edge(e, mode)[0]) / (2 * h)
            got = d.edge(e, mode)[1]
            assert got == pytest.approx(want, rel=1e-5, abs=1e-5 * max(1.0, abs(want))), (e, mode)


@pytest.mark.parametrize("name", ["tinyNetwork", "twoReticulations", "reticulationInReticulation",
                                  "synthetic_12taxa_3ret_2parts", "protein_10taxa_3ret_2parts"])
def test_fixture_matches_the_oracle(name):
    for variant in ("AVERAGE", "BEST"):
        fresh = mdg.score(CASES[name], variant)
        for key, val in fresh.items():
            assert np.allclose(val, DERIVS[name][variant][key], rtol=1e-12, atol=1e-12), key


def test_reference_formula_equals_the_true_derivative_on_edges_in_every_tree():
    """A tree edge that every displayed tree contains is active everywhere, so
    the reference's restricted AVERAGE is the true derivative; a reticulation
    edge is restricted and differs."""
    rec = DERIVS["synthetic_12taxa_3ret_2parts"]["AVERAGE"]
    from oracle import newick
    net = newick.parse_newick(CASES["synthetic_12taxa_3ret_2parts"]["newick"])
    ret_edges = set(net.ret_first_edge) | set(net.ret_second_edge)
    tips = [e for e in range(net.n_edges) if net.edge_child[e] < net.n_tips and e not in ret_edges]
    assert tips
    for e in tips:  # pendant edges lie in every displayed tree
        assert rec["d1_reference"][e] == pytest.approx(rec["d1_true"][e], rel=1e-12, abs=1e-12)
    assert any(abs(rec["d1_reference"][e] - rec["d1_true"][e]) > 1e-6 for e in ret_edges)


def test_fp64_second_derivative_step_near_the_length_clamp():
    """netlk_edge_derivatives takes d2 in FP64 as a central difference of d1
    with step min(1e-6, t/200) (one-sided at the 1e-6 clamp). On a network
    whose zero branch lengths sit at the clamp, sites that need a change on
    such a branch have L ~ t and d2 ~ -1/t^2: the oracle's FP64 arithmetic
    shows that this step recovers the analytic d2 within 1 % on every clamped
    edge, where a fixed 1e-6 step misses it by tens of percent."""
    from oracle import derivatives
    orc, d = _oracle("twoReticulations", "AVERAGE")
    base = list(orc.brlen)
    clamped = [e for e in range(orc.net.n_edges) if base[e] <= 1.0000001e-6]
    assert len(clamped) >= 10

    def fd(e, h):
        t = base[e]
        up, lo = min(t + h, 100.0), max(t - h, 1e-6)
        vals = []
        for x in (up, lo):
            orc.brlen = list(base)
            orc.brlen[e] = x
            orc.loglikelihood()
            vals.append(derivatives.EdgeDerivativeOracle(orc).edge(e)[0])
        orc.brlen = list(base)
        return (vals[0] - vals[1]) / (up - lo)

    worst_rule, worst_fixed = 0.0, 0.0
    for e in clamped:
        want = d.edge(e)[1]
        scale = max(1.0, abs(want))
        worst_rule = max(worst_rule, abs(fd(e, min(1e-6, base[e] / 200.0)) - want) / scale)
        worst_fixed = max(worst_fixed, abs(fd(e, 1e-6) - want) / scale)
    orc.loglikelihood()
    assert worst_rule < 1e-2
    assert worst_fixed > 0.1
