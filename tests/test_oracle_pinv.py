"""CPU: invariant sites (+I) in the oracle, before the GPU tests use it.

With pinv > 0 the site likelihood is (1 - pinv) times the Gamma mixture
(category rates divided by 1 - pinv) plus pinv times the frequency of the
one state every tip admits, if there is one. Checked here: the invariant-state
rule on hand-made patterns; the improved (DAG) and naive (per displayed tree)
oracles agree; the C sweeps' logL equals the DAG oracle's and their adjoint
gradient the sumtable derivatives of ``derivatives.py``, which in turn equal
central differences of the log-likelihood.
"""
import numpy as np
import pytest

from conftest import GoldenPartition, golden_cases

CASES = {c["name"]: c for c in golden_cases()}
NAMES = ["twoReticulations", "threeReticulations", "synthetic_12taxa_3ret_2parts"]


def _oracle(name, variant, pinv):
    from oracle import improved, newick, pllmath
    case = CASES[name]
    parts = []
    for d in case["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4), pinv=pinv))
    return improved.ImprovedOracle(newick.parse_newick(case["newick"]), parts, variant=variant)


def test_invariant_state_rule():
    from oracle import pllmath
    # tips x patterns: A/A/A -> A; A/R(=A|G)/A -> A; A/C -> none; N/N -> none
    # (four states in common); G/N/G -> G
    codes = np.array([[1, 1, 1, 15, 4],
                      [1, 5, 2, 15, 15],
                      [1, 1, 1, 15, 4]], np.uint32)
    assert pllmath.invariant_states(codes).tolist() == [0, 0, -1, -1, 2]


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_pinv_oracles_agree(name, variant):
    from oracle import derivatives, naive, sweep
    pinv = 0.3
    orc = _oracle(name, variant, pinv)
    logl = orc.loglikelihood()
    base = _oracle(name, variant, 0.0).loglikelihood()
    assert logl != base
    if variant == "AVERAGE":
        assert naive.naive_loglikelihood(orc)[0] == pytest.approx(logl, rel=1e-10)
    so = sweep.SweepOracle(orc)
    total, _, _, g, gr = so.evaluate()
    assert total == pytest.approx(logl, rel=1e-12)
    d = derivatives.EdgeDerivativeOracle(orc)
    g2, gr2 = d.gradient()
    scale = max(1.0, float(np.abs(g2).max()))
    assert np.abs(g - g2).max() <= 1e-8 * scale
    if len(gr):
        assert np.abs(gr - gr2).max() <= 1e-8 * max(1.0, float(np.abs(gr2).max()))
    # the sumtable derivatives against central differences of the logL
    h = 1e-6
    for e in range(0, orc.net.n_edges, 3):
        t = orc.brlen[e]
        if t < 1e-4:
            continue
        orc.brlen[e] = t + h
        up = orc.loglikelihood()
        orc.brlen[e] = t - h
        dn = orc.loglikelihood()
        orc.brlen[e] = t
        assert g2[e] == pytest.approx((up - dn) / (2 * h), rel=1e-4, abs=1e-4)
