"""CPU: the oracle's whole-DAG C sweeps (``oracle/sweep.c``) against the
other oracles, before the full-size GPU parity tests and the CPU baseline use
them.

* logL per displayed tree and per partition equals ``improved.py`` (which runs
  the same libpll arithmetic one call per variant, like the reference);
* scale counters equal ``improved.py``'s per variant, bit for bit, on the
  200-taxon case that needs 2^256 rescaling;
* the adjoint gradient (branch lengths and reticulation probabilities) equals
  the analytic per-edge sumtable derivatives of ``derivatives.py`` - the
  reference's own derivative method - stored in ``derivative_cases.json``.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, GoldenPartition, golden_cases

CASES = {c["name"]: c for c in golden_cases()}
with open(os.path.join(GOLDEN, "derivative_cases.json")) as f:
    DERIVS = {c["name"]: c for c in json.load(f)["cases"]}


def _oracle(case, variant):
    from oracle import improved, newick, pllmath
    net = newick.parse_newick(case["newick"])
    parts = []
    for d in case["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4)))
    orc = improved.ImprovedOracle(net, parts, variant=variant)
    orc.loglikelihood()
    return orc


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_sweep_loglikelihood_matches_the_per_variant_oracle(name, variant):
    from oracle import sweep
    orc = _oracle(CASES[name], variant)
    want_total, want_parts = orc.evaluate()
    so = sweep.SweepOracle(orc)
    total, parts, trees, _, _ = so.evaluate(gradient=False)
    assert total == pytest.approx(want_total, rel=1e-13, abs=1e-9)
    assert np.allclose(parts, want_parts, rtol=1e-13, atol=1e-9)
    for t, got in zip(so.trees, trees):
        assert np.allclose(got, t.partition_logl, rtol=1e-13, atol=1e-9)


def test_sweep_scale_counters_match_bit_for_bit():
    from oracle import sweep
    name = "synthetic_200taxa_2ret_deep"
    orc = _oracle(CASES[name], "AVERAGE")
    so = sweep.SweepOracle(orc)
    so.evaluate(gradient=False)
    scaled = 0
    for (node, idx), v in so.variant_of.items():
        for p in range(len(orc.parts)):
            want = orc.pernode[node][idx].scaler[p]
            got = so.keep[p]["scaler"][v]
            assert np.array_equal(got, want)
            scaled += int(want.max() > 0)
    assert scaled > 0  # the case does rescale


@pytest.mark.parametrize("name", sorted(DERIVS))
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_sweep_gradient_matches_the_sumtable_derivatives(name, variant):
    from oracle import sweep
    orc = _oracle(CASES[name], variant)
    _, _, _, g, gr = sweep.SweepOracle(orc).evaluate()
    want = DERIVS[name][variant]
    wg = np.array(want["grad_brlen"])
    scale = max(1.0, float(np.abs(wg).max()))
    assert np.abs(g - wg).max() <= 1e-8 * scale
    if orc.r:
        wr = np.array(want["grad_retprob"])
        assert np.abs(gr - wr).max() <= 1e-8 * max(1.0, float(np.abs(wr).max()))


@pytest.mark.parametrize("name", ["synthetic_12taxa_3ret_2parts", "synthetic_16taxa_4ret_3parts"])
def test_per_partition_lengths(name):
    """Each partition with its own branch lengths (the reference's unlinked
    linkage): the C sweeps' logL equals the DAG oracle's, their per-partition
    gradient the sumtable derivatives', which equal central differences of
    the logL in one partition's length."""
    from oracle import derivatives, sweep
    orc = _oracle(CASES[name], "AVERAGE")
    rng = np.random.default_rng(5)
    orc.part_brlen = [list(np.array(orc.brlen) * np.exp(0.3 * rng.standard_normal(len(orc.brlen))))
                      for _ in orc.parts]
    logl = orc.loglikelihood()
    so = sweep.SweepOracle(orc)
    total, _, _, _, _ = so.evaluate()
    assert total == pytest.approx(logl, rel=1e-12)
    gpp = so.grad_per_partition
    want = derivatives.EdgeDerivativeOracle(orc).gradient_per_partition()
    assert np.abs(gpp - want).max() <= 1e-8 * max(1.0, float(np.abs(want).max()))
    h = 1e-6
    for p in range(len(orc.parts)):
        for e in (0, 3, 7):
            t = orc.part_brlen[p][e]
            orc.part_brlen[p][e] = t + h
            up = orc.loglikelihood()
            orc.part_brlen[p][e] = t - h
            dn = orc.loglikelihood()
            orc.part_brlen[p][e] = t
            assert want[p][e] == pytest.approx((up - dn) / (2 * h), rel=1e-4, abs=1e-4)
