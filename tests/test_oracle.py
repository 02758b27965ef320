"""The CPU oracle against the reference's own invariants and the golden fixtures.

Reference test invariants restated (test/src/LikelihoodTest.cpp):
* repeated evaluations are identical (:204-255, EXPECT_DOUBLE_EQ);
* the improved displayed-tree DAG agrees with the naive per-tree evaluation
  (:241 allows 10 log units; the restatement agrees to ~1e-8);
* trees (no reticulation) give one displayed tree.
"""
import math

import numpy as np
import pytest

from conftest import GoldenPartition, golden_cases, load_golden
from oracle import improved, naive, newick, pllmath

CASES = golden_cases()


def _oracle(case, variant):
    net = newick.parse_newick(case["newick"])
    parts = []
    for d in case["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4)))
    return improved.ImprovedOracle(net, parts, variant=variant)


@pytest.mark.parametrize("case", [c for c in CASES if c["name"] != "synthetic_200taxa_2ret_deep"],
                         ids=lambda c: c["name"])
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_oracle_matches_golden_and_naive(case, variant):
    orc = _oracle(case, variant)
    a = orc.loglikelihood()
    b = orc.loglikelihood()
    assert a == b  # repeated == repeated (LikelihoodTest.cpp:236-240)
    g = case[variant]
    assert a == pytest.approx(g["logl"], rel=1e-12, abs=1e-9)
    if "naive_logl" in g:
        nv = naive.naive_loglikelihood(orc)[0]
        assert nv == pytest.approx(g["naive_logl"], rel=1e-12)
        if variant == "AVERAGE":
            assert a == pytest.approx(nv, rel=1e-9)
        else:
            # BEST over merged displayed-tree sets vs single trees; identical here
            assert abs(a - nv) < 10.0  # LikelihoodTest.cpp:241 tolerance


def test_gamma_rates_mean_known_values():
    # mean of the categories is 1 and they are increasing (Yang 1994)
    r = pllmath.gamma_rates_mean(0.8, 4)
    assert r.mean() == pytest.approx(1.0, abs=1e-12)
    assert np.all(np.diff(r) > 0)
    r1 = pllmath.gamma_rates_mean(1.0, 4)
    # alpha = 1 (exponential): closed form of the category means
    q = np.array([0.0, math.log(4 / 3), math.log(2), math.log(4), math.inf])
    exact = []
    for k in range(4):
        a, b = q[k], q[k + 1]
        fa = (a + 1) * math.exp(-a)
        fb = 0.0 if math.isinf(b) else (b + 1) * math.exp(-b)
        exact.append(4 * (fa - fb))
    assert np.allclose(r1, exact, rtol=1e-12)


def test_pmatrix_identity_and_semigroup():
    lam, U, Ui, Q = pllmath.eigensystem([1, 2.5, .8, 1.2, 3, 1], [.2, .3, .3, .2])
    P = pllmath.pmatrices(lam, U, Ui, 0.0, [1.0])
    assert np.array_equal(P[0], np.eye(4))
    a = pllmath.pmatrix(lam, U, Ui, 0.13)
    b = pllmath.pmatrix(lam, U, Ui, 0.29)
    assert np.allclose(a @ b, pllmath.pmatrix(lam, U, Ui, 0.42), atol=1e-14)
    assert np.allclose(a.sum(axis=1), 1.0, atol=1e-14)


def test_tree_has_one_displayed_tree():
    case = [c for c in CASES if c["name"] == "smallTree"][0]
    orc = _oracle(case, "AVERAGE")
    orc.loglikelihood()
    assert len(orc.root_trees()) == 1


def test_reference_case_list_is_complete():
    names = {c["name"] for c in load_golden("reference_cases.json")["cases"]}
    assert {"tinyNetwork", "smallNetwork", "celineNetwork", "reticulationInReticulation",
            "interleavedReticulations", "threeReticulations"} <= names


def test_mixture_against_mpmath_high_precision():
    """AVERAGE mixture of the oracle vs an mpmath 200-bit evaluation."""
    import mpmath
    case = [c for c in CASES if c["name"] == "twoReticulations"][0]
    orc = _oracle(case, "AVERAGE")
    total = orc.loglikelihood()
    with mpmath.workprec(200):
        acc = mpmath.mpf(0)
        for t in orc.root_trees():
            acc += mpmath.exp(mpmath.mpf(t.logprob) + mpmath.mpf(t.partition_logl[0]))
        ref = float(mpmath.log(acc))
    assert total == pytest.approx(ref, rel=1e-15, abs=1e-12)


def test_protein_fixture_regenerates_byte_for_byte():
    """tests/golden/make_golden.py reproduces the committed 20-state fixture
    exactly (simulation, pattern compression, oracle scores, central-difference
    gradients): the fixture is the output of the committed script."""
    import json
    import os
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import make_golden
    fresh = json.loads(json.dumps(make_golden.protein_cases()))
    with open(os.path.join(GOLDEN, "protein_cases.json")) as f:
        assert fresh == json.load(f)["cases"]
