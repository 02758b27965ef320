"""netlk_set_model: the hook the model optimizer calls with new parameters.

The reference re-runs pllmod_treeinfo_update_prob_matrices after its model
optimizer (pllmod_algo_opt_*, src/optimization/ModelOptimization.cpp:25-97)
changes frequencies, exchangeabilities or the Gamma shape of a partition;
netlk_set_model takes the new parameters, validates them on the host and
re-derives the eigensystem, rates and P-matrices at the next evaluation.

* CPU (host-only context): invalid parameters are rejected with
  NETLK_ERR_INVALID_ARGUMENT and a message; valid ones are accepted.
* GPU: after set_model a context gives exactly the log-likelihood and
  gradient of a context created with the new model, and the oracle's
  log-likelihood for it (FP64 1e-9, FP32 1e-6).
"""
import copy

import numpy as np
import pytest

from conftest import GoldenPartition, golden_cases

CASE = [c for c in golden_cases() if c["name"] == "synthetic_12taxa_3ret_2parts"][0]
NEW_FREQS = [0.1, 0.2, 0.3, 0.4]
NEW_EXCH = [0.5, 3.0, 1.0, 0.7, 2.5, 1.3]
NEW_ALPHA = 0.35


def _net_parts():
    from netrax_gb300.network import parse_extended_newick
    return parse_extended_newick(CASE["newick"]), [GoldenPartition(d) for d in CASE["partitions"]]


def test_set_model_validates_its_arguments():
    from netrax_gb300 import _native
    from netrax_gb300.likelihood import NetworkLikelihood
    net, parts = _net_parts()
    with NetworkLikelihood(net, parts, host_only=True) as lik:
        lik.set_model(1, NEW_FREQS, NEW_EXCH, NEW_ALPHA)
        lik.set_model(0, NEW_FREQS, NEW_EXCH, -1.0, rates=[0.2, 0.6, 1.2, 2.0])  # explicit rates: alpha unused
        bad = [
            (2, NEW_FREQS, NEW_EXCH, NEW_ALPHA, "partition"),
            (0, [0.0, 0.3, 0.3, 0.4], NEW_EXCH, NEW_ALPHA, "frequencies"),
            (0, NEW_FREQS, [1.0, -1.0, 1.0, 1.0, 1.0, 1.0], NEW_ALPHA, "exchangeabilities"),
            (0, NEW_FREQS, [1.0, float("nan"), 1.0, 1.0, 1.0, 1.0], NEW_ALPHA, "exchangeabilities"),
            (0, NEW_FREQS, NEW_EXCH, 0.0, "alpha"),
            (0, NEW_FREQS, NEW_EXCH, float("inf"), "alpha"),
        ]
        for part, f, x, a, word in bad:
            with pytest.raises(_native.NetlkError) as e:
                lik.set_model(part, f, x, a)
            assert e.value.status == _native.NETLK_ERR_INVALID_ARGUMENT
            assert word in str(e.value)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_set_model_equals_a_fresh_context_and_the_oracle(precision):
    from netrax_gb300.likelihood import NetworkLikelihood
    from oracle import improved, newick, pllmath
    net, parts = _net_parts()
    new_parts = copy.deepcopy(parts)
    new_parts[1].freqs = np.array(NEW_FREQS)
    new_parts[1].exch = np.array(NEW_EXCH)
    new_parts[1].alpha = NEW_ALPHA
    with NetworkLikelihood(net, parts, precision=precision) as lik:
        t0, _, _ = lik.loglikelihood_gradient()
        lik.set_model(1, NEW_FREQS, NEW_EXCH, NEW_ALPHA)
        t1, g1, r1 = lik.loglikelihood_gradient()
        l1 = lik.loglikelihood()
    with NetworkLikelihood(net, new_parts, precision=precision) as fresh:
        t2, g2, r2 = fresh.loglikelihood_gradient()
    assert t1 != t0
    assert t1 == t2 and l1 == t1
    assert np.array_equal(g1, g2) and np.array_equal(r1, r2)
    oparts = [improved.Partition(p.tip_states, p.weights, p.freqs, p.exch, pllmath.gamma_rates_mean(p.alpha, 4))
              for p in new_parts]
    want = improved.ImprovedOracle(newick.parse_newick(CASE["newick"]), oparts).loglikelihood()
    assert t1 == pytest.approx(want, rel=1e-9 if precision == "fp64" else 1e-6)


def test_reference_formula_refuses_scaled_lengths():
    """Mode 1 (the reference's derivative formula) on a scaled-linkage
    context returns NETLK_ERR_UNSUPPORTED before any device work, as the
    reference throws for scaled lengths (LikelihoodDerivatives.cpp:42-46);
    the sumtable entry refuses the same way."""
    from netrax_gb300 import _native
    from netrax_gb300.likelihood import NetworkLikelihood
    net, parts = _net_parts()
    with NetworkLikelihood(net, parts, host_only=True, brlen_linkage="scaled") as lik:
        for call in (lambda: lik.edge_derivatives(0, mode=1), lambda: lik.edge_derivatives_partition(0, 0, mode=1),
                     lambda: lik.edge_sumtable_derivatives(0, 0.1, mode=1)):
            with pytest.raises(_native.NetlkError) as e:
                call()
            assert e.value.status == 7 and "scaled" in str(e.value)
