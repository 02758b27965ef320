"""Edge cases of the network likelihood against the oracle: the smallest
tree, one-pattern and all-gap partitions, zero-weight patterns, clamped
lengths and probabilities, many small partitions, ten reticulations."""
import math

import numpy as np
import pytest

from netrax_gb300 import synth
from netrax_gb300.network import parse_extended_newick

pytestmark = pytest.mark.gpu

FP64_REL = 1e-9
FP32_REL = 1e-6


def _parts(rng, n_tips, sizes, gaps=False):
    out = []
    for n in sizes:
        codes = (1 << rng.integers(0, 4, size=(n_tips, n))).astype(np.uint32)
        if gaps:
            codes[:] = 15
        freqs = rng.dirichlet(np.ones(4))
        exch = rng.dirichlet(np.ones(6)) * 6
        out.append(synth.PartitionData(codes, np.ones(n), freqs, exch, 0.7, n))
    return out


def _oracle(text, parts, variant):
    from oracle import improved, newick, pllmath
    net = newick.parse_newick(text)
    ps = [improved.Partition(p.tip_states, p.weights, p.freqs, p.exch, pllmath.gamma_rates_mean(p.alpha, 4))
          for p in parts]
    return improved.ImprovedOracle(net, ps, variant=variant).loglikelihood()


def _check(text, parts, variant="AVERAGE"):
    from netrax_gb300.likelihood import NetworkLikelihood
    net = parse_extended_newick(text)
    want = _oracle(text, parts, variant)
    sites = sum(p.n_sites for p in parts)
    # FP32 rounds each site likelihood at ~1e-7 relative: where logL is near
    # zero (all-gap columns) that is an absolute error of ~1e-7 per site
    for prec, tol, atol in (("fp64", FP64_REL, 1e-12), ("fp32", FP32_REL, 2e-7 * sites)):
        with NetworkLikelihood(net, parts, variant=variant, precision=prec) as lik:
            got = lik.loglikelihood()
            assert got == pytest.approx(want, rel=tol, abs=atol)
    return want


def test_three_taxon_tree():
    rng = np.random.default_rng(0)
    _check("((A:0.1,B:0.2):0.05,C:0.3);", _parts(rng, 3, [5]))


@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_one_pattern_and_many_small_partitions(variant):
    rng = np.random.default_rng(1)
    text = synth.random_network_newick(rng, 9, 2)
    sizes = [1, 2, 3, 5, 8, 13, 21, 34, 40, 1, 7, 16]
    _check(text, _parts(rng, 9, sizes), variant)


def test_all_gap_partition_has_zero_loglikelihood():
    rng = np.random.default_rng(2)
    text = synth.random_network_newick(rng, 7, 1)
    want = _check(text, _parts(rng, 7, [11], gaps=True))
    assert abs(want) < 1e-12


def test_zero_weight_patterns_are_ignored():
    from netrax_gb300.likelihood import NetworkLikelihood
    rng = np.random.default_rng(3)
    text = synth.random_network_newick(rng, 8, 2)
    net = parse_extended_newick(text)
    p = _parts(rng, 8, [30])[0]
    w = p.weights.copy()
    w[::3] = 0.0
    zero = synth.PartitionData(p.tip_states, w, p.freqs, p.exch, p.alpha, p.n_sites)
    keep = w > 0
    dropped = synth.PartitionData(np.ascontiguousarray(p.tip_states[:, keep]), w[keep], p.freqs, p.exch,
                                  p.alpha, int(keep.sum()))
    with NetworkLikelihood(net, [zero], precision="fp64") as a, \
            NetworkLikelihood(net, [dropped], precision="fp64") as b:
        assert a.loglikelihood() == pytest.approx(b.loglikelihood(), rel=1e-14)


def test_lengths_and_probabilities_are_clamped_like_the_reference():
    """Branch lengths clamp to [1e-6, 100] and reticulation probabilities to
    [1e-6, 1 - 1e-6] (RaxmlWrapper.cpp brlen_min/max, NetraxOptions brprob bounds)."""
    from netrax_gb300.likelihood import NetworkLikelihood
    rng = np.random.default_rng(4)
    text = synth.random_network_newick(rng, 10, 2)
    net = parse_extended_newick(text)
    parts = _parts(rng, 10, [25])
    with NetworkLikelihood(net, parts, precision="fp64") as lik:
        b = net.branch_lengths.copy()
        b[0], b[1] = 0.0, 1000.0
        lik.set_branch_lengths(b)
        lik.set_reticulation_probs(np.array([0.0, 1.0]))
        l0 = lik.loglikelihood()
        b[0], b[1] = 1e-6, 100.0
        lik.set_branch_lengths(b)
        lik.set_reticulation_probs(np.array([1e-6, 1.0 - 1e-6]))
        assert lik.loglikelihood() == l0


def test_ten_reticulations():
    rng = np.random.default_rng(5)
    text = synth.random_network_newick(rng, 14, 10)
    _check(text, _parts(rng, 14, [20]))


@pytest.mark.parametrize("states,rate_cats", [(4, 1), (4, 2), (4, 8), (20, 1), (20, 2)])
def test_rate_category_counts(states, rate_cats):
    """Rate-category counts other than 4 (DNA 1/2/8, protein 1/2; the
    CUDA-core sweeps) against the oracle, with a finite gradient, and the
    edge sumtables (DNA: build walk and bulk-copy evaluation; 20 states:
    reverse path walks and their evaluation, for this rate count) at a
    proposed length against the oracle's logL and sumtable derivatives
    there."""
    from netrax_gb300.likelihood import NetworkLikelihood
    from oracle import derivatives, improved, newick, pllmath
    rng = np.random.default_rng(10 + states + rate_cats)
    text = synth.random_network_newick(rng, 10, 2)
    n = 60
    codes = (1 << rng.integers(0, states, size=(10, n))).astype(np.uint32)
    freqs = rng.dirichlet(np.ones(states))
    exch = rng.gamma(1.0, 1.0, size=states * (states - 1) // 2) + 1e-3
    part = synth.PartitionData(codes, np.ones(n), freqs, exch, 0.6, n, rate_cats=rate_cats, states=states)
    opart = improved.Partition(codes, np.ones(n), freqs, exch, pllmath.gamma_rates_mean(0.6, rate_cats))
    orc = improved.ImprovedOracle(newick.parse_newick(text), [opart], variant="AVERAGE")
    want = orc.loglikelihood()
    net = parse_extended_newick(text)
    stab_want = {}
    g_scale = max(1.0, float(np.abs(derivatives.EdgeDerivativeOracle(orc).gradient()[0]).max()))
    for e in (0, 3):
        t0 = orc.brlen[e]
        orc.brlen[e] = 0.5 * t0 + 0.02
        stab_want[e] = (orc.loglikelihood(),) + tuple(derivatives.EdgeDerivativeOracle(orc).edge(e))
        orc.brlen[e] = t0
        orc.loglikelihood()
    for prec, tol in (("fp64", FP64_REL), ("fp32", FP32_REL)):
        with NetworkLikelihood(net, [part], precision=prec) as lik:
            got, gb, gr = lik.loglikelihood_gradient()
            assert got == pytest.approx(want, rel=tol)
            assert np.all(np.isfinite(gb)) and np.all(np.isfinite(gr))
            dtol = 1e-8 if prec == "fp64" else 1e-4
            for e, (wl, w1, w2) in stab_want.items():
                l, d1, d2 = lik.edge_sumtable_derivatives(e, 0.5 * net.branch_lengths[e] + 0.02)
                assert l == pytest.approx(wl, rel=tol)
                assert abs(d1 - w1) <= dtol * max(g_scale, abs(w1)), (prec, e, d1, w1)
                assert abs(d2 - w2) <= dtol * max(g_scale, abs(w2)), (prec, e, d2, w2)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_failed_evaluation_forgets_the_stored_clvs(precision):
    """An evaluation that fails after its kernels ran (a timed-out device
    wait, a CUDA error) may leave the stored CLVs partial, so it must not
    leave them marked valid: the next edge evaluation has to run the full
    forward sweep instead of an incremental one over them. The failure is
    injected on the host (netlk_inject_failure); nothing faults on the GPU."""
    from netrax_gb300 import _native as N
    from netrax_gb300.likelihood import NetworkLikelihood
    rng = np.random.default_rng(6)
    text = synth.random_network_newick(rng, 10, 2)
    net = parse_extended_newick(text)
    parts = _parts(rng, 10, [40])
    with NetworkLikelihood(net, parts, precision=precision) as lik, \
            NetworkLikelihood(net, parts, precision=precision) as fresh:
        lik.loglikelihood()
        full = lik.last_site_updates()
        lik.edge_loglikelihood(0, net.branch_lengths[0] * 1.5)
        assert lik.last_site_updates() < full  # incremental while nothing failed
        N.check(N.lib().netlk_inject_failure(lik._h, N.NETLK_ERR_TIMEOUT))
        with pytest.raises(N.NetlkError) as ei:
            lik.edge_loglikelihood(1, net.branch_lengths[1] * 1.5)
        assert ei.value.status == N.NETLK_ERR_TIMEOUT
        got = lik.edge_loglikelihood(2, net.branch_lengths[2] * 1.5)
        assert lik.last_site_updates() == full
        b = net.branch_lengths.copy()
        b[0] *= 1.5
        b[1] *= 1.5
        b[2] *= 1.5
        fresh.set_branch_lengths(b)
        assert got == fresh.loglikelihood()
