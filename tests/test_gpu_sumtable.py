"""GPU: edge sumtables for the Newton-Raphson iterations along one edge
(``netlk_edge_sumtable`` / ``netlk_edge_sumtable_derivatives``; the
reference's computePartitionSumtables + pll_compute_loglikelihood_derivatives,
src/likelihood/LikelihoodDerivatives.cpp:95-104,249-344).

* At the current length the tables give the context's own logL and its
  analytic edge derivatives (tangent sweep): FP64 within 1e-11 / 1e-9,
  FP32 within 1e-6 relative.
* At other lengths, from the clamp (1e-6) to 10x the current one, the logL
  and derivatives equal an FP64 context set to that length: FP64 within
  1e-9 relative (d2 1e-8), FP32 logL within 1e-6 and derivatives within
  1e-4 of the gradient's scale; the context's own parameters and logL are
  left as they were.
* Unlinked lengths, one per partition: each partition's logL and df[p],
  ddf[p] against the oracle with those lengths; scaled lengths: the totals
  equal the unlinked evaluation at s_p t.
* +I; both mixtures and both derivative modes; tables rebuilt after another
  edge's length, the model or the probabilities change; 20-state tables
  (reverse walks down each tree's path) against the tangent sweep.
* The reference's Newton-Raphson pass driven by table evaluations ends where
  the same pass on the oracle ends.
"""
import numpy as np
import pytest

import optimizer_loops as opt
from conftest import GoldenPartition, golden_cases

pytestmark = pytest.mark.gpu

CASES = {c["name"]: c for c in golden_cases()}


def _lik(name, precision="fp64", variant="AVERAGE", linkage="linked", pinv=None, **kw):
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    net = parse_extended_newick(CASES[name]["newick"])
    parts = [GoldenPartition(d) for d in CASES[name]["partitions"]]
    if pinv is not None:
        for p in parts:
            p.prop_invar = pinv
    return NetworkLikelihood(net, parts, precision=precision, variant=variant, brlen_linkage=linkage, **kw)


def _scale(lik):
    _, g, _ = lik.loglikelihood_gradient()
    return max(1.0, float(np.abs(g).max()))


@pytest.mark.parametrize("name", ["twoReticulations", "celineNetwork", "synthetic_16taxa_4ret_3parts",
                                  "synthetic_200taxa_2ret_deep"])
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("mode", [0, 1])
def test_tables_at_the_current_length(name, variant, mode):
    with _lik(name, "fp64", variant) as ref:
        scale = _scale(ref)
        want = {e: ref.edge_derivatives(e, second=True, mode=mode)
                for e in range(0, ref.n_edges, max(1, ref.n_edges // 12))}
        for precision, tl, td1, td2 in (("fp64", 1e-11, 1e-9, 1e-8), ("fp32", 1e-6, 1e-5, 1e-4)):
            with _lik(name, precision, variant) as lik:
                base = lik.loglikelihood()
                for e, (want1, want2) in want.items():
                    assert lik.edge_sumtable(e)[0]
                    l, d1, d2 = lik.edge_sumtable_derivatives(e, ref.branch_lengths[e], mode=mode)
                    assert l == pytest.approx(base, rel=tl)
                    assert abs(d1 - want1) <= td1 * scale, (precision, e, d1, want1)
                    assert abs(d2 - want2) <= td2 * max(scale, abs(want2)), (precision, e, d2, want2)


@pytest.mark.parametrize("name", ["smallNetwork", "threeReticulations", "synthetic_12taxa_3ret_2parts"])
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_tables_at_other_lengths(name, variant):
    with _lik(name, "fp64", variant) as ref, _lik(name, "fp64", variant) as a, _lik(name, "fp32", variant) as b:
        base_a, base_b = a.loglikelihood(), b.loglikelihood()
        scale = _scale(ref)
        for e in range(0, ref.n_edges, max(1, ref.n_edges // 8)):
            t0 = ref.branch_lengths[e]
            for t in (1e-6, 0.3 * t0, 3.0 * t0, 10.0 * t0 + 0.01):
                want_l = ref.edge_loglikelihood(e, t)
                w1, w2 = ref.edge_derivatives(e, second=True, mode=0)
                l, d1, d2 = a.edge_sumtable_derivatives(e, t)
                assert l == pytest.approx(want_l, rel=1e-9), (e, t)
                assert d1 == pytest.approx(w1, rel=1e-9, abs=1e-9 * scale), (e, t)
                assert d2 == pytest.approx(w2, rel=1e-8, abs=1e-8 * scale), (e, t)
                l, d1, d2 = b.edge_sumtable_derivatives(e, t)
                assert l == pytest.approx(want_l, rel=1e-6), (e, t)
                assert abs(d1 - w1) <= 1e-4 * max(scale, abs(w1)), (e, t, d1, w1)
                assert abs(d2 - w2) <= 1e-4 * max(scale, abs(w2)), (e, t, d2, w2)
            ref.edge_loglikelihood(e, t0)
        # nothing was kept
        assert a.loglikelihood() == base_a and b.loglikelihood() == base_b


def test_unlinked_and_scaled_tables_match_the_oracle():
    from oracle import derivatives, improved, newick, pllmath
    name = "synthetic_16taxa_4ret_3parts"
    parts = []
    for d in CASES[name]["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4)))
    orc = improved.ImprovedOracle(newick.parse_newick(CASES[name]["newick"]), parts)
    rng = np.random.default_rng(3)
    base = np.array(orc.brlen)
    L = [np.clip(base * np.exp(0.3 * rng.standard_normal(base.size)), 1e-6, 100.0) for _ in parts]
    with _lik(name, "fp64", linkage="unlinked") as un, _lik(name, "fp64", linkage="scaled") as sc:
        for p, x in enumerate(L):
            un.set_partition_branch_lengths(p, x)
        for e in (0, 5, 11):
            prop = np.array([0.05, 0.4, 1.3])
            l, d1, d2 = un.edge_sumtable_derivatives(e, prop)
            orc.part_brlen = [list(x) for x in L]
            for p in range(len(parts)):
                orc.part_brlen[p][e] = prop[p]
            orc.loglikelihood()
            want_parts = orc.evaluate()[1]
            assert np.allclose(l, want_parts, rtol=1e-9, atol=0)
            d = derivatives.EdgeDerivativeOracle(orc)
            for p in range(len(parts)):
                w1, w2 = d.edge(e, partitions=[p])
                assert d1[p] == pytest.approx(w1, rel=1e-8, abs=1e-8)
                assert d2[p] == pytest.approx(w2, rel=1e-8, abs=1e-7)
        s = np.array([0.5, 1.7, 1.1])
        sc.set_branch_length_scalers(s)
        t = sc.branch_lengths
        with _lik(name, "fp64", linkage="unlinked") as un2:
            for p in range(3):
                un2.set_partition_branch_lengths(p, s[p] * t)
            for e in (2, 7):
                l, d1, d2 = sc.edge_sumtable_derivatives(e, 0.2)
                lu, du1, du2 = un2.edge_sumtable_derivatives(e, s * 0.2)
                assert l == pytest.approx(lu.sum(), rel=1e-12)
                assert d1 == pytest.approx((s * du1).sum(), rel=1e-10, abs=1e-10)
                assert d2 == pytest.approx((s * s * du2).sum(), rel=1e-10, abs=1e-10)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_invariant_sites(precision):
    name = "synthetic_12taxa_3ret_2parts"
    with _lik(name, precision, pinv=0.2) as a, _lik(name, "fp64", pinv=0.2) as ref:
        scale = _scale(ref)
        for e in (1, 6, 13):
            for t in (1e-6, 0.05, 0.7):
                want_l = ref.edge_loglikelihood(e, t)
                w1, w2 = ref.edge_derivatives(e, second=True)
                l, d1, d2 = a.edge_sumtable_derivatives(e, t)
                tol = 1e-9 if precision == "fp64" else 1e-4
                assert l == pytest.approx(want_l, rel=1e-9 if precision == "fp64" else 1e-6)
                assert abs(d1 - w1) <= tol * max(scale, abs(w1))
                assert abs(d2 - w2) <= tol * max(scale, abs(w2))
            ref.edge_loglikelihood(e, a.branch_lengths[e])


def test_tables_rebuilt_when_parameters_change():
    name = "threeReticulations"
    with _lik(name) as a, _lik(name) as fresh:
        e = 3
        a.edge_sumtable_derivatives(e, 0.2)
        b = a.branch_lengths.copy()
        b[5] *= 1.7
        a.set_branch_lengths(b)
        fresh.set_branch_lengths(b)
        assert a.edge_sumtable_derivatives(e, 0.2) == fresh.edge_sumtable_derivatives(e, 0.2)
        p = np.clip(a.ret_probs * 0.8 + 0.05, 0.01, 0.99)
        a.set_reticulation_probs(p)
        fresh.set_reticulation_probs(p)
        assert a.edge_sumtable_derivatives(e, 0.2) == fresh.edge_sumtable_derivatives(e, 0.2)
        gp = GoldenPartition(CASES[name]["partitions"][0])
        for lik in (a, fresh):
            lik.set_model(0, gp.freqs, gp.exch * 1.3, gp.alpha * 0.7)
        assert a.edge_sumtable_derivatives(e, 0.2) == fresh.edge_sumtable_derivatives(e, 0.2)
        # this edge's own length moves: the tables stay current and agree
        a.edge_loglikelihood(e, 0.9)
        fresh.edge_loglikelihood(e, 0.9)
        assert a.edge_sumtable_derivatives(e, 0.3) == pytest.approx(fresh.edge_sumtable_derivatives(e, 0.3),
                                                                      rel=1e-12)


@pytest.mark.parametrize("name", ["protein_8taxa_2ret", "protein_10taxa_3ret_2parts"])
def test_protein_tables_match_the_tangent_path(name):
    """20-state tables (reverse walks down each tree's path to the edge)
    against an FP64 context set to the proposal with the tangent sweep:
    logL FP64 1e-10 / FP32 1e-6, d1 and d2 FP64 1e-8 / FP32 1e-4 of the
    gradient scale; the tables' context keeps its own parameters."""
    for precision, tl, td in (("fp64", 1e-10, 1e-8), ("fp32", 1e-6, 1e-4)):
        with _lik(name, precision) as a, _lik(name, "fp64", sumtables=False) as ref:
            base = a.loglikelihood()
            assert a.edge_sumtable(2)[0]
            scale = _scale(ref)
            for e in (2, 5, 7):
                t0 = ref.branch_lengths[e]
                for t in (1e-6, 0.35 * t0 + 0.01, 2.0):
                    want_l = ref.edge_loglikelihood(e, t)
                    w1, w2 = ref.edge_derivatives(e, second=True)
                    l, d1, d2 = a.edge_sumtable_derivatives(e, t)
                    assert l == pytest.approx(want_l, rel=tl), (precision, e, t)
                    assert abs(d1 - w1) <= td * max(scale, abs(w1)), (precision, e, t, d1, w1)
                    assert abs(d2 - w2) <= td * max(scale, abs(w2)), (precision, e, t, d2, w2)
                ref.edge_loglikelihood(e, t0)
            assert a.loglikelihood() == base


@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_newton_raphson_pass_on_tables_matches_the_oracle(variant):
    from oracle import derivatives, improved, newick, pllmath
    name = "synthetic_12taxa_3ret_2parts"
    parts = []
    for d in CASES[name]["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4)))
    orc = improved.ImprovedOracle(newick.parse_newick(CASES[name]["newick"]), parts, variant=variant)
    orc.loglikelihood()

    def orc_logl(e, t):
        orc.brlen[e] = t
        return orc.loglikelihood()

    want_len, want_logl, _ = opt.optimize_branches(
        orc_logl, lambda e: derivatives.EdgeDerivativeOracle(orc).edge(e, mode="reference"), list(orc.brlen))
    # lengths: relative, or absolute within the NR stopping tolerance (1e-7)
    # in FP32, whose derivatives near the 1e-6 clamp carry ~1e-4 relative noise
    for precision, rel_len, abs_len, rel_logl in (("fp64", 1e-6, 1e-9, 1e-9), ("fp32", 1e-4, opt.NR_TOLERANCE, 1e-6)):
        with _lik(name, precision, variant) as lik:
            def at(e, t):
                return lik.edge_sumtable_derivatives(e, t, mode=1)[1:]

            lengths, logl, worse = opt.optimize_branches(lik.edge_loglikelihood, None, lik.branch_lengths,
                                                         derivs_at=at)
            assert not worse
            assert logl == pytest.approx(want_logl, rel=rel_logl)
            a, b = np.array(lengths), np.array(want_len)
            assert np.all(np.abs(a - b) <= np.maximum(abs_len, rel_len * np.abs(b))), precision


def test_unsupported_contexts_and_failures():
    """Contexts the tables do not serve report NETLK_ERR_UNSUPPORTED and stay
    usable; a failure injected into an evaluation surfaces with its status,
    drops the tables (they read the edge's child CLV on every evaluation) and
    the next call rebuilds them with the same results."""
    from netrax_gb300 import _native as N
    name = "threeReticulations"
    with _lik(name) as ref:
        want = ref.edge_sumtable_derivatives(3, 0.2)
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    net = parse_extended_newick(CASES[name]["newick"])
    parts = [GoldenPartition(d) for d in CASES[name]["partitions"]]
    with NetworkLikelihood(net, parts, precision="fp64", checkpoint_segments=2) as ck:
        base = ck.loglikelihood()
        assert ck.edge_sumtable(3) == (False, 0)
        with pytest.raises(N.NetlkError) as ei:
            ck.edge_sumtable_derivatives(3, 0.2)
        assert ei.value.status == 7  # UNSUPPORTED
        assert ck.loglikelihood() == base
    with _lik(name) as lik:
        assert lik.edge_sumtable(3)[0]
        N.check(N.lib().netlk_inject_failure(lik._h, N.NETLK_ERR_TIMEOUT))
        with pytest.raises(N.NetlkError) as ei:
            lik.edge_sumtable_derivatives(3, 0.2)
        assert ei.value.status == N.NETLK_ERR_TIMEOUT
        assert lik.edge_sumtable_derivatives(3, 0.2) == want


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_brent_branch_pass_on_tables_matches_the_oracle(precision):
    """The reference's Brent branch-length pass (BRENT_REROOT: every probe an
    edge log-likelihood) with each probe one table evaluation, against the
    same pass on the oracle: FP64 final lengths within 1e-4 relative or 1e-6
    absolute and final logL within 1e-9; FP32 (noisier probes) final logL
    within 1e-4; the pass never lowers the logL."""
    from oracle import improved, newick, pllmath
    name = "twoReticulations"
    parts = []
    for d in CASES[name]["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4)))
    orc = improved.ImprovedOracle(newick.parse_newick(CASES[name]["newick"]), parts)
    orc.loglikelihood()

    def orc_at(e, t):
        t0 = orc.brlen[e]
        orc.brlen[e] = t
        v = orc.loglikelihood()
        orc.brlen[e] = t0
        return v

    def orc_set(e, t):
        orc.brlen[e] = t
        return orc.loglikelihood()

    tol = 1e-7
    want_len, want_logl = opt.optimize_branches_brent(orc_at, orc_set, list(orc.brlen), tol)
    with _lik(name, precision) as lik:
        start = lik.loglikelihood()
        lengths, logl = opt.optimize_branches_brent(lambda e, t: lik.edge_sumtable_derivatives(e, t)[0],
                                                    lik.edge_loglikelihood, lik.branch_lengths, tol)
        assert logl >= start
        if precision == "fp64":
            assert logl == pytest.approx(want_logl, rel=1e-9)
            a, b = np.array(lengths), np.array(want_len)
            assert np.all(np.abs(a - b) <= np.maximum(1e-6, 1e-4 * np.abs(b))), np.abs(a - b).max()
        else:
            # FP32 probes carry ~1e-7 relative noise, so Brent settles at
            # slightly different points on flat edges (here a few 1e-3 of logL
            # on a -85.8 network, in either direction)
            assert logl == pytest.approx(want_logl, rel=1e-4)
