"""GPU: branch-length linkage (the reference's --brlen linked / unlinked /
scaled, src/main.cpp:101,226-230) through the C ABI against the oracle.

* Unlinked lengths equal to the linked ones give the linked context's logL
  and gradient bit for bit.
* Different lengths per partition: logL against the oracle (FP64 1e-9, FP32
  1e-6), the per-partition gradient against the oracle's adjoint and the
  gradient as its column sums, the per-partition analytic edge derivatives
  (the NR callback's df[p], ddf[p]) against the sumtable derivatives (FP64
  1e-8), incremental evaluation after one partition's lengths change equal
  to a fresh context, and netlk_edge_loglikelihood_partition equal to
  setting the length and evaluating.
* Scaled: scalers s_p give the logL of unlinked lengths s_p t bit for bit;
  the gradient w.r.t. t is sum_p s_p x the partition gradient; the scaler
  gradient sum_e t_e x row p matches central differences.
"""
import numpy as np
import pytest

from conftest import GoldenPartition, golden_cases

pytestmark = pytest.mark.gpu

CASES = {c["name"]: c for c in golden_cases()}
NAMES = ["synthetic_12taxa_3ret_2parts", "synthetic_16taxa_4ret_3parts"]


def _lik(name, precision, linkage="linked"):
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    net = parse_extended_newick(CASES[name]["newick"])
    parts = [GoldenPartition(d) for d in CASES[name]["partitions"]]
    return NetworkLikelihood(net, parts, precision=precision, brlen_linkage=linkage)


def _lengths(lik, seed):
    rng = np.random.default_rng(seed)
    base = lik.branch_lengths
    return [np.clip(base * np.exp(0.3 * rng.standard_normal(base.size)), 1e-6, 100.0) for _ in range(lik.n_parts)]


def _oracle(name, part_lengths):
    from oracle import improved, newick, pllmath
    parts = []
    for d in CASES[name]["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4)))
    orc = improved.ImprovedOracle(newick.parse_newick(CASES[name]["newick"]), parts)
    orc.part_brlen = [list(x) for x in part_lengths]
    orc.loglikelihood()
    return orc


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_unlinked_equal_lengths_match_linked(precision):
    name = NAMES[0]
    with _lik(name, precision) as a, _lik(name, precision, "unlinked") as b:
        ta, ga, ra = a.loglikelihood_gradient()
        tb, gb, rb = b.loglikelihood_gradient()
        assert ta == tb and np.array_equal(ga, gb) and np.array_equal(ra, rb)
        gp = b.partition_gradient()
        assert np.allclose(gp.sum(axis=0), gb, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_unlinked_lengths_match_the_oracle(name, precision):
    from oracle import derivatives, sweep
    tol, gtol = (1e-9, 1e-8) if precision == "fp64" else (1e-6, 1e-5)
    with _lik(name, precision, "unlinked") as lik:
        L = _lengths(lik, 11)
        for p, x in enumerate(L):
            lik.set_partition_branch_lengths(p, x)
        orc = _oracle(name, L)
        so = sweep.SweepOracle(orc)
        want, _, _, g, _ = so.evaluate()
        tot, gb, _ = lik.loglikelihood_gradient()
        assert tot == pytest.approx(want, rel=tol)
        gp = lik.partition_gradient()
        scale = max(1.0, float(np.abs(so.grad_per_partition).max()))
        assert np.abs(gp - so.grad_per_partition).max() <= gtol * scale
        assert np.abs(gb - gp.sum(axis=0)).max() <= 1e-9 * scale
        if precision == "fp64":
            d = derivatives.EdgeDerivativeOracle(orc)
            for e in range(0, lik.n_edges, 4):
                for p in range(lik.n_parts):
                    w1, w2 = d.edge(e, partitions=[p])
                    d1, d2 = lik.edge_derivatives_partition(e, p)
                    assert d1 == pytest.approx(w1, rel=1e-8, abs=1e-8)
                    assert d2 == pytest.approx(w2, rel=1e-8, abs=1e-7)
        # one partition's lengths change: incremental == a fresh context
        L[1] = L[1] * 1.1
        lik.set_partition_branch_lengths(1, L[1])
        inc = lik.loglikelihood()
        assert lik.last_site_updates() > 0
        with _lik(name, precision, "unlinked") as fresh:
            for p, x in enumerate(L):
                fresh.set_partition_branch_lengths(p, x)
            assert fresh.loglikelihood() == inc
            e = 5
            v = lik.edge_loglikelihood_partition(e, 0, 0.123)
            L[0][e] = 0.123
            fresh.set_partition_branch_lengths(0, L[0])
            assert fresh.loglikelihood() == v


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_scaled_lengths(precision):
    name = NAMES[1]
    with _lik(name, precision, "scaled") as sc, _lik(name, precision, "unlinked") as un:
        s = np.array([0.5, 1.7, 1.1][:sc.n_parts])
        t = sc.branch_lengths.copy()
        sc.set_branch_length_scalers(s)
        for p in range(un.n_parts):
            un.set_partition_branch_lengths(p, s[p] * t)
        ts, gs, rs = sc.loglikelihood_gradient()
        tu, gu, ru = un.loglikelihood_gradient()
        assert ts == tu and np.array_equal(rs, ru)
        gp = sc.partition_gradient()
        want = (s[:, None] * gp).sum(axis=0)
        assert np.abs(gs - want).max() <= 1e-9 * max(1.0, float(np.abs(want).max()))
        if precision == "fp64":
            ds = (gp * t[None, :]).sum(axis=1)  # d logL / d s_p
            h = 1e-6
            for p in range(sc.n_parts):
                up = s.copy()
                up[p] += h
                sc.set_branch_length_scalers(up)
                lu = sc.loglikelihood()
                up[p] -= 2 * h
                sc.set_branch_length_scalers(up)
                ld = sc.loglikelihood()
                assert ds[p] == pytest.approx((lu - ld) / (2 * h), rel=1e-5, abs=1e-4)
            sc.set_branch_length_scalers(s)
            d1, d2 = sc.edge_derivatives(3)
            assert d1 == pytest.approx(gs[3], rel=1e-9, abs=1e-9)
