"""GPU parity at the full sizes of the benchmark workloads, through the C ABI,
against the CPU oracle.

The oracle here is ``improved.py``'s enumeration of the displayed-tree DAG (the
reference's processNodeImproved schedule on its own {-,0,1} configuration
sets) with ``sweep.c``'s FP64 pruning, mixture and adjoint
(``tests/test_oracle_sweep.py`` pins those against the per-variant oracle
and the reference's per-edge sumtable derivatives on the golden cases).

* 100 taxa / 8 reticulations / 100k DNA sites (88,315 patterns): logL total,
  per partition and per displayed tree, AVERAGE and BEST, FP64 within 1e-9
  and FP32 within 1e-6 relative; FP64 scale counters of every variant equal
  the oracle's pattern by pattern, also with branch lengths stretched until
  sites need rescaling; gradients.
* 50 taxa / 4 reticulations / 10 uneven DNA partitions (75.5k sites).
* 40 taxa / 3 reticulations / 50k protein sites on the tensor-core path.
* four candidates of the 64-network search-move batch, scored in one batch.

Gradient tolerances are relative to the largest entry: FP64 1e-8, FP32 1e-5.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_REL = 1e-9
FP32_REL = 1e-6
GRAD_TOL = {"fp64": 1e-8, "fp32": 1e-5}

_ORACLES = {}


def _sweep_oracle(key, workload):
    """One enumeration and one set of host buffers per workload, shared by
    the tests of this module (AVERAGE and BEST differ only in the mixture)."""
    if key not in _ORACLES:
        _ORACLES.clear()  # keep one workload's buffers (tens of GB) at a time
        from oracle import improved, newick, pllmath, sweep
        net = newick.parse_newick(workload.newick)
        parts = [improved.Partition(p.tip_states, p.weights, p.freqs, p.exch,
                                    pllmath.gamma_rates_mean(p.alpha, 4)) for p in workload.partitions]
        orc = improved.ImprovedOracle(net, parts, variant="AVERAGE")
        orc.loglikelihood()
        _ORACLES[key] = sweep.SweepOracle(orc)
    return _ORACLES[key]


def _oracle_eval(so, variant):
    so.orc.variant = variant
    total, parts, trees, g, gr = so.evaluate()
    per_root = []
    used = {id(t): i for i, t in enumerate(so.trees)}
    for t in so.orc.root_trees():
        per_root.append(trees[used[id(t)]] if id(t) in used else None)
    return total, parts, per_root, g, gr


def _workload(idx):
    from netrax_gb300 import synth
    return synth.config(idx)


def _check(lik, want, precision, gradient=True):
    tol = FP64_REL if precision == "fp64" else FP32_REL
    total, parts, per_root, g, gr = want
    got_total, got_parts, got_trees = lik.loglikelihood(details=True)
    assert got_total == pytest.approx(total, rel=tol)
    assert np.allclose(got_parts, parts, rtol=tol, atol=0)
    for k, t in enumerate(per_root):
        if t is None:
            assert np.all(np.isnan(got_trees[k]))
        else:
            assert np.allclose(got_trees[k], t, rtol=tol, atol=0), k
    if gradient:
        tot2, gb, gret = lik.loglikelihood_gradient()
        assert tot2 == got_total
        scale = max(1.0, float(np.abs(g).max()))
        assert np.abs(gb - g).max() <= GRAD_TOL[precision] * scale
        if len(gr):
            assert np.abs(gret - gr).max() <= GRAD_TOL[precision] * max(1.0, float(np.abs(gr).max()))


@pytest.fixture(scope="module")
def config2():
    return _workload(2)


@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_config2_full_size(config2, variant, precision):
    from netrax_gb300.likelihood import NetworkLikelihood
    so = _sweep_oracle(2, config2)
    want = _oracle_eval(so, variant)
    with NetworkLikelihood(config2.network, config2.partitions, variant=variant, precision=precision) as lik:
        assert lik.stats["n_variants"] == so.n_var
        _check(lik, want, precision)


@pytest.mark.parametrize("stretch", [1.0, 100.0])
def test_config2_fp64_scale_counters_bit_exact(config2, stretch):
    """Every variant's per-pattern scale counters (FP64, libpll's 2^-256 rule)
    equal the oracle's; GPU variants map to the oracle's per node, in order.
    With the generated branch lengths no site reaches 2^-256 (every counter
    is 0); with every length stretched 100x (clamped at 100) a few tenths of
    a percent of the (variant, pattern) counters are 1, and the logL still
    matches in FP64 and FP32."""
    from netrax_gb300.likelihood import NetworkLikelihood
    so = _sweep_oracle(2, config2)
    so.orc.variant = "AVERAGE"
    lengths = np.clip(np.array(so.orc.brlen) * stretch, 1e-6, 100.0)
    want_total = so.evaluate(lengths, gradient=False)[0]
    with NetworkLikelihood(config2.network, config2.partitions, precision="fp64") as lik:
        lik.set_branch_lengths(lengths)
        assert lik.loglikelihood() == pytest.approx(want_total, rel=FP64_REL)
        node, _, _, _ = lik.dag_export()
        rank = {}
        scaled = 0
        for v in range(len(node)):
            idx = rank.get(int(node[v]), 0)
            rank[int(node[v])] = idx + 1
            _, sc = lik.get_clv(v, 0)
            want = so.keep[0]["scaler"][so.variant_of[(int(node[v]), idx)]]
            assert np.array_equal(sc.astype(np.uint32), want), v
            scaled += int(np.count_nonzero(want))
        assert (scaled > 0) == (stretch > 1.0)
    with NetworkLikelihood(config2.network, config2.partitions, precision="fp32") as lik:
        lik.set_branch_lengths(lengths)
        assert lik.loglikelihood() == pytest.approx(want_total, rel=FP32_REL)


@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_config1_ten_uneven_partitions_full_size(variant, precision):
    from netrax_gb300.likelihood import NetworkLikelihood
    w = _workload(1)
    assert len(w.partitions) == 10
    want = _oracle_eval(_sweep_oracle(1, w), variant)
    with NetworkLikelihood(w.network, w.partitions, variant=variant, precision=precision) as lik:
        _check(lik, want, precision)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_config3_protein_full_size(precision):
    """FP32 runs the forward and adjoint P x CLV products on the tensor cores."""
    from netrax_gb300.likelihood import NetworkLikelihood
    w = _workload(3)
    want = _oracle_eval(_sweep_oracle(3, w), "AVERAGE")
    with NetworkLikelihood(w.network, w.partitions, precision=precision) as lik:
        _check(lik, want, precision)


def test_config4_candidates_in_one_batch():
    """Four candidates of the search-move batch (different taxa, reticulation
    and partition counts) scored together in one batch graph: every
    candidate's logL and gradient against the oracle."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkBatch, NetworkLikelihood
    specs = synth.candidate_specs(64)
    pick = [0, 1, 2, 3]
    works = [synth.make_workload(*specs[i]) for i in pick]
    liks = [NetworkLikelihood(w.network, w.partitions, precision="fp32") for w in works]
    try:
        with NetworkBatch(liks) as batch:
            tot, gb, gr = batch.loglikelihood_gradient()
        for k, w in enumerate(works):
            total, _, _, g, gret = _oracle_eval(_sweep_oracle(("cand", pick[k]), w), "AVERAGE")
            assert tot[k] == pytest.approx(total, rel=FP32_REL)
            assert np.abs(gb[k] - g).max() <= GRAD_TOL["fp32"] * max(1.0, float(np.abs(g).max()))
            if len(gret):
                assert np.abs(gr[k] - gret).max() <= GRAD_TOL["fp32"] * max(1.0, float(np.abs(gret).max()))
    finally:
        for lk in liks:
            lk.close()
