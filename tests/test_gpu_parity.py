"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerances: plain FP64 GPU kernel within 1e-9 relative logL of the
oracle; FP32 CLVs with power-of-two scaling within 1e-6 relative; FP64 scale
counters bit-exact; displayed-tree enumeration bit-exact (checked on CPU in
test_dag_abi.py and here through the per-tree values). Gradients against
central finite differences of the FP64 oracle (h = 1e-5).
"""
import math

import numpy as np
import pytest

from conftest import GoldenPartition, golden_cases

pytestmark = pytest.mark.gpu

CASES = golden_cases()
FP64_REL = 1e-9
FP32_REL = 1e-6


def _lik(case, variant, precision, **kw):
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    net = parse_extended_newick(case["newick"])
    parts = [GoldenPartition(d) for d in case["partitions"]]
    return NetworkLikelihood(net, parts, variant=variant, precision=precision, **kw)


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_logl_matches_oracle(case, variant, precision):
    g = case[variant]
    tol = FP64_REL if precision == "fp64" else FP32_REL
    with _lik(case, variant, precision) as lik:
        total, part, trees = lik.loglikelihood(details=True)
        assert total == pytest.approx(g["logl"], rel=tol)
        assert np.allclose(part, g["partition_logl"], rtol=tol, atol=0)
        for k, t in enumerate(g["trees"]):
            if t["partition_logl"] is None:
                assert np.all(np.isnan(trees[k]))
                continue
            assert np.allclose(trees[k], t["partition_logl"], rtol=tol, atol=0), k
        again = lik.loglikelihood()
        assert again == total  # repeated evaluation is bit-identical


@pytest.mark.parametrize("case", [c for c in CASES if "scaler_sums" in c["AVERAGE"]], ids=lambda c: c["name"])
def test_fp64_scale_counters_bit_exact(case):
    want = case["AVERAGE"]["scaler_sums"]
    with _lik(case, "AVERAGE", "fp64") as lik:
        lik.loglikelihood()
        node, _, _, _ = lik.dag_export()
        # variants are listed node by node in the fixture; map GPU variants in the same order
        order = sorted(range(len(node)), key=lambda i: (node[i], i))
        got = []
        for i in order:
            s = 0
            for p in range(lik.n_parts):
                _, sc = lik.get_clv(i, p)
                s += int(sc.sum())
            got.append(s)
        assert got == want
        if case["name"].endswith("deep"):
            assert max(want) > 0  # the case really exercises the 2^256 rescaling


@pytest.mark.parametrize("case", [c for c in CASES if "fd_grad_brlen" in c["AVERAGE"]], ids=lambda c: c["name"])
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gradient_matches_finite_differences(case, variant, precision):
    g = case[variant]
    fd = np.array(g["fd_grad_brlen"])
    fdr = np.array(g["fd_grad_retprob"])
    rtol, atol = (1e-4, 2e-3) if precision == "fp64" else (2e-3, 2e-2)
    with _lik(case, variant, precision) as lik:
        total, gb, gr = lik.loglikelihood_gradient()
        assert total == pytest.approx(g["logl"], rel=FP64_REL if precision == "fp64" else FP32_REL)
        # edges sitting on the 1e-6 clamp only have a one-sided difference
        free = lik.branch_lengths > 2e-5
        assert np.allclose(gb[free], fd[free], rtol=rtol, atol=atol * max(1.0, np.abs(fd).max() * 1e-3))
        if len(fdr):
            assert np.allclose(gr, fdr, rtol=rtol, atol=atol)


def test_gradient_logl_equals_logl_only():
    case = [c for c in CASES if c["name"] == "synthetic_16taxa_4ret_3parts"][0]
    for precision in ("fp64", "fp32"):
        with _lik(case, "AVERAGE", precision) as lik:
            a = lik.loglikelihood()
            b, _, _ = lik.loglikelihood_gradient()
            assert a == b


def test_graph_and_direct_launch_agree():
    case = [c for c in CASES if c["name"] == "synthetic_12taxa_3ret_2parts"][0]
    with _lik(case, "AVERAGE", "fp32", use_cuda_graph=True) as a, \
            _lik(case, "AVERAGE", "fp32", use_cuda_graph=False) as b:
        ta, ga, ra = a.loglikelihood_gradient()
        tb, gb, rb = b.loglikelihood_gradient()
        assert ta == tb
        assert np.array_equal(ga, gb) and np.array_equal(ra, rb)


def test_parameter_updates_change_and_restore():
    case = [c for c in CASES if c["name"] == "twoReticulations"][0]
    with _lik(case, "AVERAGE", "fp64") as lik:
        base = lik.loglikelihood()
        bl = lik.branch_lengths.copy()
        lik.set_branch_lengths(bl * 1.5)
        changed = lik.loglikelihood()
        assert changed != base  # BrlenOptTest.cpp:248: a brlen change moves logL
        lik.set_branch_lengths(bl)
        assert lik.loglikelihood() == base  # incremental == full (DOUBLE_EQ)
        p = lik.ret_probs.copy()
        lik.set_reticulation_probs(np.clip(p * 0.5, 1e-3, None))
        assert lik.loglikelihood() != base
        lik.set_reticulation_probs(p)
        assert lik.loglikelihood() == base


def test_sharded_partials_match_whole():
    """Two contexts over disjoint pattern halves + SUM of partials == one context."""
    case = [c for c in CASES if c["name"] == "synthetic_16taxa_4ret_3parts"][0]
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    net = parse_extended_newick(case["newick"])
    full = [GoldenPartition(d) for d in case["partitions"]]
    halves = [[], []]
    for gp in full:
        n = gp.tip_states.shape[1]
        for h, sl in enumerate((slice(0, n // 2), slice(n // 2, n))):
            q = GoldenPartition(case["partitions"][0])
            q.tip_states = np.ascontiguousarray(gp.tip_states[:, sl])
            q.weights = gp.weights[sl].copy()
            q.freqs, q.exch, q.alpha = gp.freqs, gp.exch, gp.alpha
            halves[h].append(q)
    with NetworkLikelihood(net, full, precision="fp64") as whole, \
            NetworkLikelihood(net, halves[0], precision="fp64") as h0, \
            NetworkLikelihood(net, halves[1], precision="fp64") as h1:
        tw, gw, rw = whole.loglikelihood_gradient()
        glob = h0.tree_partials() + h1.tree_partials()
        t0, g0, r0, _ = h0.mix_and_backward(glob)
        t1, g1, r1, _ = h1.mix_and_backward(glob)
        assert t0 == pytest.approx(tw, rel=1e-12) and t1 == t0
        assert np.allclose(g0 + g1, gw, rtol=1e-9, atol=1e-9)
        assert np.allclose(r0, rw, rtol=1e-9, atol=1e-9)


def test_fp32_matches_fp64_on_larger_network():
    """50 taxa / 4 reticulations / 10 uneven partitions (scaled down) - FP32 vs FP64 GPU."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    w = synth.config(1, scale=0.05)
    for variant in ("AVERAGE", "BEST"):
        with NetworkLikelihood(w.network, w.partitions, variant=variant, precision="fp64") as a, \
                NetworkLikelihood(w.network, w.partitions, variant=variant, precision="fp32") as b:
            ta, ga, ra = a.loglikelihood_gradient()
            tb, gb, rb = b.loglikelihood_gradient()
            assert tb == pytest.approx(ta, rel=FP32_REL)
            assert np.allclose(gb, ga, rtol=1e-3, atol=1e-2 * max(1.0, np.abs(ga).max() * 1e-3))
            assert np.allclose(rb, ra, rtol=1e-3, atol=1e-2)


def test_fp64_matches_oracle_on_synthetic_config():
    """Config-0 shape (20 taxa / 1 reticulation / 1k sites) against the oracle, computed here."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    from oracle import improved, newick
    w = synth.config(0)
    net = newick.parse_newick(w.newick)
    parts = [improved.Partition(p.tip_states, p.weights, p.freqs, p.exch,
                                _rates(p.alpha)) for p in w.partitions]
    for variant in ("AVERAGE", "BEST"):
        ref = improved.ImprovedOracle(net, parts, variant=variant).loglikelihood()
        with NetworkLikelihood(w.network, w.partitions, variant=variant, precision="fp64") as lik:
            assert lik.loglikelihood() == pytest.approx(ref, rel=FP64_REL)


def test_protein_fp32_matches_fp64_and_oracle():
    """40 taxa / 3 reticulations / 20-state partition (scaled to 1k sites):
    FP64 GPU against the oracle, FP32 GPU against FP64 GPU, logL and gradient."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    from oracle import improved, newick
    w = synth.config(3, scale=0.02)
    net = newick.parse_newick(w.newick)
    parts = [improved.Partition(p.tip_states, p.weights, p.freqs, p.exch,
                                _rates(p.alpha)) for p in w.partitions]
    for variant in ("AVERAGE", "BEST"):
        ref = improved.ImprovedOracle(net, parts, variant=variant).loglikelihood()
        with NetworkLikelihood(w.network, w.partitions, variant=variant, precision="fp64") as a, \
                NetworkLikelihood(w.network, w.partitions, variant=variant, precision="fp32") as b:
            ta, ga, ra = a.loglikelihood_gradient()
            tb, gb, rb = b.loglikelihood_gradient()
            assert ta == pytest.approx(ref, rel=FP64_REL)
            assert tb == pytest.approx(ta, rel=FP32_REL)
            assert np.allclose(gb, ga, rtol=1e-3, atol=1e-2 * max(1.0, np.abs(ga).max() * 1e-3))
            assert np.allclose(rb, ra, rtol=1e-3, atol=1e-2)


def test_protein_tensor_cores_match_cuda_cores():
    """The tcgen05 sweeps (3xTF32, FP32 accumulation) against the CUDA-core
    FP32 sweeps and the FP64 run, on a 40-taxon / 3-reticulation protein
    workload with 2 partitions (tiles must not mix partitions): logL per
    partition and the gradient."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    w = synth.make_protein_workload("protein 2 partitions", 40, 3, [700, 1300], 77)
    for variant in ("AVERAGE", "BEST"):
        with NetworkLikelihood(w.network, w.partitions, variant=variant, precision="fp64") as a, \
                NetworkLikelihood(w.network, w.partitions, variant=variant, precision="fp32",
                                  tensor_cores=False) as b, \
                NetworkLikelihood(w.network, w.partitions, variant=variant, precision="fp32") as c:
            ta, pa = a.loglikelihood(details=True)[:2]
            tb, pb = b.loglikelihood(details=True)[:2]
            tc, pc = c.loglikelihood(details=True)[:2]
            assert tb == pytest.approx(ta, rel=FP32_REL)
            assert tc == pytest.approx(ta, rel=FP32_REL)
            assert np.allclose(pc, pa, rtol=FP32_REL, atol=0)
            _, ga, ra = a.loglikelihood_gradient()
            _, gb, rb = b.loglikelihood_gradient()
            _, gc, rc = c.loglikelihood_gradient()
            scale = max(1.0, np.abs(ga).max())
            # tensor-core adjoint (3xTF32) and CUDA-core FP32 adjoint against FP64
            assert np.abs(gc - ga).max() <= 2e-5 * scale
            assert np.abs(gb - ga).max() <= 2e-5 * scale
            assert np.allclose(rc, ra, rtol=1e-3, atol=1e-2)


def test_protein_sharded_partials_match_whole():
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    w = synth.config(3, scale=0.02)
    full = w.partitions
    halves = [[], []]
    for p in full:
        cut = p.n_patterns // 2
        for h, sl in enumerate((slice(0, cut), slice(cut, None))):
            halves[h].append(synth.PartitionData(np.ascontiguousarray(p.tip_states[:, sl]), p.weights[sl],
                                                 p.freqs, p.exch, p.alpha, p.n_sites, states=20))
    with NetworkLikelihood(w.network, full, precision="fp64") as whole, \
            NetworkLikelihood(w.network, halves[0], precision="fp64") as h0, \
            NetworkLikelihood(w.network, halves[1], precision="fp64") as h1:
        tw, gw, rw = whole.loglikelihood_gradient()
        glob = h0.tree_partials() + h1.tree_partials()
        t0, g0, r0, _ = h0.mix_and_backward(glob)
        t1, g1, r1, _ = h1.mix_and_backward(glob)
        assert t0 == pytest.approx(tw, rel=1e-12)
        assert np.allclose(g0 + g1, gw, rtol=1e-9, atol=1e-9)
        assert np.allclose(r0, rw, rtol=1e-9, atol=1e-9)


def _rates(alpha):
    from oracle import pllmath
    return pllmath.gamma_rates_mean(alpha, 4)


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    from netrax_gb300.likelihood import NetworkLogL
    case = [c for c in CASES if c["name"] == "smallNetwork"][0]
    with _lik(case, "AVERAGE", "fp64") as lik:
        b = torch.tensor(lik.branch_lengths, dtype=torch.float64, requires_grad=True)
        p = torch.tensor(lik.ret_probs, dtype=torch.float64, requires_grad=True)
        y = NetworkLogL.apply(b, p, lik)
        y.backward()
        _, gb, gr = lik.loglikelihood_gradient()
        assert np.allclose(b.grad.numpy(), gb) and np.allclose(p.grad.numpy(), gr)
        assert float(y.detach()) == pytest.approx(case["AVERAGE"]["logl"], rel=FP64_REL)


def test_launch_count_reported():
    case = [c for c in CASES if c["name"] == "tinyNetwork"][0]
    with _lik(case, "AVERAGE", "fp32") as lik:
        before = lik.launch_count()
        lik.loglikelihood_gradient()
        # P-matrices, one forward launch per level, site sums, mixture, one
        # adjoint launch per level, two gradient reduction stages
        assert lik.launch_count() - before == lik.stats["launches_per_gradient_eval"]
        assert lik.stats["launches_per_gradient_eval"] <= 5 + 2 * lik.stats["n_levels"]


def test_batch_matches_individual_contexts():
    """One CUDA graph over several candidate networks (DNA of different sizes,
    plus a protein context on the tensor-core path, so each context runs its
    own launch sequence) == each context alone; a second call picks up new
    branch lengths."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkBatch, NetworkLikelihood
    ws = synth.candidate_batch(5, scale=0.03)
    ws.append(synth.make_protein_workload("protein candidate", 30, 2, [600], 5))
    liks = [NetworkLikelihood(w.network, w.partitions, precision="fp32") for w in ws]
    try:
        with NetworkBatch(liks) as batch:
            rng = np.random.default_rng(3)
            for rep in range(2):
                if rep:
                    for lk, w in zip(liks, ws):
                        lk.set_branch_lengths(w.network.branch_lengths * np.exp(0.1 * rng.standard_normal(lk.n_edges)))
                tot, gb, gr = batch.loglikelihood_gradient()
                for i, lk in enumerate(liks):
                    t1, g1, r1 = lk.loglikelihood_gradient()
                    assert tot[i] == t1
                    assert np.array_equal(gb[i], g1)
                    assert np.array_equal(gr[i], r1)
    finally:
        for lk in liks:
            lk.close()


@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
@pytest.mark.parametrize("mode", ["persistent", "per_context"])
def test_persistent_batch_matches_individual_contexts(variant, mode):
    """Candidate networks of different sizes (DNA, FP32: the persistent
    launches, where warps take (candidate, pattern unit) items; or the graph of
    per-context launches) == each context evaluated alone, bit for bit, on
    three calls with new branch lengths; every walk shape gives the same
    bits, so the shape the batch picks does not matter."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkBatch, NetworkLikelihood
    ws = synth.candidate_batch(9, scale=0.02)
    liks = [NetworkLikelihood(w.network, w.partitions, precision="fp32", variant=variant) for w in ws]
    try:
        with NetworkBatch(liks, per_context=mode == "per_context") as batch:
            info = batch.info()
            assert info["persistent"] == (mode == "persistent")
            if info["persistent"]:
                assert info["launches_per_call"] == 9
            rng = np.random.default_rng(4)
            for rep in range(3):
                if rep:
                    for lk, w in zip(liks, ws):
                        lk.set_branch_lengths(w.network.branch_lengths * np.exp(0.1 * rng.standard_normal(lk.n_edges)))
                tot, gb, gr = batch.loglikelihood_gradient()
                for i, lk in enumerate(liks):
                    t1, g1, r1 = lk.loglikelihood_gradient()
                    assert tot[i] == t1, (rep, i)
                    assert np.array_equal(gb[i], g1)
                    assert np.array_equal(gr[i], r1)
                    assert lk.loglikelihood() == t1  # the batch left valid CLVs behind
    finally:
        for lk in liks:
            lk.close()


@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_reference_derivative_mode(variant):
    """netlk_edge_derivatives mode 1 (the reference's per-partition formula:
    AVERAGE over trees where the edge is active, BEST = derivative of the
    active tree with the largest tree_logl * tree_prob) against central
    differences of that formula evaluated from the per-tree sums."""
    case = [c for c in CASES if c["name"] == "synthetic_16taxa_4ret_3parts"][0]
    with _lik(case, variant, "fp64") as lik:
        net = lik.network
        rv, _, lp = lik.root_export()
        _, _, _, cov = lik.dag_export()
        base = net.branch_lengths.copy()
        min_lp = math.log(1e-6)
        edges = [int(net.ret_first_edge[0]), int(net.ret_second_edge[0]), int(net.ret_second_edge[-1])]
        tree_edge = [e for e in range(lik.n_edges) if net.edge_child[e] not in set(net.ret_node)][0]
        for e in edges + [tree_edge]:
            child = int(net.edge_child[e])
            act = np.ones(len(rv), bool)
            if child in set(int(x) for x in net.ret_node):
                k = [int(x) for x in net.ret_node].index(child)
                want = 1 if e == int(net.ret_second_edge[k]) else 0
                for i, v in enumerate(rv):
                    words = cov[v]
                    cfgs = [t for t in range(1 << lik.n_ret) if (int(words[t >> 6]) >> (t & 63)) & 1]
                    act[i] = any(((t >> k) & 1) == want for t in cfgs)
            use = act & (lp >= min_lp)
            t0 = lik.tree_partials()
            choice = [int(np.argmax(np.where(use, t0[:, p] * np.exp(lp), -np.inf))) for p in range(lik.n_parts)]

            def f(delta):
                b = base.copy()
                b[e] += delta
                lik.set_branch_lengths(b)
                t = lik.tree_partials()
                if variant == "AVERAGE":
                    return sum(np.logaddexp.reduce(lp[use] + t[use, p]) for p in range(lik.n_parts))
                return sum(t[choice[p], p] for p in range(lik.n_parts))

            h = 1e-5
            want_d1 = (f(h) - f(-h)) / (2 * h)
            lik.set_branch_lengths(base)
            got = lik.edge_derivatives(e, second=False, mode=1)
            assert got == pytest.approx(want_d1, rel=1e-5, abs=1e-4)
            if e == tree_edge and variant == "AVERAGE":
                assert got == pytest.approx(lik.edge_derivatives(e, second=False, mode=0), rel=1e-12, abs=1e-9)
        # the context is left evaluating the real mixture
        assert lik.loglikelihood() == pytest.approx(case[variant]["logl"], rel=FP64_REL)


@pytest.mark.parametrize("kind", ["dna_fp32", "dna_fp64", "protein_tc"])
def test_checkpointed_gradients_are_identical(kind):
    """O(sqrt n) CLV checkpointing: 2-4 segments give the same logL and
    gradient, bit for bit, as storing every CLV (the recomputed CLVs are the
    same numbers), with fewer CLV buffers."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    if kind == "protein_tc":
        w = synth.make_protein_workload("protein", 30, 3, [500], 9)
        prec = "fp32"
    else:
        w = synth.config(2, scale=0.01)
        prec = "fp32" if kind == "dna_fp32" else "fp64"
    for variant in ("AVERAGE", "BEST"):
        with NetworkLikelihood(w.network, w.partitions, variant=variant, precision=prec, checkpoint_segments=1) as a:
            ta, ga, ra = a.loglikelihood_gradient()
            la = a.loglikelihood()
            slots = a.stats["clv_slots"]
            for k in (2, 3, 4):
                with NetworkLikelihood(w.network, w.partitions, variant=variant, precision=prec,
                                       checkpoint_segments=k) as b:
                    assert b.stats["clv_slots"] < slots
                    tb, gb, rb = b.loglikelihood_gradient()
                    assert tb == ta and np.array_equal(gb, ga) and np.array_equal(rb, ra)
                    assert b.loglikelihood() == la
                    tb2, gb2, _ = b.loglikelihood_gradient()  # again, after a logL-only call
                    assert tb2 == ta and np.array_equal(gb2, ga)


@pytest.mark.parametrize("shapes", ["walk", "level"])
def test_checkpointed_walk_sweeps_are_identical(shapes, monkeypatch):
    """Checkpointing with the single-launch walk sweeps (one forward walk
    over every segment; per segment from the top a recompute walk and an
    adjoint walk), and with the level sweeps, on every walk shape: the logL
    and gradient equal storing every CLV, bit for bit."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    w = synth.config(2, scale=0.02)
    import ctypes
    from netrax_gb300 import _native as N
    with NetworkLikelihood(w.network, w.partitions, checkpoint_segments=1) as a:
        ta, ga, ra = a.loglikelihood_gradient()
        ws = ctypes.c_int32()
        N.check(N.lib().netlk_walk_shape_begin(a._h, ctypes.byref(ws)), a._h)
        first_walk = ws.value
    pairs = ([(first_walk + i, first_walk + j) for i, j in ((0, 0), (1, 2), (2, 3), (3, 4), (4, 1))]
             if shapes == "walk" else [(0, 0), (3, 5), (11, 9)])
    for k in (2, 4):
        for f, b in pairs:
            monkeypatch.setenv("NETLK_SHAPES", "%d,%d" % (f, b))
            with NetworkLikelihood(w.network, w.partitions, checkpoint_segments=k) as lik:
                tb, gb, rb = lik.loglikelihood_gradient()
                t = lik.tuning()
                assert t["backward_walk"] == (shapes == "walk") and t["backward_shape"] == b
                assert lik.stats["checkpoint_segments"] == k
                assert tb == ta and np.array_equal(gb, ga) and np.array_equal(rb, ra), (k, f, b)


@pytest.mark.parametrize("kind", ["dna_fp32", "dna_fp64", "protein_tc"])
def test_incremental_matches_full(kind):
    """Incremental evaluation (only the variants above changed branch
    lengths) gives exactly the full evaluation's logL along a sequence of
    single-edge, multi-edge, no-op, probability and model changes, and
    recomputes fewer CLVs when one edge changes; netlk_edge_loglikelihood ==
    setting the length and evaluating."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    if kind == "protein_tc":
        w = synth.make_protein_workload("protein", 24, 2, [400], 4)
        prec = "fp32"
    else:
        w = synth.config(0)
        prec = "fp32" if kind == "dna_fp32" else "fp64"
    rng = np.random.default_rng(5)
    E = w.network.n_edges
    with NetworkLikelihood(w.network, w.partitions, precision=prec) as inc, \
            NetworkLikelihood(w.network, w.partitions, precision=prec, incremental=False) as full:
        b = w.network.branch_lengths.copy()
        assert inc.loglikelihood() == full.loglikelihood()
        total_updates = inc.stats["site_clv_updates"]
        fewer = 0
        for step in range(12):
            kind_step = step % 6
            if kind_step in (0, 1, 2):       # one edge
                e = int(rng.integers(E))
                b[e] *= float(np.exp(0.3 * rng.standard_normal()))
            elif kind_step == 3:             # several edges
                for e in rng.choice(E, 3, replace=False):
                    b[e] *= float(np.exp(0.3 * rng.standard_normal()))
            elif kind_step == 4 and w.network.n_reticulations:  # probabilities only
                p = np.clip(rng.uniform(0.2, 0.8, w.network.n_reticulations), 0.01, 0.99)
                inc.set_reticulation_probs(p)
                full.set_reticulation_probs(p)
            inc.set_branch_lengths(b)
            full.set_branch_lengths(b)
            li, lf = inc.loglikelihood(), full.loglikelihood()
            assert li == lf
            if kind_step in (0, 1, 2):
                fewer += inc.last_site_updates() < total_updates
            if kind_step == 5:                # no change at all: nothing recomputed
                assert inc.last_site_updates() == 0
        assert fewer >= 1
        # the edge evaluation entry point
        e = int(rng.integers(E))
        le = inc.edge_loglikelihood(e, 0.05)
        b[e] = 0.05
        full.set_branch_lengths(b)
        assert le == full.loglikelihood()
        # a gradient evaluation in between leaves the incremental state consistent
        tg = inc.loglikelihood_gradient()[0]
        assert tg == full.loglikelihood_gradient()[0]
        b[(e + 1) % E] *= 1.5
        inc.set_branch_lengths(b)
        full.set_branch_lengths(b)
        assert inc.loglikelihood() == full.loglikelihood()


def test_adjoint_launch_shapes_agree(monkeypatch):
    """Every launch shape of the DNA FP32 sweeps (the adjoint with two, four or
    eight patterns per lane) gives the same logL and gradient, bit for bit."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    w = synth.config(1, scale=0.02)
    res = {}
    # 12-16: walk shapes (the whole sweep in one launch per chunk of units;
    # CLVs and single messages handed between consecutive ops in registers)
    for shapes in ("0,0", "0,5", "0,6", "5,2", "6,4", "7,7", "8,8", "9,9", "10,10", "11,11", "12,12", "13,13",
                   "14,14", "15,15", "16,16", "13,16", "1,12", "12,10"):
        monkeypatch.setenv("NETLK_SHAPES", shapes)
        with NetworkLikelihood(w.network, w.partitions, precision="fp32") as lik:
            res[shapes] = lik.loglikelihood_gradient()  # the first evaluation fixes the shapes
            tun = lik.tuning()
            assert (tun["forward_shape"], tun["backward_shape"]) == tuple(int(x) for x in shapes.split(","))
    t0, g0, r0 = res["0,0"]
    for k, (t, g, r) in res.items():
        # edge terms are summed per 16-pattern unit in every shape: same bits
        assert t == t0
        assert np.array_equal(g, g0) and np.array_equal(r, r0)


def test_walk_sweeps_in_several_chunks(monkeypatch):
    """A walk sweep over more warps than one wave holds runs in equal chunks
    of units; it gives the level sweeps' logL and gradient bit for bit."""
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    text = "((A:0.2,((B:0.1,C:0.15)P:0.1)X#H1:0.1::0.3)Q:0.2,(D:0.2,X#H1:0.12::0.7)R:0.2);"
    rng = np.random.default_rng(11)
    n = 200_000  # > one wave of the 16-blocks-per-SM walk shape on 152 SMs

    class Part:
        tip_states = (1 << rng.integers(0, 4, size=(4, n))).astype(np.uint32)
        weights = rng.integers(1, 4, size=n).astype(np.float64)
        freqs = np.array([0.2, 0.3, 0.3, 0.2])
        exch = np.array([1.0, 2.5, 0.8, 1.2, 3.0, 1.0])
        alpha = 0.8
        states = 4
        rate_cats = 4

    res = {}
    for shapes in ("0,0", "14,14", "12,12"):
        monkeypatch.setenv("NETLK_SHAPES", shapes)
        with NetworkLikelihood(parse_extended_newick(text), [Part], precision="fp32", device=0) as lik:
            res[shapes] = lik.loglikelihood_gradient()
            l0 = lik.launch_count()
            lik.loglikelihood_gradient()
            if shapes == "14,14":  # P-matrices, 2 x chunks, site sums, mixture, gradient reduction (2)
                n = lik.launch_count() - l0
                assert (n - 5) % 2 == 0 and (n - 5) // 2 >= 2
    t0, g0, r0 = res["0,0"]
    for t, g, r in res.values():
        assert t == t0
        assert np.array_equal(g, g0) and np.array_equal(r, r0)


@pytest.mark.parametrize("config", [1, 3], ids=["dna", "protein"])
def test_edge_derivatives_match_full_gradients(config):
    """netlk_edge_derivatives takes d1 and d2 analytically from one tangent
    sweep over the variants above the edge. DNA (50 taxa, 10 partitions) and
    protein (40 taxa): FP64 d1 equals the adjoint gradient's entry (1e-10
    relative) and d2 the central difference of two FP64 full gradients
    (1e-5); FP32 d1 equals the FP64 one within 1e-5 of the largest gradient
    entry and d2 within 1e-4 of max(1, |d2|); the context keeps evaluating
    the network at its own lengths."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    w = synth.config(config, scale=0.02)
    net = w.network
    ret_edges = [int(x) for x in net.ret_first_edge] + [int(x) for x in net.ret_second_edge]
    tip_edges = [e for e in range(net.n_edges) if int(net.edge_child[e]) < net.n_tips][:2]
    inner = [e for e in range(net.n_edges) if e not in ret_edges and e not in tip_edges][:3]
    edges = ret_edges[:2] + tip_edges + inner
    base = np.array(net.branch_lengths, np.float64)
    want = {}
    with NetworkLikelihood(net, w.partitions, precision="fp64") as lik:
        logl0, g0, _ = lik.loglikelihood_gradient()
        for e in edges:
            d1, d2 = lik.edge_derivatives(e, second=True)
            assert d1 == pytest.approx(g0[e], rel=1e-10, abs=1e-8)
            t = base[e]
            h = min(1e-6, t / 200.0)
            b = base.copy()
            b[e] = t + h
            lik.set_branch_lengths(b)
            gp = lik.loglikelihood_gradient()[1][e]
            b[e] = max(t - h, 1e-6)
            lik.set_branch_lengths(b)
            gm = lik.loglikelihood_gradient()[1][e]
            lik.set_branch_lengths(base)
            assert d2 == pytest.approx((gp - gm) / (t + h - b[e]), rel=1e-5, abs=1e-3)
            assert lik.loglikelihood() == logl0
            want[e] = (d1, d2)
    gscale = max(1.0, float(np.abs(g0).max()))
    with NetworkLikelihood(net, w.partitions, precision="fp32") as lik:
        for e in edges:
            d1, d2 = lik.edge_derivatives(e, second=True)
            print("edge %d fp32 d1 error %.2e (of %.2e), d2 error %.2e (of %.2e)"
                  % (e, abs(d1 - want[e][0]), gscale, abs(d2 - want[e][1]), abs(want[e][1])))
            assert abs(d1 - want[e][0]) <= 1e-5 * gscale
            assert abs(d2 - want[e][1]) <= 1e-4 * max(1.0, abs(want[e][1]))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_checkpointed_edge_derivatives_take_the_full_path(precision):
    """With several checkpoint segments netlk_edge_derivatives takes d1 from
    full adjoint sweeps and d2 as a central difference: they agree with the
    analytic values of a context that stores every CLV."""
    from netrax_gb300 import synth
    from netrax_gb300.likelihood import NetworkLikelihood
    w = synth.config(2, scale=0.01)
    edges = [0, 5, 17, int(w.network.ret_first_edge[0])]
    with NetworkLikelihood(w.network, w.partitions, precision=precision) as a, \
            NetworkLikelihood(w.network, w.partitions, precision=precision, checkpoint_segments=3) as b:
        for e in edges:
            x1, x2 = a.edge_derivatives(e)
            y1, y2 = b.edge_derivatives(e)
            tol = 1e-9 if precision == "fp64" else 1e-4
            assert abs(x1 - y1) <= tol * max(1.0, abs(x1))
            assert abs(x2 - y2) <= (1e-4 if precision == "fp64" else 5e-3) * max(1.0, abs(x2))
