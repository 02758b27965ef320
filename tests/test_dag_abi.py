"""C ABI surface and the displayed-tree DAG, on CPU (host_only contexts).

* the library loads and exports every function ``include/netlk.h`` declares;
* the Extended Newick reader numbers nodes / edges like the oracle (and so the
  reference, src/io/NetworkIO.cpp:39-299);
* the DAG compiled on bitsets equals the oracle's literal restatement of
  processNodeImproved node by node: same variant count and order, same covered
  configuration sets, same displayed-tree root variant per root tree, same
  tree log-probabilities (the golden ``dag`` records);
* invalid input is rejected with a status code, never a crash.
"""
import ctypes
import math
import os
import re

import numpy as np
import pytest

from conftest import ROOT, GoldenPartition, golden_cases
from netrax_gb300 import _native
from netrax_gb300.likelihood import NetworkLikelihood
from netrax_gb300.network import parse_extended_newick

CASES = golden_cases()


def test_header_symbols_exported():
    header = open(os.path.join(ROOT, "include", "netlk.h")).read()
    names = set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(netlk_\w+)\s*\(", header, re.M))
    assert len(names) >= 19
    L = _native.lib()
    for n in sorted(names):
        assert hasattr(L, n), n
    assert set(names) == set(_native.EXPORTED)


def _covered(cov_row, n_ret):
    bits = set()
    for w, word in enumerate(cov_row):
        word = int(word)
        for b in range(64):
            if (word >> b) & 1 and w * 64 + b < (1 << n_ret):
                bits.add(w * 64 + b)
    return bits


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_dag_matches_oracle_enumeration(case):
    from oracle import newick as onewick
    net = parse_extended_newick(case["newick"])
    onet = onewick.parse_newick(case["newick"])
    assert net.root == onet.root and net.n_tips == onet.n_tips
    assert list(net.edge_parent) == onet.edge_parent and list(net.edge_child) == onet.edge_child
    assert np.allclose(net.branch_lengths, onet.edge_length, rtol=0, atol=0)
    parts = [GoldenPartition(d) for d in case["partitions"]]
    lik = NetworkLikelihood(net, parts, host_only=True)
    node, ch, ed, cov = lik.dag_export()
    got = [[int(node[i]), sorted(_covered(cov[i], net.n_reticulations))] for i in range(len(node))]
    want = sorted(case["dag"], key=lambda x: x[0])
    # variants of one node keep their order; nodes are listed in id order in the fixture
    got_by_node = {}
    for v, s in got:
        got_by_node.setdefault(v, []).append(s)
    want_by_node = {}
    for v, s in want:
        want_by_node.setdefault(v, []).append(s)
    assert got_by_node == want_by_node
    rv, dt, lp = lik.root_export()
    for k, t in enumerate(case["AVERAGE"]["trees"]):
        assert lp[k] == pytest.approx(t["logprob"], rel=1e-13, abs=1e-13)
        dnode = int(node[dt[k]])
        assert dnode == t["dtroot_node"]
        same_node = [i for i in range(len(node)) if node[i] == dnode]
        assert same_node.index(dt[k]) == t["dtroot_index"]
    # children of each variant are variants of the node's children (or tips / fake)
    for i in range(len(node)):
        for j in range(2):
            if ch[i, j] >= 0:
                assert net.edge_child[ed[i, j]] == node[ch[i, j]]
            elif ch[i, j] != -(2 ** 31):
                assert net.edge_child[ed[i, j]] == -1 - ch[i, j]
    assert lik.stats["site_clv_updates"] == lik.stats["n_variants"] * lik.stats["n_patterns_total"]


def test_reference_numbering_of_small_network():
    # ((A:2,((B:1,C:1)P:1)X#H1:0::0.3)Q:2,(D:2,X#H1:0::0.7)R:2); tips in string order
    net = parse_extended_newick("((A:2,((B:1,C:1)P:1)X#H1:0::0.3)Q:2,(D:2,X#H1:0::0.7)R:2);")
    assert net.n_tips == 4 and net.n_reticulations == 1
    assert net.ret_first_probs[0] == pytest.approx(0.3)
    assert net.n_edges == net.n_tips + (net.n_nodes - net.n_tips - 1) - 1 + 2
    assert net.branch_lengths.min() == pytest.approx(1e-6)  # zero length clamped
    assert net.root == net.n_nodes - 1 - net.n_reticulations


@pytest.mark.parametrize("bad", [
    "((A,B);",                       # unbalanced
    "(A,B)",                         # no semicolon
    "((A,(B)#H1:::0.3),(C,#H1:::0.9));",  # probabilities do not sum to one
])
def test_newick_rejects_bad_input(bad):
    with pytest.raises(ValueError):
        parse_extended_newick(bad)


def _small():
    net = parse_extended_newick("((A:0.2,(B:0.1)X#H1:0.1::0.3)Q:0.2,(C:0.2,X#H1:0.1::0.7)R:0.2);")
    part = GoldenPartition({"tip_states": [[1, 2], [2, 4], [8, 1]], "weights": [1, 2],
                            "freqs": [.25] * 4, "exch": [1] * 6, "alpha": 1.0})
    return net, part


def test_invalid_arguments_return_status():
    net, part = _small()
    bad = net.__class__(**{**net.__dict__})
    bad.branch_lengths = net.branch_lengths.copy()
    bad.branch_lengths[0] = float("nan")
    with pytest.raises(_native.NetlkError) as e:
        NetworkLikelihood(bad, [part], host_only=True)
    assert e.value.status == 1
    cyc = net.__class__(**{**net.__dict__})
    cyc.edge_child = net.edge_child.copy()
    cyc.edge_child[0] = net.root  # root gets a parent -> not a rooted network
    with pytest.raises(_native.NetlkError) as e:
        NetworkLikelihood(cyc, [part], host_only=True)
    assert e.value.status == 2
    p2 = GoldenPartition({"tip_states": [[1, 0], [2, 4], [8, 1]], "weights": [1, 2],
                          "freqs": [.25] * 4, "exch": [1] * 6, "alpha": 1.0})
    p2.states = 61  # codon models are not on this path
    with pytest.raises(_native.NetlkError) as e:
        NetworkLikelihood(net, [p2], host_only=True)
    assert e.value.status == 7
    p3 = GoldenPartition({"tip_states": [[1, 0], [2, 4], [8, 1]], "weights": [1, 2],
                          "freqs": [.25] * 4, "exch": [1] * 6, "alpha": 1.0})
    p3.rate_cats = 8
    p3.states = 20
    p3.freqs = np.full(20, 0.05)
    p3.exch = np.ones(190)
    with pytest.raises(_native.NetlkError) as e:
        NetworkLikelihood(net, [p3], host_only=True)
    assert e.value.status == 7


def test_host_only_context_refuses_evaluation():
    net, part = _small()
    lik = NetworkLikelihood(net, [part], host_only=True)
    with pytest.raises(_native.NetlkError) as e:
        lik.loglikelihood()
    assert e.value.status == _native.NETLK_ERR_NO_DEVICE
    for call in (lik.loglikelihood_gradient, lambda: lik.enqueue(True), lik.result_pointers,
                 lambda: lik.edge_derivatives(0), lambda: lik.edge_loglikelihood(0, 0.1)):
        with pytest.raises(_native.NetlkError) as e:
            call()
        assert e.value.status == _native.NETLK_ERR_NO_DEVICE
    lik.set_branch_lengths(net.branch_lengths * 2)
    with pytest.raises(_native.NetlkError):
        lik.set_branch_lengths(net.branch_lengths[:-1])
    with pytest.raises(_native.NetlkError):
        lik.set_reticulation_probs([1.5])
    lik.close()


def test_too_many_reticulations_unsupported():
    from netrax_gb300 import synth
    rng = np.random.default_rng(5)
    net = parse_extended_newick(synth.random_network_newick(rng, 40, 17))
    part = GoldenPartition({"tip_states": [[1]] * 40, "weights": [1], "freqs": [.25] * 4,
                            "exch": [1] * 6, "alpha": 1.0})
    with pytest.raises(_native.NetlkError) as e:
        NetworkLikelihood(net, [part], host_only=True)
    assert e.value.status == 7


def test_batch_rejects_bad_arguments():
    import ctypes
    net, part = _small()
    L = _native.lib()
    h = ctypes.c_void_p()
    assert L.netlk_batch_create(None, 0, ctypes.byref(h)) == _native.NETLK_ERR_INVALID_ARGUMENT
    lik = NetworkLikelihood(net, [part], host_only=True)
    arr = (ctypes.c_void_p * 1)(lik._h)
    assert L.netlk_batch_create(arr, 1, ctypes.byref(h)) == _native.NETLK_ERR_NO_DEVICE
    assert b"host_only" in L.netlk_last_error(None)
    assert not h.value
    assert L.netlk_batch_loglikelihood_gradient(None, None, None, None) == _native.NETLK_ERR_INVALID_ARGUMENT
    lik.close()


def test_checkpoint_segments_reduce_clv_slots():
    """Cutting the levels into segments keeps only the CLVs read across a
    segment boundary; every other variant is recomputed once per gradient."""
    from netrax_gb300 import synth
    w = synth.config(2, scale=0.002)
    full = NetworkLikelihood(w.network, w.partitions, host_only=True, checkpoint_segments=1).stats
    assert full["checkpoint_segments"] == 1 and full["clv_slots"] == full["n_variants"]
    assert full["recompute_site_updates"] == 0
    prev = None
    for k in (2, 4):
        st = NetworkLikelihood(w.network, w.partitions, host_only=True, checkpoint_segments=k).stats
        assert st["checkpoint_segments"] == k
        assert st["clv_slots"] < full["clv_slots"]
        assert 0 < st["recompute_site_updates"] < full["site_clv_updates"]
        assert st["launches_per_gradient_eval"] > full["launches_per_gradient_eval"]
        prev = st
    # automatic mode on a host-only context stores everything
    auto = NetworkLikelihood(w.network, w.partitions, host_only=True).stats
    assert auto["checkpoint_segments"] == 1


def _check_walk(lik):
    """Invariants of the single-launch (walk) schedules, from the exported
    schedule and the DAG: the forward walk is a topological order of every
    variant; the adjoint walk visits the variants reachable from the
    displayed-tree roots, each before its children; every message is written
    to a slot no unread message holds, and read exactly once, by its child; a
    message kept in registers goes to the very next op, whose only message
    it is."""
    node, ch, ed, cov = lik.dag_export()
    rv, dt, lp = lik.root_export()[:3]
    fwd, bwd, slots = lik.walk_export()
    V = len(node)
    assert sorted(fwd.tolist()) == list(range(V))
    pos = {int(v): i for i, v in enumerate(fwd)}
    for v in range(V):
        for c in ch[v]:
            if c >= 0:
                assert pos[int(c)] < pos[v], "child computed after its parent"
    # variants the adjoint reaches: displayed-tree roots and their descendants
    reach, stack = set(), [int(x) for x in dt]
    while stack:
        v = stack.pop()
        if v in reach:
            continue
        reach.add(v)
        stack.extend(int(c) for c in ch[v] if c >= 0)
    xs = [int(r[0]) for r in bwd]
    assert sorted(xs) == sorted(reach)
    bpos = {x: i for i, x in enumerate(xs)}
    senders = {v: 0 for v in range(V)}
    for x in xs:
        for c in ch[x]:
            if c >= 0:
                assert bpos[x] < bpos[int(c)], "adjoint of a child before its parent"
                senders[int(c)] += 1
    held = {}        # slot -> (sender, receiver) of the unread message it holds
    received = {x: 0 for x in xs}
    carried_to = None
    for i, (x, out_a, out_b, from_regs, begin, count) in enumerate(bwd.tolist()):
        if from_regs:
            assert carried_to == x and count == 0 and senders[x] == 1
            received[x] += 1
        else:
            assert carried_to is None
        carried_to = None
        for s in slots[begin:begin + count].tolist():
            assert s in held and held[s][1] == x, "message read by the wrong op"
            del held[s]
            received[x] += 1
        for c, out in zip(ch[x].tolist(), (out_a, out_b)):
            if c < 0:
                assert out == -1
            elif out == -2:
                assert i + 1 < len(xs) and xs[i + 1] == c and senders[c] == 1
                carried_to = c
            else:
                assert out >= 0 and out not in held, "slot overwritten before it was read"
                held[out] = (x, c)
    assert not held, "messages never read"
    assert all(received[x] == senders[x] for x in xs)


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_walk_schedule_invariants(case):
    net = parse_extended_newick(case["newick"])
    parts = [GoldenPartition(d) for d in case["partitions"]]
    lik = NetworkLikelihood(net, parts, host_only=True)
    if parts[0].states == 4:
        _check_walk(lik)
    else:  # 20-state contexts run level sweeps only
        fwd, bwd, slots = lik.walk_export()
        assert len(fwd) == len(bwd) == len(slots) == 0
    lik.close()


@pytest.mark.parametrize("cfg", [1, 2])
def test_walk_schedule_invariants_synthetic(cfg):
    """The 50-taxon / 4-reticulation and 100-taxon / 8-reticulation networks
    (947 variants), without and with checkpoint segments."""
    from netrax_gb300 import synth
    w = synth.config(cfg, scale=0.002)
    lik = NetworkLikelihood(w.network, w.partitions, host_only=True)
    _check_walk(lik)
    fwd, bwd, slots = lik.walk_export()
    assert (bwd[:, 1] == -2).sum() + (bwd[:, 2] == -2).sum() == bwd[:, 3].sum() > 0
    lik.close()
    seg = NetworkLikelihood(w.network, w.partitions, host_only=True, checkpoint_segments=2)
    _check_walk(seg)
    seg.close()
