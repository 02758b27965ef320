"""CPU: the compiled displayed-tree DAG against the oracle on random networks.

The reference's sample networks and the synthetic workloads place every
reticulation between two tree edges. Here arcs may start or end on any edge,
reticulation edges included, which produces reticulations directly below
reticulations, arcs leaving reticulated subtrees and nodes that die in some
configurations. For 60 seeded networks (4-14 taxa, 1-5 reticulations) the
host-only context's DAG must equal the oracle's literal restatement of
processNodeImproved node by node (variant order and covered configuration
sets), with the same displayed-tree root variant and log-probability per root
tree - or both must reject the network - and its single-launch walk schedules
must keep their invariants (topological order, message slots written before
they are read and read once, register hand-offs to the next op only).
"""
import numpy as np
import pytest

from conftest import GoldenPartition
from netrax_gb300.likelihood import NetworkLikelihood
from netrax_gb300.network import parse_extended_newick
from test_dag_abi import _check_walk


def nasty_network(rng, n_taxa, n_ret, mean_brlen=0.1):
    """Extended Newick of a random tree with n_ret arcs between any two edges."""
    children, parents, length, prob = {}, {}, {}, {}
    nid = n_taxa
    lineages = list(range(n_taxa))
    while len(lineages) > 1:
        i, j = rng.choice(len(lineages), size=2, replace=False)
        a, b = lineages[i], lineages[j]
        v, nid = nid, nid + 1
        children[v] = [a, b]
        for c in (a, b):
            length[(v, c)] = rng.exponential(mean_brlen)
            parents[c] = [v]
        lineages = [x for k, x in enumerate(lineages) if k not in (i, j)] + [v]
    root = lineages[0]
    is_ret = set()

    def descendants(v):
        out, st = set(), [v]
        while st:
            x = st.pop()
            if x not in out:
                out.add(x)
                st.extend(children.get(x, []))
        return out

    added = 0
    for _ in range(10000):
        if added == n_ret:
            break
        edges = sorted(length)
        (u, v), (x, y) = [edges[k] for k in rng.choice(len(edges), 2, replace=False)]
        if u in descendants(y):
            continue  # the arc would close a cycle
        s, t = nid, nid + 1
        nid += 2
        for (p, c), new in (((u, v), s), ((x, y), t)):
            L = length.pop((p, c))
            f = rng.uniform()
            children[p] = [new if k == c else k for k in children[p]]
            children[new] = [c]
            parents[c] = [new if k == p else k for k in parents[c]]
            parents[new] = [p]
            length[(p, new)] = f * L
            length[(new, c)] = (1 - f) * L
            if (p, c) in prob:  # a split reticulation edge keeps its probability
                prob[(new, c)] = prob.pop((p, c))
        children[s].append(t)
        parents[t].append(s)
        length[(s, t)] = rng.exponential(mean_brlen)
        is_ret.add(t)
        p1 = rng.uniform(0.2, 0.8)
        prob[(x, t)] = p1
        prob[(s, t)] = 1.0 - p1
        added += 1
    assert added == n_ret
    ret_name = {t: "H%d" % (k + 1) for k, t in enumerate(sorted(is_ret))}
    seen = set()

    def emit(v, parent):
        if v in is_ret:
            tail = "#%s:%.17g::%.17g" % (ret_name[v], length[(parent, v)], prob[(parent, v)])
            if v in seen:
                return tail
            seen.add(v)
            return "(" + ",".join(emit(c, v) for c in children[v]) + ")" + tail
        brl = "" if parent is None else ":%.17g" % length[(parent, v)]
        if v < n_taxa:
            return "T%d" % v + brl
        return "(" + ",".join(emit(c, v) for c in children[v]) + ")" + brl

    return emit(root, None) + ";"


def _partition(rng, n_tips, n=6):
    return GoldenPartition({"tip_states": rng.integers(1, 16, size=(n_tips, n)).tolist(),
                            "weights": [1.0] * n, "freqs": [0.25, 0.25, 0.25, 0.25],
                            "exch": [1.0] * 6, "alpha": 1.0})


def _covered(cov_row, n_ret):
    bits = set()
    for w, word in enumerate(cov_row):
        word = int(word)
        for b in range(64):
            if (word >> b) & 1 and w * 64 + b < (1 << n_ret):
                bits.add(w * 64 + b)
    return bits


@pytest.mark.parametrize("seed", range(60))
def test_random_network_dag_matches_oracle(seed):
    from oracle import improved, newick as onewick, pllmath
    rng = np.random.default_rng(5000 + seed)
    n_taxa = int(rng.integers(4, 15))
    n_ret = int(rng.integers(1, 6))
    text = nasty_network(rng, n_taxa, n_ret)
    part = _partition(rng, n_taxa)
    onet = onewick.parse_newick(text)
    opart = improved.Partition(part.tip_states, part.weights, part.freqs, part.exch,
                               pllmath.gamma_rates_mean(part.alpha, 4))
    orc = improved.ImprovedOracle(onet, [opart])
    try:
        orc.loglikelihood()
        oracle_error = None
    except RuntimeError as e:
        oracle_error = str(e)
    net = parse_extended_newick(text)
    try:
        lik = NetworkLikelihood(net, [part], host_only=True)
    except Exception as e:  # the product must reject exactly what the oracle rejects
        assert oracle_error is not None, (text, e)
        return
    assert oracle_error is None, (text, oracle_error)
    node, _, _, cov = lik.dag_export()
    got = {}
    for i in range(len(node)):
        got.setdefault(int(node[i]), []).append(_covered(cov[i], net.n_reticulations))
    want = {v: [set(s) for s in sets] for v, sets in orc.dag_summary().items() if sets}
    assert got == want, text
    rv, dt, lp = lik.root_export()
    trees = orc.root_trees()
    assert len(trees) == len(rv)
    for k, t in enumerate(trees):
        assert lp[k] == pytest.approx(t.logprob, rel=1e-13, abs=1e-13)
        if t.dtroot is None:
            continue
        dnode = int(node[dt[k]])
        assert dnode == t.dtroot[0]
        assert [i for i in range(len(node)) if node[i] == dnode].index(dt[k]) == t.dtroot[1]
    _check_walk(lik)
    lik.close()


def test_fourteen_reticulations_compile_quickly():
    """The two-child step and the root matching find intersecting variant sets
    through per-node configuration owners instead of all pairs: a 60-taxon
    network with 14 reticulations (41k variants, 2^14 configurations) compiles
    in well under a second (56 s with the pairwise loops)."""
    import time
    from netrax_gb300 import synth
    rng = np.random.default_rng(14)
    net = parse_extended_newick(synth.random_network_newick(rng, 60, 14))
    part = _partition(rng, 60, n=8)
    t = time.perf_counter()
    lik = NetworkLikelihood(net, [part], host_only=True)
    assert time.perf_counter() - t < 20.0
    st = lik.stats
    assert st["n_variants"] > 30000 and st["n_root_variants"] > 8192
    rv, dt, lp = lik.root_export()
    assert np.isclose(np.logaddexp.reduce(lp), 0.0, atol=1e-9)  # the root variants cover every configuration once
    lik.close()


def _replay_checkpoint_plan(lik):
    """Replays one logL + gradient evaluation of a checkpointed context on
    symbolic buffers: the forward sweep level by level, then per segment from
    the top the recompute of its non-permanent variants and its adjoint levels
    (deepest first). Every CLV read - a child of a forward or recompute op, an
    adjoint op's own CLV / scale counters and its children - must find the
    expected variant in its buffer; a level's ops run in one launch, so they
    read before any of them writes and never write the same buffer."""
    node, ch, _, _ = lik.dag_export()
    _, dt, _ = lik.root_export()
    ns, n_slots, slot, perm, seg = lik.checkpoint_export()
    V = len(node)
    level = np.zeros(V, np.int64)
    for v in range(V):  # variants are stored children first
        kids = [int(c) for c in ch[v] if c >= 0]
        assert all(c < v for c in kids)
        level[v] = 1 + max([level[c] for c in kids], default=0)
    n_levels = int(level.max())
    assert seg[0, 0] == 1 and seg[-1, 1] == n_levels
    assert all(seg[i + 1, 0] == seg[i, 1] + 1 for i in range(ns - 1))
    by_level = [[v for v in range(V) if level[v] == L] for L in range(n_levels + 1)]
    adjoint = np.zeros(V, bool)
    for v in set(int(x) for x in dt):
        adjoint[v] = True
    for v in range(V - 1, -1, -1):
        if adjoint[v]:
            for c in ch[v]:
                if c >= 0:
                    adjoint[int(c)] = True
    assert slot.min() >= 0 and slot.max() < n_slots
    held = {}

    def run_level(ops):
        for v in ops:  # reads first
            for c in ch[v]:
                if c >= 0:
                    assert held.get(int(slot[c])) == int(c), ("child", v, int(c))
        written = [int(slot[v]) for v in ops]
        assert len(set(written)) == len(written), "two ops of a level write one buffer"
        for v in ops:
            held[int(slot[v])] = v

    for L in range(1, n_levels + 1):
        run_level(by_level[L])
    for s in range(ns - 1, -1, -1):
        lo, hi = int(seg[s, 0]), int(seg[s, 1])
        if s < ns - 1:
            for L in range(lo, hi + 1):
                run_level([v for v in by_level[L] if not perm[v]])
        for L in range(hi, lo - 1, -1):
            for v in by_level[L]:
                if not adjoint[v]:
                    continue
                assert held.get(int(slot[v])) == v, ("own CLV", v)
                for c in ch[v]:
                    if c >= 0:
                        assert held.get(int(slot[c])) == int(c), ("adjoint child", v, int(c))


@pytest.mark.parametrize("seed", range(30))
def test_random_network_checkpoint_plan_is_sound(seed):
    """O(sqrt n) CLV checkpointing on random networks with 2, 3 and 5
    segments: no buffer is overwritten before its last read (replayed on
    symbolic buffers), and the plan never holds more buffers than variants
    (small networks save none: every variant is read across a segment)."""
    rng = np.random.default_rng(8000 + seed)
    n_taxa = int(rng.integers(8, 30))
    n_ret = int(rng.integers(1, 7))
    net = parse_extended_newick(nasty_network(rng, n_taxa, n_ret))
    part = _partition(rng, n_taxa, n=4)
    for k in (2, 3, 5):
        lik = NetworkLikelihood(net, [part], host_only=True, checkpoint_segments=k)
        ns, n_slots, _, _, _ = lik.checkpoint_export()
        assert n_slots <= lik.n_variants
        _replay_checkpoint_plan(lik)
        if len(lik.walk_export()[0]):
            _replay_checkpointed_walk(lik)
        lik.close()


def _replay_checkpointed_walk(lik):
    """Replays the walk sweeps of a checkpointed context, as one warp runs
    them, on symbolic buffers: the forward walk over every segment, then per
    segment from the top a recompute walk of its non-permanent variants and
    its adjoint walk. Every CLV read finds the expected variant in its buffer,
    the recompute walk of a segment is exactly its non-permanent variants, a
    message handed over in registers never crosses a launch, and every message
    slot is read once, by its child, before it is written again."""
    node, ch, _, _ = lik.dag_export()
    ns, _, slot, perm, seg = lik.checkpoint_export()
    fwd, bwd, reads = lik.walk_export()
    brange, rvar, rrange = lik.walk_segments()
    assert len(brange) == ns and len(rrange) == ns
    V = len(node)
    level = np.zeros(V, np.int64)
    for v in range(V):
        level[v] = 1 + max([level[int(c)] for c in ch[v] if c >= 0], default=0)
    seg_of = np.searchsorted(seg[:, 1], level)  # segment of each variant's level
    held = {}

    def compute(v):
        for c in ch[v]:
            if c >= 0:
                assert held.get(int(slot[c])) == int(c), ("child", int(v), int(c))
        held[int(slot[v])] = int(v)

    for v in fwd:
        compute(v)
    msgs = {}
    covered = []
    for s in range(ns - 1, -1, -1):
        lo, hi = rrange[s]
        if s == ns - 1:
            assert lo == hi
        want = sorted(v for v in range(V) if seg_of[v] == s and not perm[v]) if s < ns - 1 else []
        assert sorted(rvar[lo:hi].tolist()) == want
        for v in rvar[lo:hi]:
            compute(v)
        b0, b1 = brange[s]
        covered += list(range(b0, b1))
        carried = None
        for x, oa, ob, from_regs, mb, mc in bwd[b0:b1].tolist():
            assert seg_of[x] == s
            assert held.get(int(slot[x])) == x, ("own CLV", x)
            if from_regs:
                assert carried == x
            carried = None
            for r in reads[mb:mb + mc].tolist():
                assert msgs.pop(r) == x, "message read by the wrong op"
            for c, out in zip(ch[x].tolist(), (oa, ob)):
                if c >= 0:
                    assert held.get(int(slot[c])) == c, ("adjoint child", x, c)
                if out == -2:
                    carried = c
                elif out >= 0:
                    assert out not in msgs, "message slot overwritten before it was read"
                    msgs[out] = c
        assert carried is None, "a message handed over in registers across a launch"
    assert sorted(covered) == list(range(len(bwd)))
    assert not msgs, "messages never read"


def _replay_adjoint_messages(lik):
    """Replays the level adjoint's message buffers (one launch per level): each
    op reads only messages addressed to its own variant, each message is read
    exactly once and before its buffer is written again, no buffer is both
    read and written, or written twice, within one launch, and no message is
    left unread. (The sweeps drop a buffer's lines from L2 as soon as it has
    been read, which relies on exactly this.)"""
    ops, reads, lb = lik.adjoint_export()
    held = {}
    for L in range(len(lb) - 1):
        lo, hi = int(lb[L]), int(lb[L + 1])
        read_here = []
        for x, _, _, _, _, mb, mc in ops[lo:hi]:
            for r in reads[mb:mb + mc]:
                assert held.get(int(r)) == int(x), ("message to another variant", int(r))
                read_here.append(int(r))
        assert len(set(read_here)) == len(read_here), "a buffer read twice"
        for r in read_here:
            del held[r]
        written = []
        for _, a, b, oa, ob, _, _ in ops[lo:hi]:
            for child, out in ((a, oa), (b, ob)):
                if out >= 0:
                    assert child >= 0, "message to a tip or the fake child"
                    assert int(out) not in held, "a buffer written before its message was read"
                    written.append((int(out), int(child)))
        slots = [s for s, _ in written]
        assert len(set(slots)) == len(slots), "two messages in one buffer in one launch"
        assert not set(slots) & set(read_here), "a buffer read and written in one launch"
        for s, child in written:
            held[s] = child
    assert not held, "messages left unread"


@pytest.mark.parametrize("seed", range(30))
def test_random_network_adjoint_messages_are_read_once(seed):
    rng = np.random.default_rng(9100 + seed)
    n_taxa = int(rng.integers(4, 30))
    n_ret = int(rng.integers(0, 7))
    net = parse_extended_newick(nasty_network(rng, n_taxa, n_ret))
    lik = NetworkLikelihood(net, [_partition(rng, n_taxa, n=4)], host_only=True)
    _replay_adjoint_messages(lik)
    lik.close()


def test_checkpoint_export_without_segments():
    """With one segment every variant keeps its own CLV buffer (buffer id =
    variant id) for the whole evaluation, and the plan replays trivially."""
    from netrax_gb300 import synth
    w = synth.config(2, scale=0.01)
    lik = NetworkLikelihood(w.network, w.partitions, host_only=True, checkpoint_segments=1)
    ns, n_slots, slot, perm, seg = lik.checkpoint_export()
    assert ns == 1 and n_slots == lik.n_variants
    assert np.array_equal(slot, np.arange(lik.n_variants)) and perm.all()
    assert seg.tolist() == [[1, lik.stats["n_levels"]]]
    _replay_checkpoint_plan(lik)
    _replay_checkpointed_walk(lik)
    lik.close()


@pytest.mark.parametrize("k", [2, 4, 6])
def test_checkpointed_walk_on_the_100_taxon_network(k):
    """The 100-taxon / 8-reticulation network (947 variants) with 2, 4 and 6
    checkpoint segments: the walk sweeps replay soundly on symbolic buffers."""
    from netrax_gb300 import synth
    w = synth.config(2, scale=0.01)
    lik = NetworkLikelihood(w.network, w.partitions, host_only=True, checkpoint_segments=k)
    assert lik.checkpoint_export()[0] == k
    assert len(lik.walk_export()[0]) == lik.n_variants
    _replay_checkpoint_plan(lik)
    _replay_checkpointed_walk(lik)
    lik.close()
