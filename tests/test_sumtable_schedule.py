"""CPU: the host schedule of the edge-sumtable build (``netlk_sumtable_export``
on host-only contexts), replayed on symbolic buffers, on random networks with
arcs on any edge (reticulations below reticulations, nodes that die in some
configurations) and on the golden cases:

* the ops are exactly the DAG variants whose subtree holds the edge, once
  each; mode 1 where the variant takes the edge itself, mode 2 where its
  child on the edge's side holds it, the other child as in the DAG;
* in walk order, every mode-2 op finds its child's unit directions in the
  work slot it reads (written by that child's op, not overwritten since),
  and every slot index lies below the reported count;
* the tables are the displayed-tree roots among the ops, numbered 0 ..
  n_tables - 1 once each, grouped by the child whose CLV the edge's message
  starts from (the mode-1 op at the end of the op's chain of children).
"""
import numpy as np
import pytest

from conftest import golden_cases
from netrax_gb300.likelihood import NetworkLikelihood
from netrax_gb300.network import parse_extended_newick
from test_dag_random import _partition, nasty_network


def _check_edge(lik, e, node, ch, ed, root_vars):
    ops, n_work, n_tab, gref, gbeg = lik.sumtable_export(e)
    V = len(node)
    holds = {}

    def holds_edge(v):  # the variant's subtree holds edge e
        if v not in holds:
            holds[v] = any(int(ed[v][k]) == e or (int(ch[v][k]) >= 0 and holds_edge(int(ch[v][k])))
                           for k in range(2))
        return holds[v]

    want = {v for v in range(V) if holds_edge(v)}
    xs = [int(x) for x in ops[:, 0]]
    assert sorted(xs) == sorted(want) and len(set(xs)) == len(xs)
    slots = {}
    op_of = {}
    tables = []
    for j, (x, d, o, mode, td, tx, tab) in enumerate(ops.tolist()):
        kids = [int(ch[x][0]), int(ch[x][1])]
        edges = [int(ed[x][0]), int(ed[x][1])]
        assert d in kids and sorted([d, o]) == sorted(kids)
        side = kids.index(d) if kids[0] != kids[1] else (0 if edges[0] == e else 1)
        if mode == 1:
            assert edges[side] == e and td == -1
        else:
            assert mode == 2 and d >= 0 and holds_edge(d) and edges[side] != e
            assert 0 <= td < n_work and slots.get(td) == d, (e, j, td, slots.get(td), d)
        if tx >= 0:
            assert tx < n_work
            slots[tx] = x
        op_of[x] = j
        if tab >= 0:
            tables.append((tab, j))
    assert sorted(t for t, _ in tables) == list(range(n_tab))
    assert {int(ops[j, 0]) for _, j in tables} == want & root_vars
    # groups: the child the edge's message starts from, per table
    for t, j in tables:
        while int(ops[j, 3]) == 2:
            j = op_of[int(ops[j, 1])]
        g = int(np.searchsorted(gbeg, t, side="right")) - 1
        assert 0 <= g < len(gref) and int(gref[g]) == int(ops[j, 1])
    return len(ops), n_work


def _check_network(text, n_tips):
    net = parse_extended_newick(text)
    with NetworkLikelihood(net, [_partition(np.random.default_rng(1), n_tips)], host_only=True) as lik:
        node, ch, ed, _ = lik.dag_export()
        _, dt, _ = lik.root_export()  # the variants whose CLV gives each tree's logL
        root_vars = {int(v) for v in dt}
        return [_check_edge(lik, e, node, ch, ed, root_vars) for e in range(net.n_edges)]


@pytest.mark.parametrize("seed", range(40))
def test_random_network_sumtable_schedules(seed):
    rng = np.random.default_rng(9100 + seed)
    n_taxa = int(rng.integers(4, 15))
    n_ret = int(rng.integers(1, 6))
    _check_network(nasty_network(rng, n_taxa, n_ret), n_taxa)


@pytest.mark.parametrize("case", [c for c in golden_cases() if len(c["partitions"]) == 1
                                  and c["partitions"][0].get("states", 4) == 4])
def test_golden_network_sumtable_schedules(case):
    from conftest import GoldenPartition
    net = parse_extended_newick(case["newick"])
    with NetworkLikelihood(net, [GoldenPartition(d) for d in case["partitions"]], host_only=True) as lik:
        node, ch, ed, _ = lik.dag_export()
        _, dt, _ = lik.root_export()  # the variants whose CLV gives each tree's logL
        root_vars = {int(v) for v in dt}
        work = [_check_edge(lik, e, node, ch, ed, root_vars)[1] for e in range(net.n_edges)]
    assert max(work) >= 1 or net.n_edges <= 2


def test_host_only_contexts_report_no_device():
    """On a host-only context the table build reports that it does not apply
    and every derivative entry returns NETLK_ERR_NO_DEVICE (no device work)."""
    from conftest import GoldenPartition
    from netrax_gb300 import _native as N
    case = {c["name"]: c for c in golden_cases()}["twoReticulations"]
    net = parse_extended_newick(case["newick"])
    with NetworkLikelihood(net, [GoldenPartition(d) for d in case["partitions"]], host_only=True) as lik:
        assert lik.edge_sumtable(0) == (False, 0)
        for call in (lambda: lik.edge_sumtable_derivatives(0, 0.1), lambda: lik.edge_derivatives(0),
                     lambda: lik.edge_derivatives_partition(0, 0)):
            with pytest.raises(N.NetlkError) as e:
                call()
            assert e.value.status == N.NETLK_ERR_NO_DEVICE
