"""Generate ``system_networks.json`` from the reference's regression networks.

    python tests/golden/make_system_golden.py [--reference /path/to/NetRAX]

The reference's system tests keep 19 networks that once broke its likelihood
code, as Extended Newick string literals passed to ``problemTest``
(``test/src/SystemTest.cpp:158-290``; 4 taxa, chains of reticulations below
reticulations, a trifurcating root). This script reads those literals as data,
pairs each network with a seeded random 4-taxon DNA alignment (40 sites) and
scores it with the CPU oracle under AVERAGE and BEST: network log-likelihood,
per-displayed-tree values, the naive 2^r evaluation and the displayed-tree DAG
(covered configuration sets per node). Nothing here runs at test time.

Topology. 15 of the networks have a trifurcating root with a reticulation
among the children moved under the new node. The reference's
enforceToplevelBifurcation (src/io/RootedNetworkParser.cpp:272-289) re-points
only the moved children's tree-parent pointer, so a moved reticulation keeps
its parent link to the root - which is what the oracle's parser restates -
and the root ends up with three children, which processNodeImproved asserts
against (src/likelihood/ImprovedLoglikelihood.cpp:378). The library's parser
moves the reticulation's link too and builds a binary network. For those
cases the oracle scores the library's parse ("topology": "library"); for the
other 4 both parses agree ("topology": "shared").
"""
import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import MODEL, covered_lists  # noqa: E402
from netrax_gb300.network import parse_extended_newick  # noqa: E402
from oracle import improved, naive, newick, pllmath  # noqa: E402


def oracle_network(desc, like):
    """An oracle network with the library parse's topology and numbering."""
    n = desc.n_nodes
    children = [[] for _ in range(n)]
    child_edges = [[] for _ in range(n)]
    for v in range(n):
        for e in desc.node_child_edges[2 * v:2 * v + 2]:
            if e >= 0:
                children[v].append(int(desc.edge_child[e]))
                child_edges[v].append(int(e))
    rets = [int(x) for x in desc.ret_node]
    tree_parent = [-1] * n
    for e in range(desc.n_edges):
        if int(desc.edge_child[e]) not in rets:
            tree_parent[int(desc.edge_child[e])] = int(desc.edge_parent[e])
    return newick.OracleNetwork(
        n_tips=desc.n_tips, n_nodes=n, n_edges=desc.n_edges, n_ret=len(rets), root=desc.root,
        labels=like.labels, node_is_ret=[v in rets for v in range(n)], children=children,
        child_edges=child_edges, edge_parent=[int(x) for x in desc.edge_parent],
        edge_child=[int(x) for x in desc.edge_child], edge_length=[float(x) for x in desc.branch_lengths],
        ret_node=rets, ret_first_edge=[int(x) for x in desc.ret_first_edge],
        ret_second_edge=[int(x) for x in desc.ret_second_edge],
        ret_first_parent=[int(desc.edge_parent[e]) for e in desc.ret_first_edge],
        ret_second_parent=[int(desc.edge_parent[e]) for e in desc.ret_second_edge],
        ret_first_prob=[float(x) for x in desc.ret_first_probs], tree_parent=tree_parent)


def extract(reference):
    src = open(os.path.join(reference, "test", "src", "SystemTest.cpp")).read()
    out = []
    for m in re.finditer(r"TEST\(SystemTest,\s*(\w+)\)\s*\{\s*problemTest\(\s*((?:\"[^\"]*\"\s*)+)\);", src):
        out.append((m.group(1), "".join(re.findall(r"\"([^\"]*)\"", m.group(2)))))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="path of the NetRAX source tree (read-only input)")
    a = ap.parse_args()
    cases = []
    for k, (name, text) in enumerate(extract(a.reference)):
        own = newick.parse_newick(text)
        desc = parse_extended_newick(text)
        shared = all(len(set(c)) <= 2 for c in own.children)
        net = own if shared else oracle_network(desc, own)
        rng = np.random.default_rng(400 + k)
        codes = (1 << rng.integers(0, 4, size=(net.n_tips, 40))).astype(np.uint32)
        pat, w = pllmath.compress_patterns(codes)
        pd = dict(MODEL, tip_states=pat.tolist(), weights=w.tolist())
        case = {"name": name, "newick": text, "partitions": [pd], "topology": "shared" if shared else "library",
                "edge_parent": list(net.edge_parent), "edge_child": list(net.edge_child)}
        for variant in ("AVERAGE", "BEST"):
            part = improved.Partition(pat, w, pd["freqs"], pd["exch"], pllmath.gamma_rates_mean(pd["alpha"], 4))
            orc = improved.ImprovedOracle(net, [part], variant=variant)
            total = orc.loglikelihood()
            case[variant] = {"logl": total, "naive_logl": naive.naive_loglikelihood(orc)[0],
                             "trees": [{"logprob": t.logprob,
                                        "partition_logl": t.partition_logl if t.logl_valid else None}
                                       for t in orc.root_trees()]}
        case["dag"] = covered_lists(orc)
        case["n_reticulations"] = net.n_ret
        cases.append(case)
        print(name, net.n_ret, case["AVERAGE"]["logl"], case["AVERAGE"]["naive_logl"], flush=True)
    with open(os.path.join(HERE, "system_networks.json"), "w") as f:
        json.dump({"model": MODEL, "cases": cases}, f)


if __name__ == "__main__":
    main()
