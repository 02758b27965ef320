"""Seeded synthetic workloads: networks, GTR+Gamma models and simulated MSAs.

No public benchmark data ships with this path, so every workload is generated:

* network: a random rooted binary tree on ``n_taxa`` tips (uniform random
  joins of lineages), branch lengths ~ Exp(mean 0.1); then ``n_ret``
  reticulations in the shape of NetRAX's arc insertion - split a source and a
  target tree edge at U(0,1) of their length and add an arc of length
  ~ Exp(0.1) from the source split node to the target split node, rejecting
  pairs that would close a cycle. The target's original parent is the first
  parent, with probability ~ U(0.2, 0.8).
* model per partition: GTR exchangeabilities ~ Dirichlet(1^6), base frequencies
  ~ Dirichlet(1^4), Gamma shape 0.8, 4 mean-rate categories.
* MSA: every site draws a displayed tree (each reticulation takes its first
  parent with its probability) and a rate category, and evolves from the
  stationary distribution down that tree. Columns are pattern-compressed.

The network is emitted as Extended Newick and read back with
``network.parse_extended_newick``, so node and edge ids follow the reference's
numbering.
"""
from dataclasses import dataclass
from typing import List

import numpy as np

from .network import NetworkDesc, parse_extended_newick

DNA = "ACGT"


@dataclass
class PartitionData:
    tip_states: np.ndarray       # uint32 [n_tips][n_patterns] state bitmasks
    weights: np.ndarray          # float64 [n_patterns]
    freqs: np.ndarray            # float64 [4]
    exch: np.ndarray             # float64 [6]
    alpha: float
    n_sites: int
    rate_cats: int = 4
    states: int = 4
    prop_invar: float = 0.0      # proportion of invariant sites (+I)

    @property
    def n_patterns(self):
        return self.tip_states.shape[1]


@dataclass
class Workload:
    name: str
    newick: str
    network: NetworkDesc
    partitions: List[PartitionData]
    seed: int

    @property
    def n_sites(self):
        return sum(p.n_sites for p in self.partitions)

    @property
    def n_patterns(self):
        return sum(p.n_patterns for p in self.partitions)


def random_network_newick(rng, n_taxa, n_ret, mean_brlen=0.1):
    """Extended Newick of a random network (see module docstring)."""
    children = {}
    length = {}           # (parent, child) -> branch length
    parents = {}          # child -> list of parents (first parent first)
    nid = n_taxa
    lineages = list(range(n_taxa))
    while len(lineages) > 1:
        i, j = rng.choice(len(lineages), size=2, replace=False)
        a, b = lineages[i], lineages[j]
        v = nid
        nid += 1
        children[v] = [a, b]
        for c in (a, b):
            length[(v, c)] = rng.exponential(mean_brlen)
            parents[c] = [v]
        lineages = [x for k, x in enumerate(lineages) if k not in (i, j)] + [v]
    root = lineages[0]
    is_ret = set()
    prob = {}             # (parent, ret) -> probability of that parent

    def descendants(v):
        out, st = set(), [v]
        while st:
            x = st.pop()
            if x in out:
                continue
            out.add(x)
            st.extend(children.get(x, []))
        return out

    added = 0
    attempts = 0
    while added < n_ret:
        attempts += 1
        if attempts > 100000:
            raise RuntimeError("could not place reticulations")
        tree_edges = [(p, c) for (p, c) in length
                      if p not in is_ret and c not in is_ret]
        (u, v), (x, y) = [tree_edges[k] for k in rng.choice(len(tree_edges), 2, replace=False)]
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
        children[s].append(t)
        parents[t].append(s)
        length[(s, t)] = rng.exponential(mean_brlen)
        is_ret.add(t)
        p1 = rng.uniform(0.2, 0.8)
        prob[(x, t)] = p1
        prob[(s, t)] = 1.0 - p1
        added += 1

    ret_name = {t: "H%d" % (k + 1) for k, t in enumerate(sorted(is_ret))}
    seen = set()

    def emit(v, parent):
        if v in is_ret:
            tail = "#%s:%.17g::%.17g" % (ret_name[v], length[(parent, v)], prob[(parent, v)])
            if v in seen:
                return tail
            seen.add(v)
            return "(" + ",".join(emit(c, v) for c in children[v]) + ")" + tail
        lab = "T%d" % v if v < n_taxa else ""
        brl = "" if parent is None else ":%.17g" % length[(parent, v)]
        if v < n_taxa:
            return lab + brl
        return "(" + ",".join(emit(c, v) for c in children[v]) + ")" + brl

    return emit(root, None) + ";"


def simulate_dna(rng, net: NetworkDesc, n_sites, freqs, exch, alpha, rate_cats=4):
    """Simulate DNA columns on displayed trees; returns codes [n_tips][n_sites]."""
    return simulate(rng, net, n_sites, freqs, exch, alpha, rate_cats)


def simulate(rng, net: NetworkDesc, n_sites, freqs, exch, alpha, rate_cats=4):
    """Simulate columns of any state count on displayed trees; returns state
    bitmasks (1 << state) [n_tips][n_sites]."""
    from . import model
    lam, U, Uinv = model.eigen(freqs, exch)
    rates = model.gamma_mean_rates(alpha, rate_cats)
    n_nodes = net.n_nodes
    r = net.n_reticulations
    cfg = rng.uniform(size=(n_sites, max(r, 1))) >= net.ret_first_probs[None, :] if r else None
    cat = rng.integers(0, rate_cats, size=n_sites)
    state = np.full((n_nodes, n_sites), -1, np.int64)
    cumf = np.cumsum(freqs)
    S = len(freqs)
    state[net.root] = np.minimum(np.searchsorted(cumf, rng.uniform(size=n_sites) * cumf[-1]), S - 1)
    ret_index = {int(v): k for k, v in enumerate(net.ret_node)}
    # parents before children
    order = [net.root]
    indeg = np.zeros(n_nodes, np.int64)
    for c in net.edge_child:
        indeg[c] += 1
    queue = [net.root]
    while queue:
        v = queue.pop()
        for j in range(2):
            e = net.node_child_edges[2 * v + j]
            if e < 0:
                continue
            c = net.edge_child[e]
            indeg[c] -= 1
            if indeg[c] == 0:
                order.append(c)
                queue.append(c)
    S_ = len(freqs)

    def pmats(blen):
        # [rate_cats, S, S]: U diag(exp(lam t r_c)) Uinv, clipped at 0
        P = np.einsum("ik,ck,kj->cij", U, np.exp(lam[None, :] * (blen * rates)[:, None]), Uinv)
        return np.clip(P, 0.0, None)

    for c in order[1:]:
        if c in ret_index:
            k = ret_index[c]
            e1, e2 = net.ret_first_edge[k], net.ret_second_edge[k]
            take2 = cfg[:, k]
            pstate = np.where(take2, state[net.edge_parent[e2]], state[net.edge_parent[e1]])
            rows = np.where(take2[:, None], pmats(net.branch_lengths[e2])[cat, pstate],
                            pmats(net.branch_lengths[e1])[cat, pstate])
        else:
            e = int(np.nonzero(net.edge_child == c)[0][0])
            rows = pmats(net.branch_lengths[e])[cat, state[net.edge_parent[e]]]   # [n, S]
        cum = np.cumsum(rows, axis=1)
        u = rng.uniform(size=n_sites) * cum[:, -1]
        state[c] = np.minimum((u[:, None] > cum).sum(axis=1), S_ - 1)
    return (1 << state[:net.n_tips]).astype(np.uint32)


def compress(codes):
    """Pattern compression: distinct columns (in byte order of the column) and
    their multiplicities."""
    c = np.ascontiguousarray(codes.T.astype(np.uint32))
    v = c.view(np.dtype((np.void, c.shape[1] * 4))).ravel()
    _, first, counts = np.unique(v, return_index=True, return_counts=True)
    return np.ascontiguousarray(c[first].T), counts.astype(np.float64)


def make_protein_workload(name, n_taxa, n_ret, partition_sites, seed, alpha=0.8):
    """LG-like 20-state model: 190 exchangeabilities ~ Gamma(1, 1), frequencies
    ~ Dirichlet(1^20), Gamma shape alpha, 4 mean-rate categories."""
    rng = np.random.default_rng(seed)
    text = random_network_newick(rng, n_taxa, n_ret)
    net = parse_extended_newick(text)
    parts = []
    for ns in partition_sites:
        freqs = np.maximum(rng.dirichlet(np.ones(20)), 1e-3)
        freqs /= freqs.sum()
        exch = np.maximum(rng.gamma(1.0, 1.0, size=190), 1e-3)
        codes = simulate(rng, net, ns, freqs, exch, alpha)
        pat, w = compress(codes)
        parts.append(PartitionData(pat, w, freqs, exch, alpha, ns, states=20))
    return Workload(name, text, net, parts, seed)


def make_workload(name, n_taxa, n_ret, partition_sites, seed, alpha=0.8):
    rng = np.random.default_rng(seed)
    text = random_network_newick(rng, n_taxa, n_ret)
    net = parse_extended_newick(text)
    parts = []
    for ns in partition_sites:
        freqs = rng.dirichlet(np.ones(4))
        freqs = np.maximum(freqs, 1e-3)
        freqs /= freqs.sum()
        exch = rng.dirichlet(np.ones(6)) * 6.0
        exch = np.maximum(exch, 1e-3)
        codes = simulate_dna(rng, net, ns, freqs, exch, alpha)
        pat, w = compress(codes)
        parts.append(PartitionData(pat, w, freqs, exch, alpha, ns))
    return Workload(name, text, net, parts, seed)


CONFIG_SEEDS = {0: 1000, 1: 1001, 2: 1002, 3: 1003, 4: 1004}
CONFIG1_SITES = [500, 1000, 2000, 3000, 5000, 7000, 10000, 12000, 15000, 20000]


def candidate_specs(n=64, scale=1.0, seed=None):
    """Shapes of the candidate networks of one search move, drawn
    independently: taxa ~ U{30..120}, reticulations ~ U{0..6}, 1-8 partitions
    of U{1k..30k} DNA sites each (``scale`` shrinks the site counts)."""
    rng = np.random.default_rng(CONFIG_SEEDS[4] if seed is None else seed)
    out = []
    for i in range(n):
        nt = int(rng.integers(30, 121))
        nr = int(rng.integers(0, 7))
        npart = int(rng.integers(1, 9))
        sites = [max(32, int(round(int(rng.integers(1000, 30001)) * scale))) for _ in range(npart)]
        out.append(("candidate %d: %d taxa / %d reticulations / %d partitions" % (i, nt, nr, npart),
                    nt, nr, sites, int(rng.integers(0, 2 ** 31))))
    return out


def _make_candidate(spec):
    return make_workload(*spec)


def candidate_batch(n=64, scale=1.0, seed=None, workers=1):
    """Workloads of ``candidate_specs``; ``workers`` > 1 simulates them in a
    spawned process pool (start it before any GPU work in the caller)."""
    specs = candidate_specs(n, scale, seed)
    if workers <= 1:
        return [make_workload(*sp) for sp in specs]
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_make_candidate, specs))


def config(idx, scale=1.0):
    """Configurations 0-2 (DNA), 3 (protein) and 4 (a batch of 64 candidate
    networks, returned as a list of workloads). ``scale`` shrinks the site counts."""
    s = lambda n: max(32, int(round(n * scale)))
    if idx == 0:
        return make_workload("20 taxa / 1 reticulation / 1k DNA sites", 20, 1, [s(1000)], CONFIG_SEEDS[0])
    if idx == 1:
        return make_workload("50 taxa / 4 reticulations / 10 DNA partitions (75.5k sites)", 50, 4,
                             [s(n) for n in CONFIG1_SITES], CONFIG_SEEDS[1])
    if idx == 2:
        return make_workload("100 taxa / 8 reticulations / 100k DNA sites", 100, 8, [s(100000)],
                             CONFIG_SEEDS[2])
    if idx == 3:
        return make_protein_workload("40 taxa / 3 reticulations / 50k protein sites", 40, 3, [s(50000)],
                                     CONFIG_SEEDS[3])
    if idx == 4:
        return candidate_batch(64, scale)
    raise ValueError("config %d is not built" % idx)
