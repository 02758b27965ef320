"""Oracle: branch-length derivatives the way the reference computes them.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``). Nothing in the product
imports it; ``tests/`` use it as the checker of the adjoint gradient and of
``netlk_edge_derivatives``.

The reference differentiates one branch at a time. For the edge of
``pmatrix_index`` it virtually reroots the network at the edge, pairs every
displayed tree on the source side with every compatible one on the target
side, builds a *sumtable* per pair and lets libpll turn it into the pair
tree's log-likelihood and its first and second derivatives
(``computePartitionSumtables`` / ``computeSumtable``,
``src/likelihood/LikelihoodDerivatives.cpp:249-344``;
``pll_update_sumtable`` / ``pll_compute_loglikelihood_derivatives``, called at
``:271-280`` and ``:95-104``). ``computeTreeDerivatives`` (``:13-23``) turns
log-derivatives into likelihood derivatives and ``computePartitionLhData``
(``:30-188``) combines the trees: AVERAGE as
``logL' = sum p L' / sum p L``,
``logL'' = (sum p L'' * sum p L - (sum p L')^2) / (sum p L)^2`` in MPFR
(restated in mpmath at 53 bits), BEST as the derivatives of the tree with the
largest ``tree_logl * tree_prob``.

What this module restates, and how:

* The displayed trees come from the naive per-configuration construction
  (``oracle/naive.py``: dead nodes, unary chains merged with their lengths
  summed), one representative configuration per displayed-tree root variant
  of ``improved.py`` (every configuration of a variant has the same tree).
  A tree's derivative w.r.t. a network edge is the derivative w.r.t. the
  merged branch that contains it (0 when the tree does not contain it).
* The sumtable (libpll is not vendored; this follows the published method):
  at a branch with partial likelihood ``A`` on the parent side (everything
  outside the child's subtree, root frequencies included) and ``B`` below,
  with ``P(t) = U diag(exp(lambda t)) U^-1``,
  ``L_s(t) = sum_r w_r sum_m (A_r U)_m (U^-1 B_r)_m exp(lambda_m rho_r t)``;
  the derivatives multiply each term by ``lambda_m rho_r`` and its square.
  Sites are scaled in FP64 by their maximum (a log scale per site), so no
  case underflows.
* Which trees take part. ``mode="true"``: every displayed tree with
  ``log P(T) >= log(1e-6)`` - the exact derivative of the network
  log-likelihood, which the adjoint gradient computes. ``mode="reference"``:
  only trees on which the edge is active (``isActiveBranch``,
  ``src/helper/EdgeHelper.cpp:84-95``: a reticulation edge counts where the
  tree's configuration set takes it, a tree edge always), and BEST by
  ``tree_logl * tree_prob`` (``LikelihoodDerivatives.cpp:162-166``). Trees are
  grouped by displayed-tree root variant; the reference groups by the rerooted
  (source, target) pairs at the edge, which gives the same sums unless a
  tree's probability straddles the 1e-6 cut-off.
* Reticulation probabilities: ``d logL_p / d p_k = sum_T w_T d log P(T) / d p_k``
  with the posterior weights ``w_T = P(T) L_T / sum P L`` (AVERAGE) or the
  argmax indicator (BEST), ``P(T) = sum over the variant's configurations of
  prod_k (p_k or 1 - p_k)`` (``ReticulationConfigSet.cpp:70-130``).
"""
import math

import mpmath
import numpy as np

from . import configsets as cs
from .improved import AVERAGE


def _displayed_tree(orc, brlen):
    """The current configuration's displayed tree with lengths ``brlen``:
    (root, children) where children[u] = [(child end node, merged length,
    [network edge ids])]."""
    dead, dt = orc.collect_dead_nodes()
    children = {}

    def build(u):
        if u < orc.net.n_tips:
            return
        ch = orc._active_alive_children(u, dead)
        assert len(ch) == 2, "inner node of a displayed tree must be binary"
        out = []
        for c in ch:
            e = orc.edge_to(u, c)
            edges, length, v = [e], brlen[e], c
            while v >= orc.net.n_tips:
                nxt = orc._active_alive_children(v, dead)
                if len(nxt) != 1:
                    break
                e2 = orc.edge_to(v, nxt[0])
                edges.append(e2)
                length += brlen[e2]
                v = nxt[0]
            out.append((v, length, edges))
            build(v)
        children[u] = out

    build(dt)
    return dt, children


def _scaled(x, logscale):
    """Divide each site of x [n][R][S] by its maximum; returns (x, logscale)."""
    m = x.max(axis=(1, 2))
    m = np.where(m > 0, m, 1.0)
    return x / m[:, None, None], logscale + np.log(m)


def _pmats(part, t):
    return np.stack([part.pmat(t)[r] for r in range(part.R)])


def _tree_derivatives(orc, part, n_edges, brlen):
    """(logL_T, d1[e], d2[e]) of the current configuration's displayed tree
    for one partition with lengths ``brlen``; d1, d2 are 0 for edges the tree
    does not contain."""
    dt, children = _displayed_tree(orc, brlen)
    n = part.n
    down, dscale = {}, {}

    def post(u):
        if u < orc.net.n_tips:
            down[u], dscale[u] = part.tip_clv(u), np.zeros(n)
            return
        prod, sc = np.ones((n, part.R, part.S)), np.zeros(n)
        for v, length, _ in children[u]:
            post(v)
            prod = prod * np.einsum("rij,nrj->nri", _pmats(part, length), down[v])
            sc = sc + dscale[v]
        down[u], dscale[u] = _scaled(prod, sc)

    post(dt)
    rho = part.rates
    x = part.lam[None, :] * rho[:, None]            # [R][m] exponents per unit length
    d1 = np.zeros(n_edges)
    d2 = np.zeros(n_edges)
    logl_seen = []
    # parent-side vectors: top[u] = partial likelihood of everything outside
    # u's subtree, as a function of u's state (root frequencies included)
    top = {dt: (np.broadcast_to(part.freqs, (n, part.R, part.S)).copy(), np.zeros(n))}
    stack = [dt]
    while stack:
        u = stack.pop()
        if u < orc.net.n_tips:
            continue
        tu, tsc = top[u]
        below = [np.einsum("rij,nrj->nri", _pmats(part, length), down[v]) for v, length, _ in children[u]]
        for k, (v, length, edges) in enumerate(children[u]):
            sib = below[1 - k]
            A, asc = _scaled(tu * sib, tsc + dscale[children[u][1 - k][0]])
            B, bsc = down[v], dscale[v]
            # sumtable [n][R][m]: parent side through U, child side through U^-1
            st = np.einsum("nri,im->nrm", A, part.U) * np.einsum("mj,nrj->nrm", part.Uinv, B)
            e0 = np.exp(x * length)[None, :, :]
            w = part.rate_weights[None, :, None]
            L0 = part.gamma_frac * (w * st * e0).sum(axis=(1, 2))
            L1 = part.gamma_frac * (w * st * x[None] * e0).sum(axis=(1, 2))
            L2 = part.gamma_frac * (w * st * (x * x)[None] * e0).sum(axis=(1, 2))
            sc = asc + bsc
            if part.inv_term is None:
                logl_seen.append(float(np.dot(part.weights, np.log(L0) + sc)))
                den = L0
            else:
                # + pinv * pi(invariant state) per site, in the scaled units of L0
                with np.errstate(divide="ignore"):
                    logl_seen.append(float(np.dot(part.weights,
                                                  np.logaddexp(np.log(L0) + sc, np.log(part.inv_term)))))
                den = L0 + part.inv_term * np.exp(np.minimum(-sc, 700.0))
            g1 = float(np.dot(part.weights, L1 / den))
            g2 = float(np.dot(part.weights, L2 / den - (L1 / den) ** 2))
            for e in edges:
                d1[e], d2[e] = g1, g2
            # top of v: sum_i A_i P_ij(length) (A already holds u's outside and the sibling)
            top[v] = (np.einsum("nri,rij->nrj", A, _pmats(part, length)), asc)
            stack.append(v)
    logl = logl_seen[0]
    assert all(abs(v - logl) <= 1e-9 * max(1.0, abs(logl)) for v in logl_seen), logl_seen
    return logl, d1, d2


class EdgeDerivativeOracle:
    """Per-displayed-tree log-likelihoods and branch derivatives of an
    ``ImprovedOracle`` (after ``loglikelihood()``), and their combinations."""

    def __init__(self, orc):
        self.orc = orc
        net = orc.net
        E = net.n_edges
        self.trees = []
        saved = list(orc.toggle)
        for t in orc.root_trees():
            covered = sorted(cs.covered_trees(t.configs, orc.r))
            rep = covered[0]
            for k in range(orc.r):
                orc.toggle[k] = (rep >> k) & 1
            per_part = [_tree_derivatives(orc, part, E, orc.lengths(p)) for p, part in enumerate(orc.parts)]
            self.trees.append({
                "logprob": t.logprob, "configs": covered,
                "logl": np.array([x[0] for x in per_part]),
                "d1": np.array([x[1] for x in per_part]),      # [part][edge]
                "d2": np.array([x[2] for x in per_part]),
            })
        orc.toggle = saved
        self.ret_edges = {}
        for k in range(orc.r):
            self.ret_edges[int(net.ret_first_edge[k])] = (k, 0)
            self.ret_edges[int(net.ret_second_edge[k])] = (k, 1)

    def _active(self, tree, e):
        """isActiveBranch on the tree's configuration set."""
        if e not in self.ret_edges:
            return True
        k, want = self.ret_edges[e]
        return any(((c >> k) & 1) == want for c in tree["configs"])

    def _use(self, tree):
        return tree["logprob"] >= self.orc.min_lp

    def edge(self, e, mode="true", partitions=None):
        """(d logL / d t_e, d2 logL / d t_e^2) summed over partitions (or
        over ``partitions``: each term is the derivative of the partition's
        logL w.r.t. its own length of the edge)."""
        ref = mode == "reference"
        trees = [t for t in self.trees if self._use(t) and (not ref or self._active(t, e))]
        D1 = D2 = 0.0
        for p in range(len(self.orc.parts)):
            if not trees or (partitions is not None and p not in partitions):
                continue
            if self.orc.variant == AVERAGE:
                with mpmath.workprec(53):
                    s0 = s1 = s2 = mpmath.mpf(0)
                    for t in trees:
                        lh = mpmath.exp(t["logl"][p])
                        a, b = t["d1"][p][e], t["d2"][p][e]
                        prob = mpmath.exp(t["logprob"])
                        s0 += lh * prob
                        s1 += lh * a * prob
                        s2 += (lh * a * a + lh * b) * prob
                    D1 += float(s1 / s0)
                    D2 += float((s2 * s0 - s1 * s1) / (s0 * s0))
            else:
                if ref:
                    best = max(trees, key=lambda t: t["logl"][p] * math.exp(t["logprob"]))
                else:
                    best = max(trees, key=lambda t: t["logl"][p] + t["logprob"])
                D1 += float(best["d1"][p][e])
                D2 += float(best["d2"][p][e])
        return D1, D2

    def gradient_per_partition(self):
        """d logL / d (partition p's length of edge e) [n_parts][n_edges]."""
        trees = [t for t in self.trees if self._use(t)]
        out = np.zeros((len(self.orc.parts), self.orc.net.n_edges))
        for p in range(len(self.orc.parts)):
            a = np.array([t["logprob"] + t["logl"][p] for t in trees])
            if self.orc.variant == AVERAGE:
                w = np.exp(a - a.max())
                w /= w.sum()
            else:
                w = np.zeros(len(trees))
                w[int(np.argmax(a))] = 1.0
            for i, t in enumerate(trees):
                out[p] += w[i] * t["d1"][p]
        return out

    def gradient(self):
        """(d logL / d branch length [n_edges], d logL / d p_k [r]), exact."""
        E = self.orc.net.n_edges
        r = self.orc.r
        g = np.zeros(E)
        gr = np.zeros(r)
        trees = [t for t in self.trees if self._use(t)]
        probs = self.orc.ret_probs
        # d log P(T) / d p_k
        dlp = []
        for t in trees:
            P = 0.0
            dP = np.zeros(r)
            for c in t["configs"]:
                f = [(1.0 - probs[k]) if (c >> k) & 1 else probs[k] for k in range(r)]
                P += math.prod(f)
                for k in range(r):
                    rest = math.prod(f[j] for j in range(r) if j != k)
                    dP[k] += -rest if (c >> k) & 1 else rest
            dlp.append(dP / P)
        for p in range(len(self.orc.parts)):
            if self.orc.variant == AVERAGE:
                a = np.array([t["logprob"] + t["logl"][p] for t in trees])
                w = np.exp(a - a.max())
                w /= w.sum()
            else:
                w = np.zeros(len(trees))
                w[int(np.argmax([t["logprob"] + t["logl"][p] for t in trees]))] = 1.0
            for i, t in enumerate(trees):
                g += w[i] * t["d1"][p]
                gr += w[i] * dlp[i]
        return g, gr
