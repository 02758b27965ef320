"""Oracle cross-check: naive evaluation over all 2^r displayed trees.

Test infrastructure only. Restates ``computeLoglikelihoodNaiveUtree``
(``src/likelihood/NaiveLoglikelihood.cpp:35-115``): every full reticulation
configuration is turned into its displayed tree with unary nodes removed and
their branch lengths summed (``src/helper/NetworkFunctions.cpp:132-226``) and
scored on its own; AVERAGE mixes ``P(T) L_T`` per partition, BEST takes
``max_T log P(T) + logL_T`` over single trees. It shares no schedule code with
``improved.py`` (only the libpll arithmetic of ``clv.c``), so agreement checks
the displayed-tree DAG; P(a)P(b) = P(a+b) keeps the difference near 1e-12.
"""
import math

import mpmath
import numpy as np

from . import build as cbuild
from .improved import AVERAGE


def _tree_logl(orc, part, p):
    """Score the displayed tree of the oracle's current toggles for partition p."""
    dead, dt = orc.collect_dead_nodes()

    def alive_children(u):
        return orc._active_alive_children(u, dead)

    def down(u, parent_edge_len):
        """Follow unary chains; return (node with 0 or 2 children, summed length)."""
        length = parent_edge_len
        while True:
            ch = alive_children(u)
            if len(ch) != 1 or u < orc.net.n_tips:
                return u, length
            c = ch[0]
            length += orc.lengths(p)[orc.edge_to(u, c)]
            u = c

    def clv_of(u):
        if u < orc.net.n_tips:
            return part.tip_clv(u), None
        ch = alive_children(u)
        assert len(ch) == 2, "inner node of a displayed tree must be binary"
        ops = []
        for c in ch:
            end, length = down(c, orc.lengths(p)[orc.edge_to(u, c)])
            clv, sc = clv_of(end)
            ops.append((clv, sc, part.pmat(length)))
        parent = np.empty((part.n, part.R, part.S))
        ps = np.zeros(part.n, dtype=np.uint32)
        (lc, ls, pl), (rc, rs, pr) = ops
        cbuild.update_partial(parent, ps, lc, ls, pl, rc, rs, pr)
        return parent, ps

    clv, sc = clv_of(dt)
    return cbuild.root_logl(clv, sc, part.freqs, part.rate_weights, part.weights,
                            gamma_frac=part.gamma_frac, inv_term=part.inv_term)


def naive_loglikelihood(orc):
    """Returns (network logL, per-tree [tree][partition] logL, per-tree logprob)."""
    r = orc.r
    n_trees = 1 << r
    per_tree, logprob = [], []
    for t in range(n_trees):
        lp = 0.0
        for k in range(r):
            second = (t >> k) & 1
            orc.toggle[k] = second
            lp += orc.second_lp[k] if second else orc.first_lp[k]
        logprob.append(lp)
        per_tree.append([_tree_logl(orc, part, p) for p, part in enumerate(orc.parts)])
    total = 0.0
    for p in range(len(orc.parts)):
        if orc.variant == AVERAGE:
            with mpmath.workprec(53):
                acc = mpmath.mpf(0)
                for t in range(n_trees):
                    acc += mpmath.exp(per_tree[t][p]) * mpmath.exp(logprob[t])
                total += float(mpmath.log(acc))
        else:
            total += max(per_tree[t][p] + logprob[t] for t in range(n_trees))
    return total, per_tree, logprob
