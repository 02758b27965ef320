"""Oracle restatement of NetRAX's improved network log-likelihood.

Test infrastructure only. Follows ``src/likelihood/ImprovedLoglikelihood.cpp``:

* post-order over the reversed topological sort
  (``src/helper/NetworkFunctions.cpp:542-598``), ``processNodeImproved``
  (``:347-408``) with the single-child (``:194-223``) and two-children
  (``:225-345``) cases and the tree bookkeeping of ``:30-192``;
* restriction helpers and dead-node settings of
  ``src/helper/ReticulationConfigHelper.cpp:26-186``;
* displayed-tree roots via ``collect_dead_nodes``
  (``src/helper/NetworkFunctions.cpp:228-279``) and
  ``findMatchingDisplayedTree`` (``ReticulationConfigHelper.cpp:205-249``);
* per-tree root log-likelihoods (``:410-486``) and AVERAGE / BEST mixing
  (``:521-644``, MPFR restated with mpmath at 53 bits).

The FP64 arithmetic is ``clv.c`` (libpll restatement). ``gradient_fd`` gives
central finite differences of the same function.
"""
import math
from collections import deque

import mpmath
import numpy as np

from . import build as cbuild
from . import configsets as cs
from . import pllmath

AVERAGE, BEST = "AVERAGE", "BEST"
MIN_INTERESTING_LOGPROB = math.log(1e-6)   # src/NetraxOptions.hpp:108


class Partition:
    """One alignment partition: tips, weights and a GTR+Gamma(+I) model.

    ``pinv`` > 0 adds invariant sites (``pllmath`` docstring): ``rates`` are
    then the effective category rates rates / (1 - pinv), ``gamma_frac`` is
    1 - pinv and ``inv_term[s]`` = pinv * pi(invariant state of s) or 0."""

    def __init__(self, tip_codes, weights, freqs, exch, rates, rate_weights=None, pinv=0.0):
        self.tip_codes = np.ascontiguousarray(tip_codes, dtype=np.uint32)
        self.weights = np.ascontiguousarray(weights, dtype=np.float64)
        self.freqs = np.ascontiguousarray(freqs, dtype=np.float64)
        self.exch = np.asarray(exch, dtype=np.float64)
        self.pinv = float(pinv)
        self.rates = np.asarray(rates, dtype=np.float64) / (1.0 - self.pinv)
        self.gamma_frac = 1.0 - self.pinv
        self.inv_term = None
        if self.pinv > 0.0:
            st = pllmath.invariant_states(self.tip_codes)
            self.inv_term = np.ascontiguousarray(
                np.where(st >= 0, self.pinv * self.freqs[np.maximum(st, 0)], 0.0), dtype=np.float64)
        R = self.rates.size
        self.rate_weights = (np.full(R, 1.0 / R) if rate_weights is None
                             else np.ascontiguousarray(rate_weights, dtype=np.float64))
        self.S = self.freqs.size
        self.R = R
        self.n = self.tip_codes.shape[1]
        self.lam, self.U, self.Uinv, self.Q = pllmath.eigensystem(self.exch, self.freqs)

    def tip_clv(self, tip):
        return pllmath.tip_clv(self.tip_codes[tip], self.R, self.S)

    def pmat(self, t):
        return pllmath.pmatrices(self.lam, self.U, self.Uinv, t, self.rates)


class _Tree:
    """DisplayedTreeData + TreeLoglData (src/graph/DisplayedTreeData.hpp)."""

    def __init__(self, configs, is_tip=False):
        self.configs = configs
        self.is_tip = is_tip
        self.clv = None        # per partition [n][R][S]
        self.scaler = None     # per partition [n] uint32 (None for tips)
        self.clv_valid = False
        self.logprob = math.inf
        self.logprob_valid = False
        self.logl_valid = False
        self.partition_logl = None
        self.dtroot = None      # (node, index) of the tree used for the root logL
        self.children = None    # ((node, idx) or None, edge), ((node, idx)|None, edge)


class ImprovedOracle:
    def __init__(self, net, partitions, variant=AVERAGE,
                 min_interesting_logprob=MIN_INTERESTING_LOGPROB, width=None):
        self.net = net
        self.parts = partitions
        self.variant = variant
        self.min_lp = min_interesting_logprob
        self.r = net.n_ret
        self.width = width if width is not None else max(1, net.n_ret)
        self.brlen = list(net.edge_length)
        # per-partition lengths (the reference's unlinked / scaled linkage,
        # fake_treeinfo->branch_lengths[p]); None: every partition uses brlen
        self.part_brlen = None
        self.set_ret_probs(list(net.ret_first_prob))
        self.toggle = [0] * net.n_ret   # ReticulationData active_parent_toggle
        self.ret_index = {node: k for k, node in enumerate(net.ret_node)}
        self.update_count = 0           # site-CLV updates (pattern x variant)
        self.pernode = None

    # ----------------------------------------------------------- parameters
    def set_ret_probs(self, probs):
        self.ret_probs = list(probs)
        self.first_lp = [math.log(p) for p in probs] + [0.0] * (self.width - len(probs))
        self.second_lp = [math.log(1.0 - p) for p in probs] + [0.0] * (self.width - len(probs))

    def lengths(self, p):
        """Branch lengths partition p uses."""
        return self.brlen if self.part_brlen is None else self.part_brlen[p]

    # ------------------------------------------------------ network helpers
    def is_ret(self, v):
        return self.net.node_is_ret[v]

    def first_parent(self, v):
        return self.net.ret_first_parent[self.ret_index[v]]

    def second_parent(self, v):
        return self.net.ret_second_parent[self.ret_index[v]]

    def active_parent(self, v):
        if self.is_ret(v):
            k = self.ret_index[v]
            return self.net.ret_first_parent[k] if self.toggle[k] == 0 else self.net.ret_second_parent[k]
        p = self.net.tree_parent[v]
        return None if p < 0 else p

    def nonactive_parent(self, v):
        k = self.ret_index[v]
        return self.net.ret_second_parent[k] if self.toggle[k] == 0 else self.net.ret_first_parent[k]

    def children(self, v):
        """getChildren, src/helper/ChildrenHelper.cpp:6-21 (deduplicated)."""
        out = []
        for c in self.net.children[v]:
            if c not in out:
                out.append(c)
        return out

    def edge_to(self, parent, child):
        for c, e in zip(self.net.children[parent], self.net.child_edges[parent]):
            if c == child:
                return e
        raise KeyError((parent, child))

    def neighbors(self, v):
        """Link order: incoming links first, then outgoing (NetworkIO.cpp:113-221)."""
        out = []
        if self.is_ret(v):
            out += [self.first_parent(v), self.second_parent(v)]
        elif self.net.tree_parent[v] >= 0:
            out.append(self.net.tree_parent[v])
        out += self.net.children[v]
        res = []
        for x in out:
            if x not in res:
                res.append(x)
        return res

    def restr_take(self, node, neigh):
        """getRestrictionsToTakeNeighbor, ReticulationConfigHelper.cpp:64-93."""
        v = [cs.DC] * self.width
        if self.is_ret(node):
            k = self.ret_index[node]
            if neigh == self.first_parent(node):
                v[k] = cs.FIRST
            elif neigh == self.second_parent(node):
                v[k] = cs.SECOND
        if self.is_ret(neigh):
            k = self.ret_index[neigh]
            if node == self.first_parent(neigh):
                v[k] = cs.FIRST
            elif node == self.second_parent(neigh):
                v[k] = cs.SECOND
        return [tuple(v)]

    def restr_dismiss(self, node, neigh):
        """getRestrictionsToDismissNeighbor, ReticulationConfigHelper.cpp:26-62."""
        v = [cs.DC] * self.width
        found = False
        if self.is_ret(node):
            k = self.ret_index[node]
            if neigh == self.first_parent(node):
                v[k], found = cs.SECOND, True
            elif neigh == self.second_parent(node):
                v[k], found = cs.FIRST, True
        if self.is_ret(neigh):
            k = self.ret_index[neigh]
            if node == self.first_parent(neigh):
                v[k], found = cs.SECOND, True
            elif node == self.second_parent(neigh):
                v[k], found = cs.FIRST, True
        return [tuple(v)] if found else []

    def reversed_topological_sort(self):
        """Kahn's algorithm, NetworkFunctions.cpp:542-598."""
        n = self.net.n_nodes
        parent = [self.active_parent(i) for i in range(n)]
        outdeg = [len(self.children(i)) for i in range(n)]
        q = deque(i for i in range(n) if outdeg[i] == 0)
        res = []
        while q:
            a = q.popleft()
            res.append(a)
            if not self.is_ret(a):
                p = parent[a]
                if p is not None:
                    outdeg[p] -= 1
                    if outdeg[p] == 0:
                        q.append(p)
            else:
                for nb in self.neighbors(a):
                    if parent[nb] != a:
                        outdeg[nb] -= 1
                        if outdeg[nb] == 0:
                            q.append(nb)
        if len(res) != n:
            raise RuntimeError("Cycle in network detected")
        return res

    # ----------------------------------------------------- tree bookkeeping
    def _find(self, node, configs):
        for i, t in enumerate(self.pernode[node]):
            if cs.sets_equal(t.configs, configs):
                return i
        return None

    def _present_and_fine(self, node, configs):
        i = self._find(node, configs)
        if i is None:
            return False
        t = self.pernode[node][i]
        if not t.logprob_valid:
            t.logprob = cs.set_logprob(t.configs, self.first_lp, self.second_lp)
            t.logprob_valid = True
        return t.clv_valid or t.logprob < self.min_lp

    def _add_tree(self, node, configs):
        t = _Tree(configs)
        t.logprob = cs.set_logprob(configs, self.first_lp, self.second_lp)
        t.logprob_valid = True
        self.pernode[node].append(t)
        return t

    def _compute(self, node, tree, left, right):
        """pll_update_partials_single for every partition (:125-150, :164-190)."""
        (lnode, li, le), rinfo = left, right
        ltree = self.pernode[lnode][li]
        tree.clv, tree.scaler = [], []
        for p, part in enumerate(self.parts):
            parent = np.empty((part.n, part.R, part.S))
            ps = np.zeros(part.n, dtype=np.uint32)
            lclv = part.tip_clv(lnode) if ltree.is_tip else ltree.clv[p]
            lsc = None if ltree.is_tip else ltree.scaler[p]
            pl = part.pmat(self.lengths(p)[le])
            if rinfo is None:
                cbuild.update_partial(parent, ps, lclv, lsc, pl, None, None, None)
            else:
                rnode, ri, re = rinfo
                rtree = self.pernode[rnode][ri]
                rclv = part.tip_clv(rnode) if rtree.is_tip else rtree.clv[p]
                rsc = None if rtree.is_tip else rtree.scaler[p]
                cbuild.update_partial(parent, ps, lclv, lsc, pl, rclv, rsc,
                                      part.pmat(self.lengths(p)[re]))
            tree.clv.append(parent)
            tree.scaler.append(ps)
            self.update_count += part.n
        tree.children = (left, right)
        tree.clv_valid = True

    def _add_single(self, node, child, ci, configs):
        if self._present_and_fine(node, configs):
            return
        t = self._add_tree(node, configs)
        self._compute(node, t, (child, ci, self.edge_to(node, child)), None)

    def _add_both(self, node, lc, li, rc, ri, configs):
        if self._present_and_fine(node, configs):
            return
        t = self._add_tree(node, configs)
        self._compute(node, t, (lc, li, self.edge_to(node, lc)),
                      (rc, ri, self.edge_to(node, rc)))

    def _dead_node_settings(self, child_trees, parent, child):
        """deadNodeSettings, ReticulationConfigHelper.cpp:143-186."""
        res = list(self.restr_dismiss(parent, child))
        taken = self.restr_take(parent, child)
        for t in range(1 << self.r):
            tc = cs.tree_config(t, self.r, self.width)
            if not cs.sets_compatible(tc, taken):
                continue
            if not any(cs.sets_compatible(tc, ct.configs) for ct in child_trees):
                res.append(tc[0])
        cs.simplify(res)
        return res

    def _this_only(self, this_cfg, other_dead, parent, this_child, other_child):
        """getReticulationChoicesThisOnly, ReticulationConfigHelper.cpp:95-141."""
        res = []
        restricted = cs.combine(this_cfg, self.restr_take(parent, this_child))
        if not restricted:
            return res
        res += cs.combine(restricted, self.restr_dismiss(parent, other_child))
        restricted = cs.combine(restricted, self.restr_take(parent, other_child))
        res += cs.combine(restricted, other_dead)
        cs.simplify(res)
        return res

    def _process_single(self, node, child):
        restr = self.restr_take(node, child)
        for i, ct in enumerate(self.pernode[child]):
            if cs.sets_compatible(ct.configs, restr):
                self._add_single(node, child, i, cs.combine(ct.configs, restr))

    def _process_two(self, node, lc, rc):
        both = cs.combine(self.restr_take(node, lc), self.restr_take(node, rc))
        ltrees, rtrees = self.pernode[lc], self.pernode[rc]
        for i, lt in enumerate(ltrees):
            if not cs.sets_compatible(lt.configs, both):
                continue
            for j, rt in enumerate(rtrees):
                if not cs.sets_compatible(rt.configs, both):
                    continue
                if cs.sets_compatible(lt.configs, rt.configs):
                    c = cs.combine(lt.configs, rt.configs)
                    c = cs.combine(c, both)
                    self._add_both(node, lc, i, rc, j, c)
        rdead = self._dead_node_settings(rtrees, node, rc)
        for i, lt in enumerate(ltrees):
            only = self._this_only(lt.configs, rdead, node, lc, rc)
            if only:
                self._add_single(node, lc, i, only)
        ldead = self._dead_node_settings(ltrees, node, lc)
        for j, rt in enumerate(rtrees):
            only = self._this_only(rt.configs, ldead, node, rc, lc)
            if only:
                self._add_single(node, rc, j, only)

    # -------------------------------------------------- displayed-tree roots
    def _active_alive_children(self, u, dead):
        out = []
        for c in self.children(u):
            if dead[c]:
                continue
            if self.is_ret(c) and self.active_parent(c) != u:
                continue
            out.append(c)
        return out

    def collect_dead_nodes(self):
        """collect_dead_nodes, NetworkFunctions.cpp:228-279 (megablob root = root)."""
        n = self.net.n_nodes
        dead = [False] * n
        q = deque(self.nonactive_parent(self.net.ret_node[k]) for k in range(self.r))
        while q:
            u = q.popleft()
            if u is None:
                continue
            if len(self._active_alive_children(u, dead)) == 0:
                dead[u] = True
                if self.is_ret(u):
                    q.append(self.first_parent(u))
                    q.append(self.second_parent(u))
                else:
                    q.append(self.active_parent(u))
        dt = self.net.root
        ch = self._active_alive_children(dt, dead)
        while len(ch) == 1:
            dead[dt] = True
            dt = ch[0]
            ch = self._active_alive_children(dt, dead)
        return dead, dt

    def _apply_choices(self, vec):
        for k in range(self.r):
            if vec[k] == cs.FIRST:
                self.toggle[k] = 0
            elif vec[k] == cs.SECOND:
                self.toggle[k] = 1

    def _tree_logl(self, tree):
        """computeDisplayedTreeLoglikelihood, ImprovedLoglikelihood.cpp:410-486."""
        if not tree.logprob_valid:
            tree.logprob = cs.set_logprob(tree.configs, self.first_lp, self.second_lp)
            tree.logprob_valid = True
        if tree.logprob < self.min_lp:
            return
        self._apply_choices(tree.configs[0])
        _, dt = self.collect_dead_nodes()
        matches = [i for i, t in enumerate(self.pernode[dt])
                   if cs.sets_compatible(tree.configs, t.configs)]
        if len(matches) != 1:
            raise RuntimeError("Found %s suitable displayed trees" % len(matches))
        m = self.pernode[dt][matches[0]]
        tree.dtroot = (dt, matches[0])
        tree.partition_logl = []
        for p, part in enumerate(self.parts):
            ll = cbuild.root_logl(m.clv[p], m.scaler[p], part.freqs,
                                  part.rate_weights, part.weights, gamma_frac=part.gamma_frac,
                                  inv_term=part.inv_term)
            tree.partition_logl.append(ll)
        tree.logl_valid = True

    # ---------------------------------------------------------- evaluation
    def forward(self):
        """processPartitionsImproved, ImprovedLoglikelihood.cpp:488-519."""
        n = self.net.n_nodes
        self.update_count = 0
        self.pernode = [[] for _ in range(n)]
        for t in range(self.net.n_tips):
            self.pernode[t].append(_Tree([tuple([cs.DC] * self.width)], is_tip=True))
        self.travbuffer = self.reversed_topological_sort()
        for v in self.travbuffer:
            if v < self.net.n_tips:
                continue
            ch = self.children(v)
            if len(ch) > 2:
                raise RuntimeError("node with more than two children")
            if len(ch) == 1:
                self._process_single(v, ch[0])
            elif len(ch) == 2:
                self._process_two(v, ch[0], ch[1])
        for t in self.pernode[self.net.root]:
            self._tree_logl(t)

    def recompute(self):
        """Re-run the pruning of an enumerated DAG (after ``forward``) for new
        branch lengths: the arithmetic of processPartitionsImproved without the
        host-side enumeration. This is the timed CPU baseline."""
        self.update_count = 0
        pm = {}
        for p, part in enumerate(self.parts):
            for e in range(self.net.n_edges):
                pm[(p, e)] = part.pmat(self.lengths(p)[e])
        for v in self.travbuffer:
            for tree in self.pernode[v]:
                if tree.is_tip or tree.children is None:
                    continue
                (lnode, li, le), rinfo = tree.children
                ltree = self.pernode[lnode][li]
                for p, part in enumerate(self.parts):
                    lclv = part.tip_clv(lnode) if ltree.is_tip else ltree.clv[p]
                    lsc = None if ltree.is_tip else ltree.scaler[p]
                    if rinfo is None:
                        cbuild.update_partial(tree.clv[p], tree.scaler[p], lclv, lsc, pm[(p, le)],
                                              None, None, None)
                    else:
                        rnode, ri, re = rinfo
                        rtree = self.pernode[rnode][ri]
                        rclv = part.tip_clv(rnode) if rtree.is_tip else rtree.clv[p]
                        rsc = None if rtree.is_tip else rtree.scaler[p]
                        cbuild.update_partial(tree.clv[p], tree.scaler[p], lclv, lsc, pm[(p, le)],
                                              rclv, rsc, pm[(p, re)])
                    self.update_count += part.n
        for t in self.pernode[self.net.root]:
            if t.logprob < self.min_lp or t.dtroot is None:
                continue
            dn, di = t.dtroot
            m = self.pernode[dn][di]
            t.partition_logl = [cbuild.root_logl(m.clv[p], m.scaler[p], part.freqs, part.rate_weights,
                                                 part.weights, gamma_frac=part.gamma_frac,
                                                 inv_term=part.inv_term) for p, part in enumerate(self.parts)]
        return self.evaluate()[0]

    def root_trees(self):
        return self.pernode[self.net.root]

    def evaluate(self):
        """evaluateTrees / evaluateTreesPartition, :521-644."""
        trees = self.root_trees()
        part_logl = []
        for p in range(len(self.parts)):
            if self.variant == AVERAGE:
                with mpmath.workprec(53):
                    acc = mpmath.mpf(0)
                    for t in trees:
                        if t.logprob < self.min_lp:
                            continue
                        if not t.logl_valid:
                            raise RuntimeError("invalid tree logl")
                        acc += mpmath.exp(t.logprob) * mpmath.exp(t.partition_logl[p])
                    part_logl.append(float(mpmath.log(acc)))
            else:
                best = -math.inf
                for t in trees:
                    if t.logprob < self.min_lp:
                        continue
                    if not t.logl_valid:
                        raise RuntimeError("invalid tree logl")
                    best = max(best, t.logprob + t.partition_logl[p])
                part_logl.append(best)
        total = 0.0
        for x in part_logl:
            total += x
        if total == -math.inf:
            raise RuntimeError("Invalid network likelihood: negative infinity")
        return total, part_logl

    def loglikelihood(self):
        self.forward()
        return self.evaluate()[0]

    # ---------------------------------------------------------- gradients
    def gradient_fd(self, edges=None, h=1e-6):
        """Central finite differences of the network logL w.r.t. branch lengths."""
        edges = range(self.net.n_edges) if edges is None else edges
        base = list(self.brlen)
        out = {}
        for e in edges:
            self.brlen = list(base)
            self.brlen[e] = base[e] + h
            up = self.loglikelihood()
            self.brlen[e] = base[e] - h
            dn = self.loglikelihood()
            out[e] = (up - dn) / (2 * h)
        self.brlen = base
        return out

    def retprob_gradient_fd(self, h=1e-6):
        base = list(self.ret_probs)
        out = []
        for k in range(self.r):
            p = list(base)
            p[k] = base[k] + h
            self.set_ret_probs(p)
            up = self.loglikelihood()
            p[k] = base[k] - h
            self.set_ret_probs(p)
            dn = self.loglikelihood()
            out.append((up - dn) / (2 * h))
        self.set_ret_probs(base)
        return out

    # ------------------------------------------------------ introspection
    def dag_summary(self):
        """Per node: list of (covered tree-index set) in variant order."""
        out = {}
        for v in range(self.net.n_tips, self.net.n_nodes):
            out[v] = [frozenset(_covered(t.configs, self.r, self.width)) for t in self.pernode[v]]
        return out


def _covered(configs, r, width):
    res = set()
    for t in range(1 << r):
        if cs.sets_compatible(cs.tree_config(t, r, width), configs):
            res.add(t)
    return res
