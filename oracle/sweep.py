"""Whole-DAG FP64 sweeps in C over the schedule ``improved.py`` enumerates.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the checker of the GPU
library at the full sizes of the benchmark workloads, and the timed CPU
baseline. ``sweep.c`` holds the arithmetic; this module flattens an
``ImprovedOracle``'s displayed-tree DAG (after ``loglikelihood()``, which
runs the reference's enumeration, ``ImprovedLoglikelihood.cpp:194-408``) into
a post-order op list and runs:

* the forward pruning of every variant with libpll's per-site scaling and the
  root log-likelihood of every displayed tree (``:125-190``, ``:410-486``),
* the AVERAGE / BEST mixture per partition (``evaluateTreesPartition``,
  ``:521-604``; FP64 log-sum-exp, which at 53 bits is what the MPFR sum
  computes),
* an adjoint sweep giving d logL / d every branch length, and
  d logL / d p_k = sum_T w_T d log P(T) / d p_k for the reticulation
  probabilities (``P(T)`` over the tree's configuration set,
  ``ReticulationConfigSet.cpp:70-130``).
"""
import ctypes
import math

import numpy as np

from . import build as cbuild
from . import configsets as cs
from . import pllmath
from .improved import AVERAGE

FAKE = -2 ** 31


class _Op(ctypes.Structure):
    _fields_ = [("out", ctypes.c_int32), ("a", ctypes.c_int32), ("b", ctypes.c_int32),
                ("ea", ctypes.c_int32), ("eb", ctypes.c_int32), ("first", ctypes.c_int32)]


class _Part(ctypes.Structure):
    _fields_ = [("R", ctypes.c_int32), ("S", ctypes.c_int32), ("n", ctypes.c_int64),
                ("tips", ctypes.c_void_p), ("weights", ctypes.c_void_p), ("freqs", ctypes.c_void_p),
                ("rate_weights", ctypes.c_void_p), ("pmat", ctypes.c_void_p), ("dpmat", ctypes.c_void_p),
                ("clv", ctypes.c_void_p), ("scaler", ctypes.c_void_p), ("adj", ctypes.c_void_p),
                ("gamma_frac", ctypes.c_double), ("inv_term", ctypes.c_void_p)]


def _lib():
    L = cbuild.lib()
    if not getattr(L, "_sweep_ready", False):
        L.oracle_sweep_forward.argtypes = [ctypes.c_int32, ctypes.POINTER(_Op), ctypes.c_int32,
                                           ctypes.POINTER(_Part), ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p]
        L.oracle_sweep_forward.restype = ctypes.c_int
        L.oracle_sweep_adjoint.argtypes = [ctypes.c_int32, ctypes.POINTER(_Op), ctypes.c_int32, ctypes.c_int32,
                                           ctypes.POINTER(_Part), ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
        L.oracle_sweep_adjoint.restype = ctypes.c_int
        L.oracle_sweep_threads.restype = ctypes.c_int
        L._sweep_ready = True
    return L


def threads():
    return int(_lib().oracle_sweep_threads())


class SweepOracle:
    """Forward + adjoint over an enumerated ``ImprovedOracle``.

    ``variant_of[(node, index)]`` maps the oracle's per-node variant to the
    CLV index used here (post-order over ``travbuffer``)."""

    def __init__(self, orc, with_gradient=True):
        if orc.pernode is None:
            orc.loglikelihood()
        self.orc = orc
        net = orc.net
        self.variant_of = {}
        for v in orc.travbuffer:
            if v < net.n_tips:
                continue
            for i, t in enumerate(orc.pernode[v]):
                self.variant_of[(v, i)] = len(self.variant_of)
        ops = []
        for v in orc.travbuffer:
            if v < net.n_tips:
                continue
            for i, t in enumerate(orc.pernode[v]):
                (ln, li, le), rinfo = t.children
                a = -1 - ln if orc.pernode[ln][li].is_tip else self.variant_of[(ln, li)]
                if rinfo is None:
                    b, eb = FAKE, -1
                else:
                    rn, ri, re = rinfo
                    b = -1 - rn if orc.pernode[rn][ri].is_tip else self.variant_of[(rn, ri)]
                    eb = re
                ops.append((self.variant_of[(v, i)], a, b, le, eb, 0))
        self.n_var = len(self.variant_of)
        self.ops = (_Op * len(ops))(*[_Op(*o) for o in ops])
        # displayed trees in use and their root slots
        self.trees = [t for t in orc.root_trees() if t.logprob >= orc.min_lp]
        slots = []
        self.tree_slot = []
        for t in self.trees:
            v = self.variant_of[t.dtroot]
            if v not in slots:
                slots.append(v)
            self.tree_slot.append(slots.index(v))
        self.slots = np.array(slots, np.int32)
        # adjoint ops: variants reachable from a used root slot, parents first
        # (a variant's first adjoint contribution stores, later ones add:
        # seeds come first, then messages in this order)
        reach = np.zeros(self.n_var, bool)
        reach[self.slots] = True
        bwd = []
        for o in reversed(ops):
            if reach[o[0]]:
                first = 0
                for bit, c in ((1, o[1]), (2, o[2])):
                    if c >= 0:
                        if not reach[c]:
                            first |= bit
                        reach[c] = True
                bwd.append(o[:5] + (first,))
        self.bwd = (_Op * len(bwd))(*[_Op(*o) for o in bwd])
        self.n_bwd = len(bwd)
        self.covered = [sorted(cs.covered_trees(t.configs, orc.r)) for t in self.trees]
        # partition buffers
        self.keep = []
        self.parts = (_Part * len(orc.parts))()
        for p, part in enumerate(orc.parts):
            rec = self.parts[p]
            rec.R, rec.S, rec.n = part.R, part.S, part.n
            rec.gamma_frac = part.gamma_frac
            clv = np.empty((self.n_var, part.n, part.R, part.S))
            sc = np.empty((self.n_var, part.n), np.uint32)
            adj = np.empty_like(clv) if with_gradient else None
            pm = np.empty((net.n_edges, part.R, part.S, part.S))
            dpm = np.empty_like(pm)
            arrs = dict(tips=part.tip_codes, weights=part.weights, freqs=part.freqs,
                        rate_weights=part.rate_weights, pmat=pm, dpmat=dpm, clv=clv, scaler=sc, adj=adj,
                        inv_term=part.inv_term)
            for k, a in arrs.items():
                if a is not None:
                    assert a.flags["C_CONTIGUOUS"]
                    setattr(rec, k, a.ctypes.data)
            self.keep.append(arrs)
        self.site_updates = sum(part.n for part in orc.parts) * self.n_var

    def _pmats(self, brlen, grad):
        for p, part in enumerate(self.orc.parts):
            pm, dpm = self.keep[p]["pmat"], self.keep[p]["dpmat"]
            lengths = brlen if self.orc.part_brlen is None or brlen is not self.orc.brlen else self.orc.lengths(p)
            for e, t in enumerate(lengths):
                pm[e] = pllmath.pmatrices(part.lam, part.U, part.Uinv, t, part.rates)
                if grad:
                    dpm[e] = pllmath.dpmatrices(part.lam, part.U, part.Uinv, t, part.rates)

    def evaluate(self, brlen=None, gradient=True):
        """(total, partition logL [P], per-tree logL [n_trees][P], d logL / d
        branch length [n_edges] or None, d logL / d p_k [r] or None). With
        ``brlen`` None the oracle's own lengths (per partition where it has
        them); the per-partition gradient of the last call is kept in
        ``grad_per_partition`` [P][n_edges]."""
        orc = self.orc
        brlen = orc.brlen if brlen is None else brlen
        L = _lib()
        P = len(orc.parts)
        self._pmats(brlen, gradient)
        slot_logl = np.empty((len(self.slots), P))
        if L.oracle_sweep_forward(len(self.ops), self.ops, P, self.parts, len(self.slots),
                                  self.slots.ctypes.data, slot_logl.ctypes.data):
            raise MemoryError("oracle_sweep_forward")
        lp = np.array([t.logprob for t in self.trees])
        tree_logl = slot_logl[self.tree_slot]                     # [trees][P]
        a = lp[:, None] + tree_logl
        if orc.variant == AVERAGE:
            m = a.max(axis=0)
            e = np.exp(a - m[None, :])
            part_logl = m + np.log(e.sum(axis=0))
            w = e / e.sum(axis=0)[None, :]
        else:
            part_logl = a.max(axis=0)
            w = np.zeros_like(a)
            w[np.argmax(a, axis=0), np.arange(P)] = 1.0
        total = float(math.fsum(part_logl))
        if not gradient:
            return total, part_logl, tree_logl, None, None
        slot_w = np.zeros((len(self.slots), P))
        for i, s in enumerate(self.tree_slot):
            slot_w[s] += w[i]
        gpp = np.empty((P, orc.net.n_edges))
        if L.oracle_sweep_adjoint(self.n_bwd, self.bwd, self.n_var, P, self.parts, len(self.slots),
                                  self.slots.ctypes.data, slot_w.ctypes.data, orc.net.n_edges,
                                  gpp.ctypes.data):
            raise MemoryError("oracle_sweep_adjoint")
        self.grad_per_partition = gpp
        grad = gpp.sum(axis=0)
        r = orc.r
        probs = orc.ret_probs
        gret = np.zeros(r)
        for i, cov in enumerate(self.covered):
            Pt = 0.0
            dP = np.zeros(r)
            for c in cov:
                f = [(1.0 - probs[k]) if (c >> k) & 1 else probs[k] for k in range(r)]
                Pt += math.prod(f)
                for k in range(r):
                    rest = math.prod(f[j] for j in range(r) if j != k)
                    dP[k] += -rest if (c >> k) & 1 else rest
            gret += w[i].sum() * dP / Pt
        return total, part_logl, tree_logl, grad, gret
