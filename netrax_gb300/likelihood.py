"""Python host API over the netlk C ABI.

Mirrors the reference's likelihood entry points:

* ``NetworkLikelihood.loglikelihood()`` - ``computeLoglikelihood(ann_network,
  incremental, update_pmatrices)`` (``src/likelihood/LikelihoodComputation.hpp:17-18``);
  per-partition values mirror ``fake_treeinfo->partition_loglh`` and per-tree
  values ``TreeLoglData::tree_partition_logl``.
* ``loglikelihood_gradient()`` - one forward + one adjoint sweep giving
  d logL / d branch length for every edge and d logL / d reticulation
  probability, replacing the per-edge sumtable derivatives of
  ``src/likelihood/LikelihoodDerivatives.cpp:190-344``.
* ``set_branch_lengths`` / ``set_reticulation_probs`` / ``set_model`` - the
  parameter updates the optimizers make (``src/optimization/NetworkState.cpp``,
  ``ReticulationOptimization.cpp:25-38``).
* ``NetworkLogL`` - a ``torch.autograd.Function`` over branch lengths and
  reticulation probabilities.

All evaluation runs in the CUDA library; there is no CPU fallback.
"""
import ctypes
import math

import numpy as np

from . import _native as N
from .network import NetworkDesc

VARIANTS = {"AVERAGE": N.NETLK_AVERAGE, "BEST": N.NETLK_BEST}
PRECISIONS = {"fp64": N.NETLK_FP64, "fp32": N.NETLK_FP32}


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct)) if a is not None else None


class NetworkLikelihood:
    def __init__(self, network: NetworkDesc, partitions, variant="AVERAGE", precision="fp32",
                 min_interesting_tree_logprob=math.log(1e-6), device=0, use_cuda_graph=True,
                 host_only=False, rates=None, autotune=True, tensor_cores=True, checkpoint_segments=0,
                 incremental=True, brlen_linkage="linked", sumtables=True):
        L = N.lib()
        self.network = network
        self.n_parts = len(partitions)
        self.n_edges = network.n_edges
        self.n_ret = network.n_reticulations
        keep = []

        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a

        topo = N.Topology()
        topo.n_nodes = network.n_nodes
        topo.n_tips = network.n_tips
        topo.n_edges = network.n_edges
        topo.n_reticulations = network.n_reticulations
        topo.root = network.root
        topo.edge_parent = _ptr(arr(network.edge_parent, np.int32), ctypes.c_int32)
        topo.edge_child = _ptr(arr(network.edge_child, np.int32), ctypes.c_int32)
        topo.node_child_edges = _ptr(arr(network.node_child_edges, np.int32), ctypes.c_int32)
        topo.ret_node = _ptr(arr(network.ret_node, np.int32), ctypes.c_int32)
        topo.ret_first_edge = _ptr(arr(network.ret_first_edge, np.int32), ctypes.c_int32)
        topo.ret_second_edge = _ptr(arr(network.ret_second_edge, np.int32), ctypes.c_int32)
        parts = (N.Partition * self.n_parts)()
        self.n_patterns = []
        self.states = getattr(partitions[0], "states", 4)
        self.rate_cats = getattr(partitions[0], "rate_cats", 4)
        for i, pd in enumerate(partitions):
            p = parts[i]
            p.states = getattr(pd, "states", 4)
            p.rate_cats = getattr(pd, "rate_cats", 4)
            ts = arr(pd.tip_states, np.uint32)
            p.n_patterns = ts.shape[1]
            self.n_patterns.append(ts.shape[1])
            p.tip_states = _ptr(ts, ctypes.c_uint32)
            p.pattern_weights = _ptr(arr(pd.weights, np.float64), ctypes.c_double)
            p.freqs = _ptr(arr(pd.freqs, np.float64), ctypes.c_double)
            p.exchangeabilities = _ptr(arr(pd.exch, np.float64), ctypes.c_double)
            p.alpha = float(pd.alpha)
            r = None if rates is None else rates[i]
            p.rates = _ptr(arr(r, np.float64), ctypes.c_double) if r is not None else None
            p.rate_weights = None
            p.prop_invar = float(getattr(pd, "prop_invar", 0.0))
        opts = N.Options()
        L.netlk_options_default(ctypes.byref(opts))
        opts.variant = VARIANTS[variant]
        opts.precision = PRECISIONS[precision]
        opts.min_interesting_tree_logprob = float(min_interesting_tree_logprob)
        opts.device = int(device)
        opts.use_cuda_graph = int(bool(use_cuda_graph))
        opts.host_only = int(bool(host_only))
        opts.autotune = int(bool(autotune))
        opts.tensor_cores = int(bool(tensor_cores))
        opts.checkpoint_segments = int(checkpoint_segments)
        opts.incremental = int(bool(incremental))
        opts.brlen_linkage = {"linked": N.NETLK_BRLEN_LINKED, "unlinked": N.NETLK_BRLEN_UNLINKED,
                              "scaled": N.NETLK_BRLEN_SCALED}[brlen_linkage]
        opts.sumtables = int(bool(sumtables))
        bl = arr(network.branch_lengths, np.float64)
        rp = arr(network.ret_first_probs, np.float64) if self.n_ret else None
        h = ctypes.c_void_p()
        st = L.netlk_create(ctypes.byref(topo), parts, self.n_parts, _ptr(bl, ctypes.c_double),
                            _ptr(rp, ctypes.c_double), ctypes.byref(opts), ctypes.byref(h))
        N.check(st, None)
        self._h = h
        self.variant, self.precision = variant, precision
        self.branch_lengths = np.array(network.branch_lengths, np.float64)
        self.ret_probs = np.array(network.ret_first_probs, np.float64)
        st0 = self.stats
        self.n_roots = st0["n_root_variants"]
        self.n_variants = st0["n_variants"]

    @property
    def stats(self):
        """netlk_dag_stats as a dict, queried now (the launch count per
        evaluation follows the launch shapes the first evaluation chose)."""
        s = N.DagStats()
        N.check(N.lib().netlk_get_dag_stats(self._h, ctypes.byref(s)), self._h)
        return s.as_dict()

    # ----------------------------------------------------------- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            N.lib().netlk_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------- parameters
    def set_branch_lengths(self, b):
        b = np.ascontiguousarray(b, np.float64)
        N.check(N.lib().netlk_set_branch_lengths(self._h, _ptr(b, ctypes.c_double), b.size), self._h)
        self.branch_lengths = b.copy()

    def set_reticulation_probs(self, p):
        p = np.ascontiguousarray(p, np.float64)
        N.check(N.lib().netlk_set_reticulation_probs(self._h, _ptr(p, ctypes.c_double), p.size), self._h)
        self.ret_probs = p.copy()

    def set_model(self, part, freqs, exch, alpha, rates=None):
        f = np.ascontiguousarray(freqs, np.float64)
        x = np.ascontiguousarray(exch, np.float64)
        r = None if rates is None else np.ascontiguousarray(rates, np.float64)
        N.check(N.lib().netlk_set_model(self._h, part, _ptr(f, ctypes.c_double), _ptr(x, ctypes.c_double),
                                        float(alpha), _ptr(r, ctypes.c_double)), self._h)

    def set_partition_branch_lengths(self, part, b):
        """One partition's own branch lengths (unlinked contexts)."""
        b = np.ascontiguousarray(b, np.float64)
        N.check(N.lib().netlk_set_partition_branch_lengths(self._h, int(part), _ptr(b, ctypes.c_double), b.size),
                self._h)

    def set_branch_length_scalers(self, scalers):
        """Per-partition length scalers (scaled contexts)."""
        sc = np.ascontiguousarray(scalers, np.float64)
        N.check(N.lib().netlk_set_branch_length_scalers(self._h, _ptr(sc, ctypes.c_double), sc.size), self._h)

    def partition_gradient(self):
        """d logL / d (partition p's length of edge e) [n_parts][n_edges] of
        the last logL + gradient evaluation."""
        out = np.zeros(self.n_parts * self.n_edges)
        N.check(N.lib().netlk_partition_gradient(self._h, _ptr(out, ctypes.c_double)), self._h)
        return out.reshape(self.n_parts, self.n_edges)

    def edge_loglikelihood_partition(self, edge, part, length):
        tot = ctypes.c_double()
        N.check(N.lib().netlk_edge_loglikelihood_partition(self._h, int(edge), int(part), float(length),
                                                           ctypes.byref(tot)), self._h)
        return tot.value

    def edge_derivatives_partition(self, edge, part, mode=0):
        d1, d2 = ctypes.c_double(), ctypes.c_double()
        N.check(N.lib().netlk_edge_derivatives_partition(self._h, int(edge), int(part), int(mode), ctypes.byref(d1),
                                                         ctypes.byref(d2)), self._h)
        return d1.value, d2.value

    def edge_sumtable(self, edge):
        """Builds the edge's sumtables now: (built, number of tables); built
        is False where that path does not apply (evaluations then take the
        tangent path)."""
        built, n_tab = ctypes.c_int32(), ctypes.c_int32()
        N.check(N.lib().netlk_edge_sumtable(self._h, int(edge), ctypes.byref(built), ctypes.byref(n_tab)), self._h)
        return bool(built.value), n_tab.value

    def edge_sumtable_derivatives(self, edge, length, mode=0):
        """(logL, d1, d2) with ``edge`` at ``length``, the context unchanged:
        one length -> totals; one length per partition (unlinked) -> arrays."""
        lens = np.atleast_1d(np.asarray(length, dtype=np.float64))
        n = lens.size
        out = [np.zeros(n) for _ in range(3)]
        N.check(N.lib().netlk_edge_sumtable_derivatives(self._h, int(edge), _ptr(lens, ctypes.c_double), n,
                                                        int(mode), *[_ptr(o, ctypes.c_double) for o in out]),
                self._h)
        if np.ndim(length) == 0:
            return tuple(float(o[0]) for o in out)
        return tuple(out)

    def sumtable_export(self, edge):
        """The walk of an edge's table build: (ops [n, 7] = (x, d, o, mode,
        work slot read, work slot written, table), work slots, tables,
        group_ref, group_begin)."""
        n, w, t, g = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        N.check(N.lib().netlk_sumtable_export(self._h, int(edge), ctypes.byref(n), ctypes.byref(w), ctypes.byref(t),
                                              ctypes.byref(g), None, None, None), self._h)
        ops = np.zeros(7 * max(1, n.value), np.int32)
        gref = np.zeros(max(1, g.value), np.int32)
        gbeg = np.zeros(g.value + 1, np.int32)
        N.check(N.lib().netlk_sumtable_export(self._h, int(edge), ctypes.byref(n), ctypes.byref(w), ctypes.byref(t),
                                              ctypes.byref(g), _ptr(ops, ctypes.c_int32), _ptr(gref, ctypes.c_int32),
                                              _ptr(gbeg, ctypes.c_int32)), self._h)
        return ops[:7 * n.value].reshape(-1, 7), w.value, t.value, gref[:g.value], gbeg

    def set_prop_invar(self, part, prop_invar):
        """Proportion of invariant sites (+I) of one partition."""
        N.check(N.lib().netlk_set_prop_invar(self._h, int(part), float(prop_invar)), self._h)

    # ---------------------------------------------------------- evaluation
    def loglikelihood(self, details=False):
        tot = ctypes.c_double()
        pl = np.zeros(self.n_parts)
        tl = np.zeros(self.n_roots * self.n_parts) if details else None
        N.check(N.lib().netlk_loglikelihood(self._h, ctypes.byref(tot), _ptr(pl, ctypes.c_double),
                                            _ptr(tl, ctypes.c_double)), self._h)
        if details:
            return tot.value, pl, tl.reshape(self.n_roots, self.n_parts)
        return tot.value

    def loglikelihood_gradient(self, details=False):
        tot = ctypes.c_double()
        pl = np.zeros(self.n_parts)
        gb = np.zeros(self.n_edges)
        gr = np.zeros(max(1, self.n_ret))
        N.check(N.lib().netlk_loglikelihood_gradient(self._h, ctypes.byref(tot), _ptr(pl, ctypes.c_double),
                                                     _ptr(gb, ctypes.c_double), _ptr(gr, ctypes.c_double)),
                self._h)
        if details:
            return tot.value, gb, gr[:self.n_ret], pl
        return tot.value, gb, gr[:self.n_ret]

    def edge_loglikelihood(self, edge, length):
        """Network logL with branch ``edge`` set to ``length`` (kept)."""
        tot = ctypes.c_double()
        N.check(N.lib().netlk_edge_loglikelihood(self._h, int(edge), float(length), ctypes.byref(tot)), self._h)
        return tot.value

    def last_site_updates(self):
        n = ctypes.c_int64()
        N.check(N.lib().netlk_last_site_updates(self._h, ctypes.byref(n)), self._h)
        return n.value

    def edge_derivatives(self, edge, second=True, mode=0):
        """d logL / d t_edge (and the second derivative): mode 0 the true
        derivative, mode 1 the reference's own formula with its restrictions."""
        d1, d2 = ctypes.c_double(), ctypes.c_double()
        N.check(N.lib().netlk_edge_derivatives(self._h, edge, int(mode), ctypes.byref(d1),
                                               ctypes.byref(d2) if second else None), self._h)
        return (d1.value, d2.value) if second else d1.value

    def tree_partials(self):
        out = np.zeros(self.n_roots * self.n_parts)
        N.check(N.lib().netlk_tree_partials(self._h, _ptr(out, ctypes.c_double)), self._h)
        return out.reshape(self.n_roots, self.n_parts)

    def mix_and_backward(self, global_partials):
        g = np.ascontiguousarray(global_partials, np.float64).ravel()
        tot = ctypes.c_double()
        pl = np.zeros(self.n_parts)
        gb = np.zeros(self.n_edges)
        gr = np.zeros(max(1, self.n_ret))
        N.check(N.lib().netlk_mix_and_backward(self._h, _ptr(g, ctypes.c_double), ctypes.byref(tot),
                                               _ptr(pl, ctypes.c_double), _ptr(gb, ctypes.c_double),
                                               _ptr(gr, ctypes.c_double)), self._h)
        return tot.value, gb, gr[:self.n_ret], pl

    # ------------------------------------------------------- introspection
    def dag_export(self):
        V = self.n_variants
        words = max(1, (1 << self.n_ret) // 64)
        node = np.zeros(V, np.int32)
        ch = np.zeros(2 * V, np.int32)
        ed = np.zeros(2 * V, np.int32)
        cov = np.zeros(V * words, np.uint64)
        N.check(N.lib().netlk_dag_export(self._h, _ptr(node, ctypes.c_int32), _ptr(ch, ctypes.c_int32),
                                         _ptr(ed, ctypes.c_int32), _ptr(cov, ctypes.c_uint64), words), self._h)
        return node, ch.reshape(V, 2), ed.reshape(V, 2), cov.reshape(V, words)

    def root_export(self):
        R = self.n_roots
        rv = np.zeros(R, np.int32)
        dt = np.zeros(R, np.int32)
        lp = np.zeros(R)
        N.check(N.lib().netlk_root_export(self._h, _ptr(rv, ctypes.c_int32), _ptr(dt, ctypes.c_int32),
                                          _ptr(lp, ctypes.c_double)), self._h)
        return rv, dt, lp

    def adjoint_export(self):
        """Level adjoint schedule: (ops [n][7], slot_reads [m], level_begin [levels + 1])."""
        n, m, nl = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        N.check(N.lib().netlk_adjoint_export(self._h, ctypes.byref(n), ctypes.byref(m), ctypes.byref(nl),
                                             None, None, None), self._h)
        ops = np.zeros(7 * max(1, n.value), np.int32)
        reads = np.zeros(max(1, m.value), np.int32)
        lb = np.zeros(nl.value + 1, np.int32)
        N.check(N.lib().netlk_adjoint_export(self._h, ctypes.byref(n), ctypes.byref(m), ctypes.byref(nl),
                                             _ptr(ops, ctypes.c_int32), _ptr(reads, ctypes.c_int32),
                                             _ptr(lb, ctypes.c_int32)), self._h)
        return ops[:7 * n.value].reshape(-1, 7), reads[:m.value], lb

    def checkpoint_export(self):
        """(n_segments, n_clv_slots, var_slot [V], permanent [V], seg_levels [n_segments][2])."""
        ns, nc = ctypes.c_int32(), ctypes.c_int32()
        N.check(N.lib().netlk_checkpoint_export(self._h, ctypes.byref(ns), ctypes.byref(nc), None, None, None),
                self._h)
        V = self.n_variants
        slot = np.zeros(V, np.int32)
        perm = np.zeros(V, np.int32)
        seg = np.zeros(2 * ns.value, np.int32)
        N.check(N.lib().netlk_checkpoint_export(self._h, ctypes.byref(ns), ctypes.byref(nc),
                                                _ptr(slot, ctypes.c_int32), _ptr(perm, ctypes.c_int32),
                                                _ptr(seg, ctypes.c_int32)), self._h)
        return ns.value, nc.value, slot, perm, seg.reshape(-1, 2)

    def walk_export(self):
        """The walk schedule of the single-launch sweeps: (forward variants in
        walk order, adjoint ops [n, 6] = (variant, slot out a, slot out b,
        message from registers, first slot read, slot reads), slot reads);
        empty arrays when the context has no walk schedule."""
        nf, nb, ns = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        N.check(N.lib().netlk_walk_export(self._h, ctypes.byref(nf), ctypes.byref(nb), ctypes.byref(ns),
                                          None, None, None), self._h)
        fwd = np.zeros(max(1, nf.value), np.int32)
        bwd = np.zeros(max(1, 6 * nb.value), np.int32)
        slots = np.zeros(max(1, ns.value), np.int32)
        N.check(N.lib().netlk_walk_export(self._h, ctypes.byref(nf), ctypes.byref(nb), ctypes.byref(ns),
                                          _ptr(fwd, ctypes.c_int32), _ptr(bwd, ctypes.c_int32),
                                          _ptr(slots, ctypes.c_int32)), self._h)
        return fwd[:nf.value], bwd[:6 * nb.value].reshape(nb.value, 6), slots[:ns.value]

    def walk_segments(self):
        """Per checkpoint segment of the walk schedule: (adjoint op ranges
        [n_segments][2] into walk_export's adjoint ops, recomputed variants,
        their ranges [n_segments][2]); empty arrays without a walk schedule."""
        ns, nr = ctypes.c_int32(), ctypes.c_int32()
        N.check(N.lib().netlk_walk_segments(self._h, ctypes.byref(ns), ctypes.byref(nr), None, None, None),
                self._h)
        br = np.zeros(max(1, 2 * ns.value), np.int32)
        rv = np.zeros(max(1, nr.value), np.int32)
        rr = np.zeros(max(1, 2 * ns.value), np.int32)
        N.check(N.lib().netlk_walk_segments(self._h, ctypes.byref(ns), ctypes.byref(nr), _ptr(br, ctypes.c_int32),
                                            _ptr(rv, ctypes.c_int32), _ptr(rr, ctypes.c_int32)), self._h)
        return (br[:2 * ns.value].reshape(-1, 2), rv[:nr.value], rr[:2 * ns.value].reshape(-1, 2))

    def get_clv(self, variant, part):
        n = self.n_patterns[part]
        clv = np.zeros(n * self.rate_cats * self.states)
        sc = np.zeros(n, np.int32)
        N.check(N.lib().netlk_get_clv(self._h, variant, part, _ptr(clv, ctypes.c_double),
                                      _ptr(sc, ctypes.c_int32)), self._h)
        return clv.reshape(n, self.rate_cats, self.states), sc

    # ------------------------------------------------ device-resident stepping
    def set_branch_lengths_device(self, dev_ptr):
        """Enqueue a copy of branch lengths from a device pointer (e.g. a CUDA tensor)."""
        N.check(N.lib().netlk_set_branch_lengths_device(self._h, ctypes.c_void_p(dev_ptr), self.n_edges),
                self._h)

    def enqueue(self, with_gradient=True):
        N.check(N.lib().netlk_enqueue(self._h, int(bool(with_gradient))), self._h)

    def result_pointers(self):
        o, g = ctypes.c_void_p(), ctypes.c_void_p()
        N.check(N.lib().netlk_result_pointers(self._h, ctypes.byref(o), ctypes.byref(g)), self._h)
        return o.value, g.value

    def set_profiling(self, enable=True):
        N.check(N.lib().netlk_set_profiling(self._h, int(bool(enable))), self._h)

    KERNELS = ("pmatrix", "forward", "tree_reduce", "mix", "backward", "grad_reduce")

    def kernel_times(self):
        ms = np.zeros(6)
        cnt = np.zeros(6, np.int64)
        N.check(N.lib().netlk_kernel_times(self._h, _ptr(ms, ctypes.c_double),
                                           cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), 6), self._h)
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNELS)}

    def tuning(self, n=32):
        fs, bs = ctypes.c_int32(), ctypes.c_int32()
        fm, bm = np.zeros(n), np.zeros(n)
        N.check(N.lib().netlk_tuning(self._h, ctypes.byref(fs), ctypes.byref(bs), _ptr(fm, ctypes.c_double),
                                     _ptr(bm, ctypes.c_double), n), self._h)
        ws = ctypes.c_int32()
        N.check(N.lib().netlk_walk_shape_begin(self._h, ctypes.byref(ws)), self._h)
        return {"forward_shape": fs.value, "backward_shape": bs.value,
                "forward_walk": fs.value >= ws.value, "backward_walk": bs.value >= ws.value,
                "forward_ms": [x for x in fm if x > 0], "backward_ms": [x for x in bm if x > 0]}

    def stream(self):
        s = ctypes.c_void_p()
        N.check(N.lib().netlk_get_stream(self._h, ctypes.byref(s)), self._h)
        return s.value

    def launch_count(self):
        n = ctypes.c_int64()
        N.check(N.lib().netlk_launch_count(self._h, ctypes.byref(n)), self._h)
        return n.value


def compute_loglikelihood(lik: NetworkLikelihood, incremental=1, update_pmatrices=1):
    """Same role and arguments as the reference's ``computeLoglikelihood``.

    The context keeps the branch lengths its stored CLVs were computed with;
    with its ``incremental`` option on (the default) a call recomputes only
    the variants above the changed edges, otherwise every CLV. The P-matrices
    are recomputed on the GPU at every call, so the two arguments only exist
    for call-site parity.
    """
    del incremental, update_pmatrices
    return lik.loglikelihood()


try:
    import torch

    class NetworkLogL(torch.autograd.Function):
        """logL(branch_lengths, reticulation_probs) with the adjoint-sweep gradient."""

        @staticmethod
        def forward(ctx, branch_lengths, ret_probs, lik):
            lik.set_branch_lengths(branch_lengths.detach().cpu().double().numpy())
            if lik.n_ret:
                lik.set_reticulation_probs(ret_probs.detach().cpu().double().numpy())
            val, gb, gr = lik.loglikelihood_gradient()
            ctx.save_for_backward(torch.from_numpy(gb), torch.from_numpy(np.array(gr, np.float64)))
            ctx.devs = (branch_lengths.device, ret_probs.device)
            return torch.tensor(val, dtype=torch.float64, device=branch_lengths.device)

        @staticmethod
        def backward(ctx, grad_out):
            gb, gr = ctx.saved_tensors
            g = grad_out.detach().cpu().double()
            return (g * gb).to(ctx.devs[0]), (g * gr).to(ctx.devs[1]), None
except ImportError:  # torch is optional for the C ABI itself
    NetworkLogL = None


class NetworkBatch:
    """Candidate networks of one search move scored together: one CUDA graph
    holding a logL + gradient evaluation of every context, launched once per
    call (``netlk_batch_*``). The contexts stay owned by the caller and must
    outlive the batch."""

    def __init__(self, liks, per_context=False):
        """per_context: each context's own launch sequence in the graph
        instead of the persistent launches over all candidates."""
        self.liks = list(liks)
        L = N.lib()
        arr = (ctypes.c_void_p * len(self.liks))(*[lk._h for lk in self.liks])
        h = ctypes.c_void_p()
        N.check(L.netlk_batch_create_ex(arr, len(self.liks), 1 if per_context else 0, ctypes.byref(h)))
        self._h = h

    def info(self):
        """(persistent launches in use, kernels per call, forward / adjoint walk shape)."""
        pers, fs, bs = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        n = ctypes.c_int64()
        N.check(N.lib().netlk_batch_info(self._h, ctypes.byref(pers), ctypes.byref(n), ctypes.byref(fs),
                                         ctypes.byref(bs)))
        return {"persistent": bool(pers.value), "launches_per_call": n.value, "forward_shape": fs.value,
                "backward_shape": bs.value}

    def loglikelihood_gradient(self):
        """Returns (totals [n], list of d logL / d branch length, list of
        d logL / d reticulation probability)."""
        n = len(self.liks)
        tot = np.zeros(n)
        gb = [np.zeros(lk.n_edges) for lk in self.liks]
        gr = [np.zeros(max(1, lk.n_ret)) for lk in self.liks]
        pb = (ctypes.POINTER(ctypes.c_double) * n)(*[_ptr(g, ctypes.c_double) for g in gb])
        pr = (ctypes.POINTER(ctypes.c_double) * n)(*[_ptr(g, ctypes.c_double) for g in gr])
        N.check(N.lib().netlk_batch_loglikelihood_gradient(self._h, _ptr(tot, ctypes.c_double), pb, pr))
        return tot, gb, [g[:lk.n_ret] for g, lk in zip(gr, self.liks)]

    def close(self):
        if getattr(self, "_h", None):
            N.lib().netlk_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
