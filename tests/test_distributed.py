"""Two-rank pattern sharding on CPU (gloo): sharded == whole.

The ranks run ``netrax_gb300.distributed.ShardedLikelihood`` - slice the
patterns, all-reduce the (tree, partition) partials, mix, run the local
adjoint, all-reduce the gradient - with a CPU backend built on the oracle (no
GPU here). The whole-data oracle is the reference answer.
"""
import math
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, GoldenPartition, golden_cases

torch = pytest.importorskip("torch")


class OracleBackend:
    """tree_partials / mix_and_backward on a pattern slice, computed by the oracle.

    The local adjoint is replaced by central differences of the local per-tree
    log-likelihoods with the global weights held fixed - the same quantity the
    GPU adjoint computes."""

    def __init__(self, newick, parts, h=1e-6):
        from oracle import improved, newick as onewick, pllmath
        net = onewick.parse_newick(newick)
        ops = [improved.Partition(p.tip_states, p.weights, p.freqs, p.exch,
                                  pllmath.gamma_rates_mean(p.alpha, 4)) for p in parts]
        self.orc = improved.ImprovedOracle(net, ops, variant="AVERAGE")
        self.h = h

    def _local(self):
        self.orc.forward()
        return np.array([t.partition_logl for t in self.orc.root_trees()])

    def tree_partials(self):
        return self._local()

    def mix_and_backward(self, glob):
        from oracle import configsets as cs
        trees = self.orc.root_trees()
        lp = np.array([t.logprob for t in trees])
        val = lp[:, None] + glob
        m = val.max(axis=0)
        part_logl = m + np.log(np.exp(val - m).sum(axis=0))
        w = np.exp(val - part_logl)
        total = float(part_logl.sum())
        base = list(self.orc.brlen)
        g = np.zeros(len(base))
        for e in range(len(base)):
            self.orc.brlen = list(base)
            self.orc.brlen[e] = base[e] + self.h
            up = self._local()
            self.orc.brlen[e] = base[e] - self.h
            dn = self._local()
            g[e] = float((w * (up - dn)).sum() / (2 * self.h))
        self.orc.brlen = base
        self._local()
        probs = list(self.orc.ret_probs)
        gr = np.zeros(self.orc.r)
        for k in range(self.orc.r):
            dl = []
            for sgn in (1, -1):
                p = list(probs)
                p[k] = probs[k] + sgn * self.h
                self.orc.set_ret_probs(p)
                dl.append(np.array([cs.set_logprob(t.configs, self.orc.first_lp, self.orc.second_lp)
                                    for t in trees]))
            self.orc.set_ret_probs(probs)
            gr[k] = float((w * ((dl[0] - dl[1]) / (2 * self.h))[:, None]).sum())
        return total, g, gr, part_logl


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, case, out):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    from netrax_gb300.distributed import ShardedLikelihood, shard_partition
    from netrax_gb300.network import parse_extended_newick
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    parts = [GoldenPartition(d) for d in case["partitions"]]
    local = [shard_partition(p, rank, world) for p in parts]
    sh = ShardedLikelihood(parse_extended_newick(case["newick"]), parts, rank, world,
                           backend=OracleBackend(case["newick"], local))
    total, g, gr, pl = sh.loglikelihood_gradient()
    out[rank] = (total, g.tolist(), list(gr), list(pl))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("name", ["twoReticulations", "synthetic_12taxa_3ret_2parts"])
def test_two_rank_sharding_matches_whole(name):
    case = [c for c in golden_cases() if c["name"] == name][0]
    ctx = torch.multiprocessing.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, case, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    whole = OracleBackend(case["newick"], [GoldenPartition(d) for d in case["partitions"]])
    wt, wg, wgr, wpl = whole.mix_and_backward(whole.tree_partials())
    assert wt == pytest.approx(case["AVERAGE"]["logl"], rel=1e-12)
    for r in range(2):
        t, g, gr, pl = out[r]
        assert t == pytest.approx(wt, rel=1e-12)
        assert np.allclose(g, wg, rtol=1e-6, atol=1e-6)
        assert np.allclose(gr, wgr, rtol=1e-6, atol=1e-6)
        assert np.allclose(pl, wpl, rtol=1e-12)
