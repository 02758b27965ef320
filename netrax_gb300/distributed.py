"""Pattern-sharded evaluation across ranks (one GPU each).

Sites are independent until the per-(displayed tree, partition) sums, so each
rank holds a contiguous slice of every partition's patterns. One evaluation:

1. local per-(tree, partition) log-likelihood partials (``tree_partials``);
2. all-reduce SUM of that ``trees x partitions`` vector - the exchange the
   reference makes through ``parallel_reduce_cb``
   (``src/likelihood/ImprovedLoglikelihood.cpp:473-483``);
3. every rank mixes the global partials (AVERAGE / BEST) and runs its local
   adjoint sweep with the global tree weights (``mix_and_backward``);
4. all-reduce SUM of the branch-length gradient partials. The reticulation
   gradient depends only on the global weights, so it is already global.

The backend is a ``NetworkLikelihood`` on the rank's slice by default; any
object with ``tree_partials()`` and ``mix_and_backward(global)`` works.
"""
import copy

import numpy as np


def shard_partition(part, rank, world_size):
    """Contiguous pattern slice ``rank`` of ``world_size`` (same model)."""
    n = part.tip_states.shape[1]
    bounds = np.linspace(0, n, world_size + 1).round().astype(int)
    lo, hi = bounds[rank], bounds[rank + 1]
    if hi <= lo:
        raise ValueError("partition with %d patterns cannot be split over %d ranks" % (n, world_size))
    q = copy.copy(part)
    q.tip_states = np.ascontiguousarray(part.tip_states[:, lo:hi])
    q.weights = np.ascontiguousarray(part.weights[lo:hi])
    return q


class ShardedLikelihood:
    def __init__(self, network, partitions, rank, world_size, group=None, backend=None, **kw):
        self.rank, self.world_size, self.group = rank, world_size, group
        self.local_partitions = [shard_partition(p, rank, world_size) for p in partitions]
        if backend is None:
            from .likelihood import NetworkLikelihood
            backend = NetworkLikelihood(network, self.local_partitions, **kw)
        self.backend = backend

    def _allreduce(self, arr):
        import torch
        import torch.distributed as dist
        t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64))
        if self.world_size > 1:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
        return t.numpy()

    def loglikelihood_gradient(self):
        partials = self.backend.tree_partials()
        glob = self._allreduce(partials)
        total, d_brlen_local, d_ret, part_logl = self.backend.mix_and_backward(glob)
        d_brlen = self._allreduce(d_brlen_local)
        return total, d_brlen, d_ret, part_logl
