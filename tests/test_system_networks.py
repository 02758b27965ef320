"""The reference's regression networks (``tests/golden/system_networks.json``).

Nineteen networks that once broke the reference's likelihood code
(``test/src/SystemTest.cpp:158-290``; 4 taxa, up to 7 reticulations, chains of
reticulations below reticulations, a trifurcating root), each with a seeded
40-site alignment, scored by the oracle (``tests/golden/make_system_golden.py``
says which topology: the shared parse, or the library's for a trifurcating
root with a reticulation child).

* CPU: the library parses each network into the fixture's edges; its DAG
  equals the oracle's enumeration node by node with the same tree
  log-probabilities; the walk schedule, the level adjoint's message buffers and
  the checkpointing plan (2 and 3 segments) replay soundly; the oracle's
  improved and naive AVERAGE evaluations agree (the reference's own
  compareLikelihoodFunctions invariant, there within 10 log units).
* GPU: log-likelihood against the oracle, FP64 1e-9 and FP32 1e-6 relative,
  AVERAGE and BEST.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, GoldenPartition
from netrax_gb300.likelihood import NetworkLikelihood
from netrax_gb300.network import parse_extended_newick
from test_dag_abi import _check_walk
from test_dag_random import _covered, _replay_adjoint_messages, _replay_checkpoint_plan

with open(os.path.join(GOLDEN, "system_networks.json")) as _f:
    CASES = json.load(_f)["cases"]


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_system_network_dag_and_schedules(case):
    net = parse_extended_newick(case["newick"])
    assert list(net.edge_parent) == case["edge_parent"] and list(net.edge_child) == case["edge_child"]
    parts = [GoldenPartition(d) for d in case["partitions"]]
    lik = NetworkLikelihood(net, parts, host_only=True)
    node, _, _, cov = lik.dag_export()
    got = {}
    for i in range(len(node)):
        got.setdefault(int(node[i]), []).append(sorted(_covered(cov[i], net.n_reticulations)))
    want = {}
    for v, s in case["dag"]:
        want.setdefault(v, []).append(s)
    assert got == want
    _, _, lp = lik.root_export()
    assert np.allclose(lp, [t["logprob"] for t in case["AVERAGE"]["trees"]], rtol=1e-13, atol=1e-13)
    _check_walk(lik)
    _replay_adjoint_messages(lik)
    lik.close()
    for k in (2, 3):
        seg = NetworkLikelihood(net, parts, host_only=True, checkpoint_segments=k)
        _replay_checkpoint_plan(seg)
        seg.close()
    # AVERAGE only: under BEST the improved evaluation scores a displayed tree
    # with the summed probability of all configurations that display it, the
    # naive one each configuration on its own
    g = case["AVERAGE"]
    assert g["logl"] == pytest.approx(g["naive_logl"], rel=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_system_network_loglikelihood(case, precision):
    net = parse_extended_newick(case["newick"])
    parts = [GoldenPartition(d) for d in case["partitions"]]
    tol = 1e-9 if precision == "fp64" else 1e-6
    for variant in ("AVERAGE", "BEST"):
        with NetworkLikelihood(net, parts, variant=variant, precision=precision) as lik:
            total, _, trees = lik.loglikelihood(details=True)
        assert total == pytest.approx(case[variant]["logl"], rel=tol)
        for k, t in enumerate(case[variant]["trees"]):
            if t["partition_logl"] is not None:
                assert np.allclose(trees[k], t["partition_logl"], rtol=tol, atol=0)
