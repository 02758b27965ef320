"""The allocation-free mixing entry point against the context path.

``netlk_mix_site_loglikelihoods_noalloc`` serves callers that cannot allocate
device memory (memory owned by another allocator or a fixed budget, loops
that must not pay for the device synchronisation of cudaMalloc). It works in a fixed device array inside the library, so this test
only hands it input and output buffers. The per-site log-likelihoods of every
displayed tree come from the oracle; the answer must equal what
``netlk_loglikelihood`` (the existing entry point, FP64 context) returns for
the same network and alignment, within the FP64 parity tolerance, on two
calls in a row (the second call reuses the array the first one filled).
This file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

from conftest import GoldenPartition, golden_cases

pytestmark = pytest.mark.gpu

FP64_REL = 1e-9


def _site_logl_from_oracle(case, variant):
    from oracle import build as obuild
    from oracle import improved, newick, pllmath
    net = newick.parse_newick(case["newick"])
    parts = []
    for d in case["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4)))
    orc = improved.ImprovedOracle(net, parts, variant=variant)
    orc.loglikelihood()
    rows, logprob = [], []
    for t in orc.root_trees():
        dn, di = t.dtroot
        m = orc.pernode[dn][di]
        row = []
        for p, part in enumerate(parts):
            persite = np.empty(part.n)
            obuild.root_logl(m.clv[p], m.scaler[p], part.freqs, part.rate_weights, part.weights, persite)
            row.append(persite * part.weights)
        rows.append(np.concatenate(row))
        logprob.append(t.logprob)
    begin = np.concatenate([[0], np.cumsum([part.n for part in parts])]).astype(np.int64)
    return np.array(rows), begin, np.array(logprob)


@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_noalloc_mixing_matches_context_path(variant):
    torch = pytest.importorskip("torch")
    from netrax_gb300 import _native
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    case = [c for c in golden_cases() if c["name"] == "synthetic_16taxa_4ret_3parts"][0]
    net = parse_extended_newick(case["newick"])
    parts = [GoldenPartition(d) for d in case["partitions"]]
    with NetworkLikelihood(net, parts, variant=variant, precision="fp64") as lik:
        want_total, want_parts = lik.loglikelihood(details=True)[:2]

    site, begin, logprob = _site_logl_from_oracle(case, variant)
    dev = torch.device("cuda", 0)
    d_site = torch.from_numpy(np.ascontiguousarray(site)).to(dev)
    d_begin = torch.from_numpy(begin).to(dev)
    d_lp = torch.from_numpy(logprob).to(dev)
    L = _native.lib()
    code = _native.NETLK_AVERAGE if variant == "AVERAGE" else _native.NETLK_BEST
    results = []
    for _ in range(2):
        d_out = torch.full((1 + len(parts),), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = L.netlk_mix_site_loglikelihoods_noalloc(
            ctypes.c_void_p(d_site.data_ptr()), site.shape[0], site.shape[1],
            ctypes.c_void_p(d_begin.data_ptr()), len(parts), ctypes.c_void_p(d_lp.data_ptr()), code,
            float(np.log(1e-6)), ctypes.c_void_p(d_out.data_ptr()), None)
        assert st == 0, L.netlk_last_error(None)
        torch.cuda.synchronize()
        results.append(d_out.cpu().numpy())
    for out in results:
        assert out[0] == pytest.approx(want_total, rel=FP64_REL)
        assert np.allclose(out[1:], want_parts, rtol=FP64_REL, atol=0)
    assert np.array_equal(results[0], results[1])


def test_noalloc_rejects_sizes_beyond_its_array():
    pytest.importorskip("torch")
    import torch
    from netrax_gb300 import _native
    L = _native.lib()
    dev = torch.device("cuda", 0)
    d = torch.zeros(8, dtype=torch.float64, device=dev)
    b = torch.zeros(2, dtype=torch.int64, device=dev)
    st = L.netlk_mix_site_loglikelihoods_noalloc(
        ctypes.c_void_p(d.data_ptr()), 65537, 1, ctypes.c_void_p(b.data_ptr()), 1,
        ctypes.c_void_p(d.data_ptr()), 0, -13.8, ctypes.c_void_p(d.data_ptr()), None)
    assert st == 1
    assert b"exceeds the fixed working array" in L.netlk_last_error(None)
