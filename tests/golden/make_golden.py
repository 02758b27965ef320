"""Generate the golden fixtures of the parity tests.

Run in a checkout that has the NetRAX reference tree next to it:

    python tests/golden/make_golden.py [--reference /path/to/NetRAX]

Cases:
* ``reference_cases.json`` - the reference's own likelihood test cases
  (network + fake alignment pairs of ``test/src/LikelihoodTest.cpp:281-360``,
  read from ``test/sample_networks``), scored by the CPU oracle under a fixed
  GTR+G4 model with AVERAGE and BEST: network logL, per-partition logL,
  per-displayed-tree logL, the naive 2^r evaluation, the displayed-tree DAG
  (covered configuration sets per node), central-difference gradients.
* ``protein_cases.json`` - 20-state (LG-like) cases on small seeded networks,
  with gaps and an ambiguity code.
* ``synthetic_cases.json`` - seeded synthetic networks (several partitions,
  and one deep 200-taxon case whose FP64 CLVs trigger the 2^256 scaling)
  with the same outputs plus per-variant scale-counter checksums.

The oracle is the CPU restatement in ``oracle/``; nothing here is used at run
time by the product.
"""
import argparse
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import improved, naive, newick, pllmath  # noqa: E402

MODEL = {"freqs": [0.2, 0.3, 0.3, 0.2], "exch": [1.0, 2.5, 0.8, 1.2, 3.0, 1.0], "alpha": 0.8}

# test/src/LikelihoodTest.cpp:281-360
REFERENCE_CASES = [
    ("tinyNetwork", "tiny.nw", "tiny_fake_alignment.txt"),
    ("smallNetwork", "small.nw", "small_fake_alignment.txt"),
    ("smallTree", "tree.nw", "small_fake_alignment.txt"),
    ("clvAveraging", "clv_averaging.nw", "5_taxa_fake_alignment.txt"),
    ("twoReticulations", "two_reticulations.nw", "5_taxa_fake_alignment.txt"),
    ("threeReticulations", "three_reticulations.nw", "7_taxa_fake_alignment.txt"),
    ("interleavedReticulations", "interleaved_reticulations.nw", "5_taxa_fake_alignment.txt"),
    ("reticulationInReticulation", "reticulation_in_reticulation.nw", "small_fake_alignment.txt"),
    ("celineNetwork", "celine.nw", "celine_fake_alignment.txt"),
    ("celineNetworkSmaller", "celine_smaller_1.nw", "celine_fake_alignment_smaller.txt"),
    ("celineNetworkNonzeroBranches", "celine_nonzero_branches.nw", "celine_fake_alignment.txt"),
]


def covered_lists(orc):
    out = []
    for v, sets in sorted(orc.dag_summary().items()):
        for s in sets:
            out.append([v, sorted(s)])
    return out


def fd_gradient(orc, h=1e-5):
    """Central differences; one-sided where the 1e-6 length clamp binds."""
    g = []
    base = list(orc.brlen)
    for e in range(orc.net.n_edges):
        lo = max(base[e] - h, 1e-6)
        orc.brlen = list(base)
        orc.brlen[e] = base[e] + h
        up = orc.loglikelihood()
        orc.brlen[e] = lo
        dn = orc.loglikelihood()
        g.append((up - dn) / (base[e] + h - lo))
    orc.brlen = base
    gr = []
    probs = list(orc.ret_probs)
    for k in range(orc.r):
        p = list(probs)
        p[k] = probs[k] + h
        orc.set_ret_probs(p)
        up = orc.loglikelihood()
        p[k] = probs[k] - h
        orc.set_ret_probs(p)
        dn = orc.loglikelihood()
        gr.append((up - dn) / (2 * h))
    orc.set_ret_probs(probs)
    return g, gr


def score(net, parts_data, variant, with_grad=True, with_naive=True, scalers=False):
    parts = []
    for pd in parts_data:
        rates = pllmath.gamma_rates_mean(pd["alpha"], 4)
        parts.append(improved.Partition(np.array(pd["tip_states"], np.uint32), np.array(pd["weights"]),
                                        pd["freqs"], pd["exch"], rates))
    orc = improved.ImprovedOracle(net, parts, variant=variant)
    total = orc.loglikelihood()
    _, part_logl = orc.evaluate()
    trees = []
    for t in orc.root_trees():
        trees.append({"logprob": t.logprob,
                      "partition_logl": t.partition_logl if t.logl_valid else None,
                      "dtroot_node": t.dtroot[0] if t.dtroot else None,
                      "dtroot_index": t.dtroot[1] if t.dtroot else None})
    res = {"logl": total, "partition_logl": part_logl, "trees": trees,
           "site_clv_updates": orc.update_count}
    if scalers:
        sums, maxs = [], []
        for v in range(net.n_tips, net.n_nodes):
            for t in orc.pernode[v]:
                sums.append(int(sum(int(s.sum()) for s in t.scaler)))
                maxs.append(int(max(int(s.max()) for s in t.scaler)))
        res["scaler_sums"] = sums
        res["scaler_max"] = maxs
    if with_naive:
        res["naive_logl"] = naive.naive_loglikelihood(orc)[0]
    if with_grad:
        g, gr = fd_gradient(orc)
        res["fd_grad_brlen"] = g
        res["fd_grad_retprob"] = gr
    return res, orc


def reference_cases(ref):
    base = os.path.join(ref, "test", "sample_networks")
    out = []
    for name, nw, aln in REFERENCE_CASES:
        text = open(os.path.join(base, nw)).read().strip().splitlines()[0]
        net = newick.parse_newick(text)
        names, seqs = pllmath.read_fasta(open(os.path.join(base, aln)).read())
        rows = []
        for tip in range(net.n_tips):
            rows.append(pllmath.encode_dna(seqs[names.index(net.labels[tip])]))
        pat, w = pllmath.compress_patterns(np.array(rows))
        pd = dict(MODEL, tip_states=pat.tolist(), weights=w.tolist())
        case = {"name": name, "newick": text, "network_file": nw, "alignment_file": aln,
                "labels": net.labels[:net.n_tips], "partitions": [pd]}
        grad = name in ("tinyNetwork", "smallNetwork", "twoReticulations", "celineNetworkNonzeroBranches",
                        "threeReticulations")
        for variant in ("AVERAGE", "BEST"):
            res, orc = score(net, [pd], variant, with_grad=grad)
            case[variant] = res
        case["dag"] = covered_lists(orc)
        out.append(case)
        print(name, case["AVERAGE"]["logl"], case["BEST"]["logl"], flush=True)
    return out


def synthetic_cases():
    from netrax_gb300 import synth
    specs = [
        ("synthetic_12taxa_3ret_2parts", 12, 3, [300, 500], 11, 0.1),
        ("synthetic_16taxa_4ret_3parts", 16, 4, [200, 333, 150], 12, 0.1),
        ("synthetic_200taxa_2ret_deep", 200, 2, [120], 13, 1.0),
    ]
    out = []
    for name, nt, nr, sites, seed, mean_len in specs:
        rng = np.random.default_rng(seed)
        text = synth.random_network_newick(rng, nt, nr, mean_brlen=mean_len)
        from netrax_gb300.network import parse_extended_newick
        pnet = parse_extended_newick(text)
        parts = []
        for ns in sites:
            freqs = rng.dirichlet(np.ones(4))
            freqs = np.maximum(freqs, 1e-3)
            freqs /= freqs.sum()
            exch = rng.dirichlet(np.ones(6)) * 6
            codes = synth.simulate_dna(rng, pnet, ns, freqs, exch, 0.8)
            pat, w = pllmath.compress_patterns(codes)  # columns in lexicographic order of their codes
            parts.append({"freqs": freqs.tolist(), "exch": exch.tolist(), "alpha": 0.8,
                          "tip_states": pat.tolist(), "weights": w.tolist()})
        net = newick.parse_newick(text)
        case = {"name": name, "newick": text, "partitions": parts}
        deep = nt > 100
        for variant in ("AVERAGE", "BEST"):
            res, orc = score(net, parts, variant, with_grad=not deep, with_naive=not deep and nr <= 3,
                             scalers=True)
            case[variant] = res
        case["dag"] = covered_lists(orc)
        out.append(case)
        print(name, case["AVERAGE"]["logl"], case["BEST"]["logl"],
              "max scaler", max(case["AVERAGE"]["scaler_max"]), flush=True)
    return out


def protein_cases():
    """20-state cases: an LG-like model on small seeded networks."""
    from netrax_gb300 import synth
    from netrax_gb300.network import parse_extended_newick
    specs = [("protein_8taxa_2ret", 8, 2, [150], 21), ("protein_10taxa_3ret_2parts", 10, 3, [120, 90], 22)]
    out = []
    for name, nt, nr, sites, seed in specs:
        rng = np.random.default_rng(seed)
        text = synth.random_network_newick(rng, nt, nr)
        pnet = parse_extended_newick(text)
        parts = []
        for ns in sites:
            freqs = np.maximum(rng.dirichlet(np.ones(20)), 1e-3)
            freqs /= freqs.sum()
            exch = np.maximum(rng.gamma(1.0, 1.0, size=190), 1e-3)
            codes = synth.simulate(rng, pnet, ns, freqs, exch, 0.8)
            if name.endswith("2parts"):
                codes[0, :5] = (1 << 20) - 1  # gaps: every state
                codes[1, 3] = (1 << 2) | (1 << 7)  # an ambiguity
            pat, w = pllmath.compress_patterns(codes)  # columns in lexicographic order of their codes
            parts.append({"freqs": freqs.tolist(), "exch": exch.tolist(), "alpha": 0.8,
                          "tip_states": pat.tolist(), "weights": w.tolist(), "states": 20})
        net = newick.parse_newick(text)
        case = {"name": name, "newick": text, "partitions": parts, "states": 20}
        for variant in ("AVERAGE", "BEST"):
            res, orc = score(net, parts, variant, with_grad=True, with_naive=nr <= 3, scalers=True)
            case[variant] = res
        case["dag"] = covered_lists(orc)
        out.append(case)
        print(name, case["AVERAGE"]["logl"], case["BEST"]["logl"], flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True,
                    help="path of the NetRAX source tree (read-only input)")
    a = ap.parse_args()
    with open(os.path.join(HERE, "reference_cases.json"), "w") as f:
        json.dump({"model": MODEL, "cases": reference_cases(a.reference)}, f)
    with open(os.path.join(HERE, "synthetic_cases.json"), "w") as f:
        json.dump({"cases": synthetic_cases()}, f)
    with open(os.path.join(HERE, "protein_cases.json"), "w") as f:
        json.dump({"cases": protein_cases()}, f)


if __name__ == "__main__":
    main()
