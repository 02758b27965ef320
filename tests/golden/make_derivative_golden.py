"""Generate ``derivative_cases.json``: analytic branch-length derivatives.

    python tests/golden/make_derivative_golden.py

Reads the networks, partitions and models of the committed likelihood
fixtures (``reference_cases.json``, ``synthetic_cases.json``,
``protein_cases.json``) and scores them with ``oracle/derivatives.py`` - the
restatement of the reference's per-edge sumtable derivatives
(``src/likelihood/LikelihoodDerivatives.cpp``) - under AVERAGE and BEST:

* ``grad_brlen`` / ``grad_retprob``: the exact gradient of the network
  log-likelihood (what ``netlk_loglikelihood_gradient`` returns);
* ``d1_true`` / ``d2_true``: per edge, first and second derivative of the
  network log-likelihood (``netlk_edge_derivatives`` mode 0);
* ``d1_reference`` / ``d2_reference``: per edge, the reference's own formula
  with its restriction to trees where the edge is active and BEST by
  ``tree_logl * tree_prob`` (mode 1).

Nothing here runs at test time on the GPU host; the tests compare against the
committed file, and a CPU test re-derives a few cases to pin it to the oracle.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import derivatives, improved, newick, pllmath  # noqa: E402

SOURCES = ("reference_cases.json", "synthetic_cases.json", "protein_cases.json")
SKIP = {"synthetic_200taxa_2ret_deep"}  # a scaling case; its gradient adds nothing


def oracle_for(case, variant):
    net = newick.parse_newick(case["newick"])
    parts = []
    for d in case["partitions"]:
        parts.append(improved.Partition(np.array(d["tip_states"], np.uint32), np.array(d["weights"]),
                                        d["freqs"], d["exch"], pllmath.gamma_rates_mean(d["alpha"], 4)))
    orc = improved.ImprovedOracle(net, parts, variant=variant)
    orc.loglikelihood()
    return orc


def score(case, variant):
    orc = oracle_for(case, variant)
    d = derivatives.EdgeDerivativeOracle(orc)
    g, gr = d.gradient()
    true = [d.edge(e, "true") for e in range(orc.net.n_edges)]
    ref = [d.edge(e, "reference") for e in range(orc.net.n_edges)]
    return {"grad_brlen": g.tolist(), "grad_retprob": gr.tolist(),
            "d1_true": [x[0] for x in true], "d2_true": [x[1] for x in true],
            "d1_reference": [x[0] for x in ref], "d2_reference": [x[1] for x in ref]}


def main():
    out = []
    for src in SOURCES:
        with open(os.path.join(HERE, src)) as f:
            cases = json.load(f)["cases"]
        for case in cases:
            if case["name"] in SKIP:
                continue
            t = time.time()
            rec = {"name": case["name"], "source": src}
            for variant in ("AVERAGE", "BEST"):
                rec[variant] = score(case, variant)
            out.append(rec)
            print(case["name"], "%.1fs" % (time.time() - t), flush=True)
    with open(os.path.join(HERE, "derivative_cases.json"), "w") as f:
        json.dump({"cases": out}, f)


if __name__ == "__main__":
    main()
