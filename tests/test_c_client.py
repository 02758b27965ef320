"""CPU: a plain C99 program against include/netlk.h and the built library.

``tests/abi_client.c`` is what a reference-side binding looks like without
Python: it fills the descriptors by hand in the reference's numbering, runs
the alignment front end, builds a host-only context, reads an edge's
sumtable schedule and exercises the error surface. It is compiled with ``-std=c99 -Wall -Wextra -Werror -pedantic``
(the header is C, not only C++) and its DAG statistics must equal those of the
same network and alignment built through the Python harness.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

NEWICK = "((A:0.1,(B:0.2)#H1:0.05::0.6):0.1,(C:0.3,#H1:0.1::0.4):0.2);"
ROWS = ["ACGTACGA", "ACGTTCGA", "AYGTACNA"]


def test_c_client_builds_and_matches_python(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    from netrax_gb300 import _native
    lib = _native.lib()  # builds the library if needed
    libdir = os.path.dirname(lib._name)
    exe = str(tmp_path / "abi_client")
    subprocess.check_call([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                           os.path.join(ROOT, "tests", "abi_client.c"), "-I", os.path.join(ROOT, "include"),
                           lib._name, "-Wl,-rpath," + libdir, "-lm", "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    got = dict(line.split("=", 1) for line in out.stdout.strip().splitlines())

    from conftest import GoldenPartition
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    from oracle import pllmath
    net = parse_extended_newick(NEWICK)
    codes = np.array([pllmath.encode_dna(r) for r in ROWS])
    pat, w = pllmath.compress_patterns(codes)
    part = GoldenPartition({"tip_states": pat.tolist(), "weights": w.tolist(), "freqs": [0.2, 0.3, 0.3, 0.2],
                            "exch": [1.0, 2.5, 0.8, 1.2, 3.0, 1.0], "alpha": 0.8})
    with NetworkLikelihood(net, [part], host_only=True) as lik:
        st = lik.stats
        ops, _, n_tab, gref, _ = lik.sumtable_export(2)
    assert int(got["n_site_patterns"]) == len(w)
    for k in ("n_variants", "n_root_variants", "n_levels", "n_backward_ops", "site_clv_updates"):
        assert int(got[k]) == st[k], k
    assert (int(got["sumtable_ops"]), int(got["sumtable_tables"]), int(got["sumtable_groups"])) == \
        (len(ops), n_tab, len(gref))
    assert got["evaluate_status"] == "no CUDA device"
    assert "branch length" in got["nan_length_error"]
