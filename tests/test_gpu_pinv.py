"""GPU: invariant sites (+I) through the C ABI against the oracle.

With ``prop_invar`` p > 0 a site's likelihood is (1 - p) times the rate
mixture (category rates divided by 1 - p) plus p times the frequency of the
one state every tip admits, if any. On golden DNA and protein cases (the
200-taxon case rescales in FP64; protein FP32 runs on the tensor cores), with
a different p per partition: logL (FP64 1e-9, FP32 1e-6 relative), the
adjoint gradient against ``oracle/sweep.c`` (FP64 1e-8, FP32 1e-5 of the
largest entry), the analytic edge derivatives (both modes) against
``oracle/derivatives.py`` (FP64 1e-8), and ``netlk_set_prop_invar`` on a
running context against a context created with the same p.
"""
import numpy as np
import pytest

from conftest import GoldenPartition, golden_cases

pytestmark = pytest.mark.gpu

CASES = {c["name"]: c for c in golden_cases()}
NAMES = ["twoReticulations", "synthetic_12taxa_3ret_2parts", "synthetic_200taxa_2ret_deep", "protein_8taxa_2ret",
         "protein_10taxa_3ret_2parts"]
PINV = [0.3, 0.15]


class _P(GoldenPartition):
    def __init__(self, d, pinv):
        super().__init__(d)
        self.prop_invar = pinv


def _parts(name):
    return [_P(d, PINV[k % 2]) for k, d in enumerate(CASES[name]["partitions"])]


def _lik(name, variant, precision, parts=None, **kw):
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    net = parse_extended_newick(CASES[name]["newick"])
    return NetworkLikelihood(net, parts if parts is not None else _parts(name), variant=variant,
                             precision=precision, **kw)


def _oracle(name, variant):
    from oracle import improved, newick, pllmath
    parts = [improved.Partition(p.tip_states, p.weights, p.freqs, p.exch, pllmath.gamma_rates_mean(p.alpha, 4),
                                pinv=p.prop_invar) for p in _parts(name)]
    orc = improved.ImprovedOracle(newick.parse_newick(CASES[name]["newick"]), parts, variant=variant)
    orc.loglikelihood()
    return orc


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_pinv_logl_and_gradient_match_the_oracle(name, variant):
    from oracle import sweep
    orc = _oracle(name, variant)
    want = orc.evaluate()[0]
    _, _, _, g, gr = sweep.SweepOracle(orc).evaluate()
    for precision, tol, gtol in (("fp64", 1e-9, 1e-8), ("fp32", 1e-6, 1e-5)):
        with _lik(name, variant, precision) as lik:
            got = lik.loglikelihood()
            assert got == pytest.approx(want, rel=tol)
            tot, gb, gret = lik.loglikelihood_gradient()
            assert tot == got
            assert np.abs(gb - g).max() <= gtol * max(1.0, float(np.abs(g).max()))
            if len(gr):
                assert np.abs(gret - gr).max() <= gtol * max(1.0, float(np.abs(gr).max()))


@pytest.mark.parametrize("name", NAMES[:3] + NAMES[3:4])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("sumtables", [True, False])
def test_pinv_edge_derivatives_match_the_sumtable_oracle(name, mode, sumtables):
    """Both derivative paths (edge sumtables; the tangent sweep) with +I."""
    from oracle import derivatives
    orc = _oracle(name, "AVERAGE")
    d = derivatives.EdgeDerivativeOracle(orc)
    key = "true" if mode == 0 else "reference"
    with _lik(name, "AVERAGE", "fp64", sumtables=sumtables) as lik:
        for e in range(0, lik.n_edges, max(1, lik.n_edges // 12)):
            w1, w2 = d.edge(e, mode=key)
            d1, d2 = lik.edge_derivatives(e, second=True, mode=mode)
            assert d1 == pytest.approx(w1, rel=1e-8, abs=1e-8)
            assert d2 == pytest.approx(w2, rel=1e-8, abs=1e-7)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_set_prop_invar_matches_a_new_context(precision):
    name = "synthetic_12taxa_3ret_2parts"
    plain = [GoldenPartition(d) for d in CASES[name]["partitions"]]
    with _lik(name, "AVERAGE", precision, parts=plain) as lik, _lik(name, "AVERAGE", precision) as ref:
        l0 = lik.loglikelihood()
        for k in range(len(plain)):
            lik.set_prop_invar(k, PINV[k % 2])
        t1, g1, r1 = lik.loglikelihood_gradient()
        t2, g2, r2 = ref.loglikelihood_gradient()
        assert t1 == t2 and t1 != l0
        assert np.array_equal(g1, g2) and np.array_equal(r1, r2)
        for k in range(len(plain)):
            lik.set_prop_invar(k, 0.0)
        assert lik.loglikelihood() == l0
