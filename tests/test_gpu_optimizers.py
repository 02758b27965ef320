"""The reference's optimizer loops driven through the C ABI, against the same
loops on the oracle (``tests/optimizer_loops.py`` restates them).

* Branch lengths: one Newton-Raphson pass over every edge with the
  reference's derivative formula (``netlk_edge_derivatives`` mode 1, each NR
  step after ``netlk_edge_loglikelihood`` sets the proposal) against the same
  pass with ``oracle/derivatives.py``'s sumtable derivatives and the oracle's
  log-likelihood. The final lengths agree within 1e-6 (FP64) / 1e-4 (FP32)
  relative or 1e-9 (FP64) / 1e-7 (FP32, the NR stopping tolerance) absolute, the final logL within 1e-9 (FP64) / 1e-6 (FP32)
  relative, and no step lowers the log-likelihood. With the true
  derivatives (mode 0) repeated passes converge: the gradient vanishes on the
  edges away from the length bounds.
* Reticulation probabilities: the Brent loop on ``netlk_set_reticulation_probs``
  + ``netlk_loglikelihood`` against the same loop on the oracle; the
  probabilities agree within 1e-5 and the logL within 1e-9 / 1e-6.
* Model parameters: Brent on each partition's Gamma shape and on the
  exchangeabilities through ``netlk_set_model`` + ``netlk_loglikelihood``
  (the model optimizer's callback) against the same searches on the oracle:
  parameters within 1e-4 (FP64) / 1e-2 (FP32) relative, logL within 1e-9 /
  1e-6.
"""
import numpy as np
import pytest

import optimizer_loops as opt
from conftest import GoldenPartition, golden_cases

pytestmark = pytest.mark.gpu

CASES = {c["name"]: c for c in golden_cases()}
NAMES = ["twoReticulations", "synthetic_12taxa_3ret_2parts"]


def _lik(name, variant, precision):
    from netrax_gb300.likelihood import NetworkLikelihood
    from netrax_gb300.network import parse_extended_newick
    case = CASES[name]
    net = parse_extended_newick(case["newick"])
    return NetworkLikelihood(net, [GoldenPartition(d) for d in case["partitions"]], variant=variant,
                             precision=precision)


def _oracle(name, variant):
    from oracle import improved, newick, pllmath
    case = CASES[name]
    parts = []
    for d in case["partitions"]:
        gp = GoldenPartition(d)
        parts.append(improved.Partition(gp.tip_states, gp.weights, gp.freqs, gp.exch,
                                        pllmath.gamma_rates_mean(gp.alpha, 4)))
    orc = improved.ImprovedOracle(newick.parse_newick(case["newick"]), parts, variant=variant)
    orc.loglikelihood()
    return orc


def _oracle_branch_pass(name, variant):
    from oracle import derivatives
    orc = _oracle(name, variant)

    def edge_logl(e, t):
        orc.brlen[e] = t
        return orc.loglikelihood()

    def edge_derivs(e):
        return derivatives.EdgeDerivativeOracle(orc).edge(e, mode="reference")

    return opt.optimize_branches(edge_logl, edge_derivs, list(orc.brlen))


def _close(a, b, rel, atol):
    a, b = np.asarray(a), np.asarray(b)
    return np.all(np.abs(a - b) <= np.maximum(atol, rel * np.abs(b)))


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_newton_raphson_branch_pass_matches_the_oracle(name, variant):
    want_len, want_logl, want_worse = _oracle_branch_pass(name, variant)
    assert not want_worse
    # lengths: relative, or absolute within the NR stopping tolerance (1e-7)
    # in FP32, whose derivatives near the 1e-6 clamp carry ~1e-4 relative noise
    for precision, rel_len, abs_len, rel_logl in (("fp64", 1e-6, 1e-9, 1e-9), ("fp32", 1e-4, opt.NR_TOLERANCE, 1e-6)):
        with _lik(name, variant, precision) as lik:
            start = lik.loglikelihood()
            lengths, logl, worse = opt.optimize_branches(
                lik.edge_loglikelihood, lambda e: lik.edge_derivatives(e, second=True, mode=1),
                lik.branch_lengths)
            assert not worse and logl >= start - 1e-9 * abs(start)
            assert logl == pytest.approx(want_logl, rel=rel_logl)
            assert _close(lengths, want_len, rel_len, abs_len), (precision, np.abs(np.array(lengths) - want_len).max())
            assert lik.loglikelihood() == pytest.approx(logl, rel=1e-12)


@pytest.mark.parametrize("name", NAMES)
def test_newton_raphson_with_true_derivatives_converges(name):
    """Repeated passes with the true derivatives (mode 0): the log-likelihood
    rises with every pass, and the adjoint gradient shrinks to under 1 % of
    its start on every edge away from the length bounds (coordinate ascent)."""
    with _lik(name, "AVERAGE", "fp64") as lik:
        start, g0, _ = lik.loglikelihood_gradient()
        lengths, logl = list(lik.branch_lengths), start
        for _ in range(20):
            lengths, new, worse = opt.optimize_branches(
                lik.edge_loglikelihood, lambda e: lik.edge_derivatives(e, second=True, mode=0), lengths)
            assert not worse and new >= logl - 1e-9 * abs(logl)
            if new - logl < 1e-8:
                break
            logl = new
        _, g, _ = lik.loglikelihood_gradient()
        interior = (np.array(lengths) > 1e-5) & (np.array(lengths) < 99.0)
        assert interior.any()
        assert np.abs(g[interior]).max() <= 1e-2 * np.abs(g0).max()


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("variant", ["AVERAGE", "BEST"])
def test_brent_reticulation_loop_matches_the_oracle(name, variant):
    orc = _oracle(name, variant)

    def orc_logl(probs):
        orc.set_ret_probs(probs)
        return orc.loglikelihood()

    want_p, want_logl = opt.optimize_reticulations(orc_logl, list(orc.ret_probs), tol=1e-8)
    for precision, rel_logl, tol_p in (("fp64", 1e-9, 1e-5), ("fp32", 1e-6, 1e-3)):
        with _lik(name, variant, precision) as lik:
            def logl_at(probs):
                lik.set_reticulation_probs(np.array(probs))
                return lik.loglikelihood()

            p, logl = opt.optimize_reticulations(logl_at, list(lik.ret_probs), tol=1e-8)
            assert logl == pytest.approx(want_logl, rel=rel_logl)
            assert np.abs(np.array(p) - np.array(want_p)).max() <= tol_p, (precision, p, want_p)


@pytest.mark.parametrize("name,exch", [("twoReticulations", True), ("synthetic_12taxa_3ret_2parts", False)])
def test_model_optimizer_callbacks_match_the_oracle(name, exch):
    """The model optimizer's searches (Gamma shape, exchangeabilities) on the
    oracle, every model they evaluate recorded: the library's logL at each of
    those models equals the oracle's (FP64 1e-9, FP32 1e-6), and the same
    searches on the library end at the oracle's optimum within the searches'
    own tolerance (Brent can take a different path when values differ in the
    last bits: logL 1e-6 relative, parameters 5 %)."""
    from oracle import pllmath
    orc = _oracle(name, "AVERAGE")
    start = [(p.freqs, p.exch, GoldenPartition(d).alpha) for p, d in zip(orc.parts, CASES[name]["partitions"])]
    seen = []

    def orc_logl(models):
        for part, (f, x, a) in zip(orc.parts, models):
            part.exch = np.asarray(x, float)
            part.rates = pllmath.gamma_rates_mean(a, part.R)
            part.lam, part.U, part.Uinv, part.Q = pllmath.eigensystem(part.exch, part.freqs)
        v = orc.loglikelihood()
        seen.append(([(f, x.copy(), a) for f, x, a in models], v))
        return v

    want_models, want_logl = opt.optimize_model(orc_logl, start, exchangeabilities=exch)
    for precision, rel_logl in (("fp64", 1e-9), ("fp32", 1e-6)):
        with _lik(name, "AVERAGE", precision) as lik:
            def logl_at(models):
                for p, (f, x, a) in enumerate(models):
                    lik.set_model(p, f, x, a)
                return lik.loglikelihood()

            for models, v in seen[::max(1, len(seen) // 40)]:
                assert logl_at(models) == pytest.approx(v, rel=rel_logl)
            start_logl = logl_at(start)
            models, logl = opt.optimize_model(logl_at, start, exchangeabilities=exch)
            assert logl >= start_logl
            assert logl == pytest.approx(want_logl, rel=1e-6)
            for (f, x, a), (wf, wx, wa) in zip(models, want_models):
                assert a == pytest.approx(wa, rel=5e-2)
                assert np.allclose(x, wx, rtol=5e-2)
