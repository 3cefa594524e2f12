"""The batched compressible-EOS consistency iteration
(``pyrometheus_gb300.eos_consistency.CompressibleEOS``) on the CPU: run on
the oracle's pieces it reproduces, flamelet by flamelet, the single-flamelet
restatement of the reference's outer loop
(``oracle/eos_consistency_oracle.py``, after
``pyrometheus/flamelets/thermodynamic_consistency.py:310-706``) — params,
iteration counts, residual and ``(<h>, <T>)`` histories, states — with both
update methods, although the batch iterates only the flamelets still
running."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from flamelet_solver_cases import (EOS_FLAMELETS, OracleEquations,  # noqa
                                   eos_case, eos_config, flamelet_batch,
                                   mechanism, split)
from oracle.eos_consistency_oracle import CompressibleEOSOracle  # noqa: E402
from pyrometheus_gb300.eos_consistency import CompressibleEOS  # noqa: E402
from pyrometheus_gb300.flamelet_solver import FlameletSolver  # noqa: E402


@pytest.fixture(scope="module")
def case():
    np.seterr(all="ignore")
    sol = mechanism()
    b = flamelet_batch(sol, EOS_FLAMELETS)
    return sol, b, eos_case(sol, b)


def _eos(sol, b, config):
    eq = OracleEquations(sol, b["lengths"], b["dx"], b["y_ox"], b["y_fu"])
    return CompressibleEOS(config, FlameletSolver.from_equations(eq))


@pytest.mark.parametrize("method, tol", [("gauss_newton", 1e-12),
                                         ("picard", 1e-6)])
def test_outer_loop_matches_the_single_flamelet_oracle(case, method, tol):
    sol, b, (pdf, true, start, rho, e) = case
    cfg = eos_config(method, maxiter=3, tol=tol)
    eos = _eos(sol, b, cfg)
    st, temp, params, its, deltas, res, hist, flag = eos.ensure_consistency(
        rho, e, start, pdf, b["chi"], b["visc"], b["T"], b["phi"])
    assert flag is False
    n = b["lengths"]
    phis = split(torch.cat([st.enthalpy[None], st.mass_fractions]).numpy(),
                 n)
    temps = split(temp.numpy(), n)
    for s, (phi0, chi, visc, tg, w) in enumerate(zip(
            split(b["phi"], n), split(b["chi"], n), split(b["visc"], n),
            split(b["T"], n), split(pdf, n))):
        orc = CompressibleEOSOracle(sol, b["dx"][s], b["y_ox"], b["y_fu"],
                                    cfg)
        phi, t, p, it, d, r, h = orc.ensure_consistency(
            rho[s], e[s], start[:, s], w, chi, visc, tg, phi0)
        assert its[s] == it
        np.testing.assert_array_equal(params[:, s], p)
        assert deltas[s] == d
        np.testing.assert_array_equal(res[:, s], r)
        np.testing.assert_array_equal(hist[:, :, s], h)
        np.testing.assert_array_equal(phis[s], phi)
        np.testing.assert_array_equal(temps[s], t)
    if method == "gauss_newton":
        # the pressure converges to the one the targets came from
        assert np.allclose(params[0], true[0], rtol=1e-8, atol=0)
        assert (its == 2).all()
    else:
        # the Picard fixed point p = rho_sim <R T> differs from it by the
        # PDF average's Jensen gap; both flamelets stop at their second
        # update
        assert (its == 1).all() and (deltas < tol).all()


def test_config_and_errors(case):
    sol, b, (pdf, true, start, rho, e) = case
    eos = _eos(sol, b, eos_config("gauss_newton"))
    eos.update_config_option("eos/update_method", "newton")
    eos.update_config_option("extra/level/value", 3)
    assert eos.config["extra"]["level"]["value"] == 3
    with pytest.raises(ValueError, match="not implemented"):
        eos.ensure_consistency(rho, e, start, pdf, b["chi"], b["visc"],
                               b["T"], b["phi"])
    with pytest.raises(TypeError, match="not a dict"):
        eos.update_config_option("eos/update_size/x", 1.0)
    eos.update_config_option("eos/update_method", "gauss_newton")
    with pytest.raises(ValueError, match="params"):
        eos.ensure_consistency(rho, e, start[:2], pdf, b["chi"], b["visc"],
                               b["T"], b["phi"])


def test_flamelets_leave_the_batch_as_they_converge(case):
    """One flamelet starts at the parameters its targets came from and stops
    after its first update (|v| = 0); the other goes on alone as a packed
    sub-batch.  Both still match the single-flamelet oracle bit for bit."""
    sol, b, (pdf, true, start, rho, e) = case
    start = start.copy()
    start[:, 0] = true[:, 0]
    cfg = eos_config("gauss_newton", maxiter=3, tol=1e-6)
    eos = _eos(sol, b, cfg)
    st, temp, params, its, deltas, res, hist, _ = eos.ensure_consistency(
        rho, e, start, pdf, b["chi"], b["visc"], b["T"], b["phi"])
    assert its.tolist() == [0, 2] and deltas[0] == 0.0
    assert np.isnan(res[1:, 0]).all() and not np.isnan(res[:, 1]).any()
    n = b["lengths"]
    phis = split(torch.cat([st.enthalpy[None], st.mass_fractions]).numpy(),
                 n)
    for s, (phi0, chi, visc, tg, w) in enumerate(zip(
            split(b["phi"], n), split(b["chi"], n), split(b["visc"], n),
            split(b["T"], n), split(pdf, n))):
        orc = CompressibleEOSOracle(sol, b["dx"][s], b["y_ox"], b["y_fu"],
                                    cfg)
        phi, t, p, it, d, r, h = orc.ensure_consistency(
            rho[s], e[s], start[:, s], w, chi, visc, tg, phi0)
        assert its[s] == it
        np.testing.assert_array_equal(params[:, s], p)
        np.testing.assert_array_equal(res[:, s], r)
        np.testing.assert_array_equal(phis[s], phi)
        np.testing.assert_array_equal(split(temp.numpy(), n)[s], t)
