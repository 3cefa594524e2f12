"""The batched compressible-EOS consistency iteration on the device pieces
(flamelet solver, adjoint gradients with one shared factorisation, R T on
the GPU) against the single-flamelet oracle of the reference's outer loop
(central-difference Jacobians): the same iteration counts, parameters to
1e-8 of the pressure and 1e-9 of the boundary enthalpies, the first two
residuals to 1e-6 relative (the last one is at rounding level), and the
final temperatures to 1e-3 K.  The tolerances leave a margin of two orders
over the change seen on the oracle when its difference steps go from 1e-6
to 3e-7."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from flamelet_solver_cases import (EOS_FLAMELETS, eos_case,  # noqa: E402
                                   eos_config, flamelet_batch, mechanism,
                                   split)


@pytest.mark.parametrize("method, tol, last", [("gauss_newton", 1e-12, 2),
                                               ("picard", 1e-6, 1)])
def test_device_outer_loop_matches_the_oracle(method, tol, last):
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from oracle.eos_consistency_oracle import CompressibleEOSOracle
    from pyrometheus_gb300 import get_thermochem_class
    from pyrometheus_gb300.eos_consistency import CompressibleEOS
    from pyrometheus_gb300.flamelet_solver import FlameletSolver
    np.seterr(all="ignore")
    sol = mechanism()
    b = flamelet_batch(sol, EOS_FLAMELETS)
    pdf, true, start, rho, e = eos_case(sol, b)
    cfg = eos_config(method, maxiter=3, tol=tol)
    th = get_thermochem_class(sol)()
    fs = FlameletSolver(th, b["lengths"], b["dx"], (b["y_ox"], b["y_fu"]))
    eos = CompressibleEOS(cfg, fs)
    st, temp, params, its, deltas, res, hist, _ = eos.ensure_consistency(
        rho, e, start, pdf, b["chi"], b["visc"], b["T"], b["phi"])
    n = b["lengths"]
    temps = split(temp.cpu().numpy(), n)
    for s, (phi0, chi, visc, tg, w) in enumerate(zip(
            split(b["phi"], n), split(b["chi"], n), split(b["visc"], n),
            split(b["T"], n), split(pdf, n))):
        orc = CompressibleEOSOracle(sol, b["dx"][s], b["y_ox"], b["y_fu"],
                                    cfg)
        phi, t, p, it, d, r, h = orc.ensure_consistency(
            rho[s], e[s], start[:, s], w, chi, visc, tg, phi0)
        assert its[s] == it == last, s
        assert abs(params[0, s] - p[0]) <= 1e-8 * p[0], s
        assert np.all(np.abs(params[1:, s] - p[1:]) <= 1e-9 * np.abs(p[1:]))
        assert np.all(np.abs(res[:2, s] - r[:2]) <= 1e-6 * r[:2]), s
        assert np.abs(temps[s] - t).max() <= 1e-3, s
    if method == "gauss_newton":
        assert np.allclose(params[0], true[0], rtol=1e-8, atol=0)
