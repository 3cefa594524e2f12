"""The flamelet-solver and compressible-EOS oracles against the reference's
own driver code (``pyrometheus/flamelets/solver.py``,
``thermodynamic_consistency.py``) run live on the same oracle pieces, with
a JAX stand-in (``oracle/refdriver.py``).  This pins the single-flamelet
restatements that the batched product drivers are tested against.
Skipped where the reference checkout is not present (it never is on a GPU
host)."""

import numpy as np
import pytest

from flamelet_solver_cases import (EOS_FLAMELETS, FLAMELETS, PRESSURE,
                                   SOLVE, eos_case, eos_config,
                                   flamelet_batch, mechanism, split)
from oracle import refgen

pytestmark = pytest.mark.skipif(not refgen.reference_available(),
                                reason="reference checkout not present")


def _cases(b):
    n = b["lengths"]
    return enumerate(zip(split(b["phi"], n), split(b["chi"], n),
                         split(b["visc"], n), split(b["T"], n)))


def _arr(state):
    return np.vstack([np.asarray(state.enthalpy),
                      np.asarray(state.mass_fractions)])


def test_oracle_driver_matches_the_reference_solver():
    """``FlameletSolver.solve`` of the reference and the oracle driver:
    identical states and temperatures on a steady-Newton flamelet, a
    time-march rescue and a second steady-Newton flamelet."""
    from oracle import refdriver
    from oracle.flamelet_solver_oracle import FlameletSolverOracle
    np.seterr(all="ignore")
    sol = mechanism()
    b = flamelet_batch(sol, [FLAMELETS[i] for i in (0, 1, 3)])
    stages = []
    for s, (phi0, chi, visc, tg) in _cases(b):
        ref = refdriver.reference_solver(sol, b["lengths"][s], b["dx"][s],
                                         b["y_ox"], b["y_fu"])
        st, temp = ref.solve(False, *SOLVE.values(), chi, visc, tg,
                             PRESSURE, b["h_ox"][s], b["h_fu"][s],
                             refdriver.state_of(phi0))
        orc = FlameletSolverOracle(sol, b["dx"][s], b["y_ox"], b["y_fu"])
        phi, t, info = orc.solve(*SOLVE.values(), chi, visc, tg, PRESSURE,
                                 b["h_ox"][s], b["h_fu"][s], phi0)
        np.testing.assert_array_equal(_arr(st), phi)
        np.testing.assert_array_equal(np.asarray(temp), t)
        stages.append(info["stage"])
    assert stages == [0, 1, 0]


def test_oracle_steps_match_the_reference():
    """``flamelet_newton_step`` and ``flamelet_time_step`` (with the
    reference's ``block_thomas``) against the oracle's update and step."""
    from oracle import refdriver
    from oracle.flamelet_solver_oracle import FlameletSolverOracle
    np.seterr(all="ignore")
    sol = mechanism()
    b = flamelet_batch(sol, [FLAMELETS[0]])
    _, (phi0, chi, visc, tg) = next(_cases(b))
    args = (chi, visc, tg, PRESSURE, b["h_ox"][0], b["h_fu"][0])
    ref = refdriver.reference_solver(sol, b["lengths"][0], b["dx"][0],
                                     b["y_ox"], b["y_fu"])
    orc = FlameletSolverOracle(sol, b["dx"][0], b["y_ox"], b["y_fu"])
    v = ref.flamelet_newton_step(refdriver.state_of(phi0), *args)
    ref_v = orc.newton_update(lambda x: orc.rhs(x, *args),
                              lambda x: orc.jac(x, *args[:4]), phi0)
    np.testing.assert_array_equal(_arr(v), ref_v)
    st, it, delta = ref.flamelet_time_step(
        refdriver.state_of(phi0), 20, 1e-9, refdriver.state_of(phi0), 1e-5,
        *args)
    phi, it2, d2 = orc.time_step(phi0, 20, 1e-9, phi0, 1e-5, *args)
    np.testing.assert_array_equal(_arr(st), phi)
    assert int(it) == it2 and float(delta) == d2


@pytest.mark.parametrize("method, tol", [("gauss_newton", 1e-12),
                                         ("picard", 1e-6)])
def test_oracle_eos_loop_matches_the_reference(method, tol):
    """``CompressibleEOS.ensure_consistency`` of the reference (its own
    adjoint gradients and updates) and the oracle loop: identical params,
    iteration counts, update norms, residual and ``(<h>, <T>)`` histories
    and states."""
    from oracle import refdriver
    from oracle.eos_consistency_oracle import CompressibleEOSOracle
    np.seterr(all="ignore")
    sol = mechanism()
    b = flamelet_batch(sol, EOS_FLAMELETS)
    pdf, true, start, rho, e = eos_case(sol, b)
    cfg = eos_config(method, maxiter=3, tol=tol)
    pdfs = split(pdf, b["lengths"])
    for s, (phi0, chi, visc, tg) in _cases(b):
        ref = refdriver.reference_eos(cfg, refdriver.reference_solver(
            sol, b["lengths"][s], b["dx"][s], b["y_ox"], b["y_fu"]))
        st, temp, params, it, delta, res, hist, flag = \
            ref.ensure_consistency(rho[s], e[s], start[:, s], pdfs[s], chi,
                                   visc, tg, refdriver.state_of(phi0))
        orc = CompressibleEOSOracle(sol, b["dx"][s], b["y_ox"], b["y_fu"],
                                    cfg)
        phi, t, p, it2, d2, r2, h2 = orc.ensure_consistency(
            rho[s], e[s], start[:, s], pdfs[s], chi, visc, tg, phi0)
        assert flag is False and it == it2 and float(delta) == d2
        np.testing.assert_array_equal(np.asarray(params), p)
        np.testing.assert_array_equal(res, r2)
        np.testing.assert_array_equal(hist, h2)
        np.testing.assert_array_equal(_arr(st), phi)
        np.testing.assert_array_equal(np.asarray(temp), t)


@pytest.mark.parametrize("n, nv", [(3, 10), (12, 10), (64, 54)])
def test_oracle_laplacian_matches_the_reference(n, nv):
    """The reference's ``Laplacian.assemble_block_form`` and
    ``apply_operator`` (``onedim_laplacian.py:144-212``, with its stencils
    and domain) against the oracle's blocks and Laplacian, bit for bit."""
    from oracle import refdriver
    from oracle.flamelet_oracle import FlameletOracle
    lap = refdriver.reference_laplacian(n)
    lap.assemble_block_form(nv)
    dx = 1.0 / (n - 1)
    assert lap.domain.dx == dx
    # chi = 2 makes the oracle's chi/2 factor exactly one
    lo, c, up = FlameletOracle.blocks(np.zeros((n, nv, nv)),
                                      np.full(n, 2.0), dx)
    np.testing.assert_array_equal(lo, lap.lower_blocks)
    np.testing.assert_array_equal(c, lap.central_blocks)
    np.testing.assert_array_equal(up, lap.upper_blocks)
    phi = np.random.default_rng(n).standard_normal((nv, n))
    np.testing.assert_array_equal(
        _arr(lap.apply_operator(refdriver.state_of(phi))),
        FlameletOracle.laplacian(phi, dx))


@pytest.mark.parametrize("tag", ["s9", "s53"])
def test_reference_flamelet_equations_live(tag):
    """The reference's ``FlameletEquations.rhs`` (``equations.py:167-238``,
    around its generated class and ``make_pyro_object``) run live: equal to
    the golden residual bit for bit and to the oracle within 1e-12 of the
    term magnitudes; its vmapped ``compressible_eos_rt`` against the
    oracle's ``R T`` (per-point against batch-wide temperature iteration
    stops: 1e-12 relative)."""
    from oracle import refdriver
    from oracle.flamelet_oracle import FlameletOracle
    from test_flamelet import _golden, _resid_scale
    np.seterr(all="ignore")
    sol, d = _golden(tag)
    n = d["h"].shape[0]
    eq = refdriver.reference_flamelet_equations(sol, n, d["y_ox"],
                                                d["y_fu"])
    phi = np.vstack([d["h"], d["Y"]])
    r = _arr(eq.rhs(refdriver.state_of(phi), refdriver._ready(d["chi"]),
                    d["visc"], d["T_guess"], float(d["P"]),
                    float(d["h_ox"]), float(d["h_fu"])))
    np.testing.assert_array_equal(r, d["resid"])
    fo = FlameletOracle(sol)
    ref = fo.residual(d["h"], d["Y"], d["chi"], d["visc"], d["T_guess"],
                      float(d["P"]), float(d["h_ox"]), float(d["h_fu"]),
                      d["y_ox"], d["y_fu"], float(d["dx"]))
    assert np.all(np.abs(r - ref) <= 1e-12 * _resid_scale(d))
    rt = np.asarray(eq.compressible_eos_rt(phi, d["T_guess"],
                                           float(d["P"])))
    ort = fo.eos_rt(d["h"], d["Y"], d["T_guess"])
    assert np.abs(rt - ort).max() <= 1e-12 * np.abs(ort).max()
    # the pieces of rhs: source terms, equation of state, boundary values
    src = _arr(eq.source_terms(refdriver.state_of(phi), d["visc"],
                               d["T_guess"], float(d["P"])))
    np.testing.assert_array_equal(src, d["src"])
    osrc = fo.source(d["h"], d["Y"], d["visc"], d["T_guess"], float(d["P"]))
    assert np.all(np.abs(src - osrc) <= 1e-12 * np.abs(osrc).max(
        axis=1, keepdims=True))
    rho, t = eq.equation_of_state(refdriver.state_of(phi), d["T_guess"],
                                  float(d["P"]))
    ot = fo.temperature(d["h"], d["Y"], d["T_guess"])
    np.testing.assert_array_equal(np.asarray(t), ot)
    # the generated class and the oracle sum 1/W_mix in different orders
    np.testing.assert_allclose(np.asarray(rho), fo.th.get_density(
        float(d["P"]), ot, d["Y"]), rtol=1e-15, atol=0)
    bc = _arr(eq.boundary_conditions(float(d["h_ox"]), float(d["h_fu"])))
    ref_bc = np.zeros_like(phi)
    ref_bc[0, 0], ref_bc[0, -1] = d["h_ox"], d["h_fu"]
    ref_bc[1:, 0], ref_bc[1:, -1] = d["y_ox"], d["y_fu"]
    np.testing.assert_array_equal(bc, ref_bc)


@pytest.mark.parametrize("tag", ["s9", "s53"])
def test_oracle_jacobian_assembly_matches_the_reference(tag):
    """The reference's ``jac`` and ``jacobian_action``
    (``equations.py:228-282, 411-450``) with central differences standing
    in for ``jax.jacfwd`` against the oracle's blocks and
    ``jacobian_action``: L and U bit for bit, the central blocks and the
    action within 1e-8 of each row's largest entry (the two difference
    Jacobians differ only by where the temperature iterations stop, per
    point in the reference, batch-wide in the oracle).  Both sides use the
    same central-difference source Jacobian, so this checks the assembly
    (Laplacian, per-point contraction, boundary handling), not dS/dphi
    itself; the device jacobian_action is checked against the oracle's in
    the GPU flamelet tests."""
    from oracle import refdriver
    from oracle.flamelet_oracle import FlameletOracle
    from test_flamelet import _golden
    np.seterr(all="ignore")
    sol, d = _golden(tag)
    n = d["h"].shape[0]
    eq = refdriver.reference_flamelet_equations(sol, n, d["y_ox"],
                                                d["y_fu"], fd_jacobian=True)
    phi = np.vstack([d["h"], d["Y"]])
    args = (refdriver._ready(d["chi"]), d["visc"], d["T_guess"],
            float(d["P"]))
    fo = FlameletOracle(sol)
    sj = fo.source_jacobian_fd(d["h"], d["Y"], d["visc"], d["T_guess"],
                               float(d["P"]))
    lo, c, up = (np.asarray(x) for x in eq.jac(refdriver.state_of(phi),
                                               *args))
    olo, oc, oup = fo.blocks(sj, d["chi"], float(d["dx"]))
    np.testing.assert_array_equal(lo, olo)
    np.testing.assert_array_equal(up, oup)
    assert np.all(np.abs(c - oc)
                  <= 1e-8 * np.abs(oc).max(axis=2, keepdims=True))
    v = np.random.default_rng(1).standard_normal(phi.shape)
    ja = _arr(eq.jacobian_action(refdriver.state_of(v),
                                 refdriver.state_of(phi), *args))
    ref = fo.jacobian_action(v, d["h"], d["Y"], d["chi"], d["visc"],
                             d["T_guess"], float(d["P"]), float(d["dx"]))
    assert np.all(np.abs(ja - ref)
                  <= 1e-8 * np.abs(ref).max(axis=1, keepdims=True))
