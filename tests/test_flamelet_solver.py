"""The batched flamelet-solver driver (``pyrometheus_gb300.flamelet_solver``)
on the CPU: run on the oracle's pieces, it must reproduce, flamelet by
flamelet, the single-flamelet restatement of the reference driver
(``oracle/flamelet_solver_oracle.py``, after
``pyrometheus/flamelets/solver.py``) — same branch, same iteration counts,
same states — although the batch iterates only the flamelets still running
and packs them into sub-batches as they finish."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from flamelet_solver_cases import (PRESSURE, SOLVE, OracleEquations,  # noqa
                                   flamelet_batch, mechanism, split)
from oracle.flamelet_solver_oracle import FlameletSolverOracle  # noqa: E402
from pyrometheus_gb300.flamelet_solver import FlameletSolver  # noqa: E402


@pytest.fixture(scope="module")
def case():
    np.seterr(all="ignore")
    sol = mechanism()
    b = flamelet_batch(sol)
    eq = OracleEquations(sol, b["lengths"], b["dx"], b["y_ox"], b["y_fu"])
    return sol, b, FlameletSolver.from_equations(eq)


def _per_flamelet(b):
    n = b["lengths"]
    return zip(split(b["phi"], n), split(b["chi"], n), split(b["visc"], n),
               split(b["T"], n))


def _phi(state):
    return torch.cat([state.enthalpy[None], state.mass_fractions]).numpy()


def test_solve_matches_the_single_flamelet_driver(case):
    sol, b, fs = case
    st, temp = fs.solve(False, *SOLVE.values(), b["chi"], b["visc"], b["T"],
                        PRESSURE, b["h_ox"], b["h_fu"], b["phi"])
    rec = fs.last_solve
    phis = split(_phi(st), b["lengths"])
    temps = split(temp.numpy(), b["lengths"])
    for s, (phi0, chi, visc, tg) in enumerate(_per_flamelet(b)):
        orc = FlameletSolverOracle(sol, b["dx"][s], b["y_ox"], b["y_fu"])
        phi, t, info = orc.solve(*SOLVE.values(), chi, visc, tg, PRESSURE,
                                 b["h_ox"][s], b["h_fu"][s], phi0)
        assert rec["stage"][s] == info["stage"], s
        assert rec["newton_iterations"][s] == info["newton_iterations"], s
        assert rec["converged"][s] == (info["stage"] >= 0)
        np.testing.assert_array_equal(phis[s], phi)
        np.testing.assert_array_equal(temps[s], t)
    # the batch covers every branch of the driver
    assert set(rec["stage"].tolist()) == {0, 1, -1}


def test_time_march_and_newton_step_match(case):
    sol, b, fs = case
    steps, maxiter, tol, dt = 2, 20, 1e-9, 1e-5
    st, temp = fs.flamelet_time_march(False, maxiter, tol, steps, dt,
                                      b["chi"], b["visc"], b["T"], PRESSURE,
                                      b["h_ox"], b["h_fu"], b["phi"])
    v = fs.flamelet_newton_step(b["phi"], b["chi"], b["visc"], b["T"],
                                PRESSURE, b["h_ox"], b["h_fu"])
    st1, it1, d1 = fs.flamelet_time_step(b["phi"], maxiter, tol, b["phi"],
                                         dt, b["chi"], b["visc"], b["T"],
                                         PRESSURE, b["h_ox"], b["h_fu"])
    phis, temps = split(_phi(st), b["lengths"]), split(temp.numpy(),
                                                       b["lengths"])
    vs, phis1 = split(_phi(v), b["lengths"]), split(_phi(st1), b["lengths"])
    for s, (phi0, chi, visc, tg) in enumerate(_per_flamelet(b)):
        orc = FlameletSolverOracle(sol, b["dx"][s], b["y_ox"], b["y_fu"])
        args = (chi, visc, tg, PRESSURE, b["h_ox"][s], b["h_fu"][s])
        phi, t = orc.time_march(maxiter, tol, steps, dt, *args, phi0)
        np.testing.assert_array_equal(phis[s], phi)
        np.testing.assert_array_equal(temps[s], t)
        ref_v = orc.newton_update(lambda x: orc.rhs(x, *args),
                                  lambda x: orc.jac(x, *args[:4]), phi0)
        np.testing.assert_array_equal(vs[s], ref_v)
        phi1, it, d = orc.time_step(phi0, maxiter, tol, phi0, dt, *args)
        np.testing.assert_array_equal(phis1[s], phi1)
        assert it1[s] == it
        assert d1[s] == pytest.approx(d, rel=1e-12)


def test_inputs_are_checked(case):
    _, b, fs = case
    with pytest.raises(ValueError, match="state must have shape"):
        fs.flamelet_newton_step(b["phi"][:, :-1], b["chi"], b["visc"],
                                b["T"], PRESSURE, b["h_ox"], b["h_fu"])
    with pytest.raises(ValueError, match="diss_rate"):
        fs.flamelet_newton_step(b["phi"], b["chi"][:-1], b["visc"], b["T"],
                                PRESSURE, b["h_ox"], b["h_fu"])
    with pytest.raises(ValueError, match="h_ox"):
        fs.flamelet_newton_step(b["phi"], b["chi"], b["visc"], b["T"],
                                PRESSURE, b["h_ox"][:-1], b["h_fu"])
    with pytest.raises(ValueError, match="Unknown warmup"):
        fs.warmup("flamelet_solve")


def test_no_attempts_returns_the_guess(case):
    """``max_attempts = 0`` and no steady Newton: the guess comes back
    (``solver.py:562-600``)."""
    _, b, fs = case
    kw = dict(SOLVE, try_newton=False, max_attempts=0)
    st, temp = fs.solve(False, *kw.values(), b["chi"], b["visc"], b["T"],
                        PRESSURE, b["h_ox"], b["h_fu"], b["phi"])
    np.testing.assert_array_equal(_phi(st), b["phi"])
    np.testing.assert_array_equal(temp.numpy(), b["T"])
    assert not fs.last_solve["converged"].any()


def test_verbose_solve_reports_each_stage(capsys):
    """The progress lines of ``solver.py`` (Newton iterations, time steps,
    attempts, the summary) on one flamelet that needs a march."""
    np.seterr(all="ignore")
    sol = mechanism()
    b = flamelet_batch(sol, [(9, 1000.0, 5, False)])
    eq = OracleEquations(sol, b["lengths"], b["dx"], b["y_ox"], b["y_fu"])
    fs = FlameletSolver.from_equations(eq)
    kw = dict(SOLVE, try_newton=False, max_attempts=1, bdf_maxsteps=2)
    fs.solve(True, *kw.values(), b["chi"], b["visc"], b["T"], PRESSURE,
             b["h_ox"], b["h_fu"], b["phi"])
    out = capsys.readouterr().out
    assert "Attempt 0 of BDF time marching" in out
    assert out.count("BDF time step") == 2
    assert "Newton iter 0" in out
    assert fs.last_solve["stage"][0] in (1, -1)
    if fs.last_solve["stage"][0] == -1:
        assert "did not converge" in out


def test_from_domain_takes_the_reference_constructor_order(monkeypatch):
    """``FlameletSolver.from_domain(domain, gas, (y_ox, y_fu))``: grids with
    ``num_x`` and ``dx`` (one or a list) become the packed lengths and
    spacings of the flamelet equations."""
    import types

    import pyrometheus_gb300.flamelet as fl
    seen = {}

    class Recorder:
        def __init__(self, thermo, lengths, dx, y_ox, y_fu, device=None):
            seen.update(thermo=thermo, lengths=list(lengths), dx=list(dx),
                        y_ox=y_ox, y_fu=y_fu)
            self.nv, self.lengths = 3, np.asarray(lengths)

    monkeypatch.setattr(fl, "FlameletEquations", Recorder)
    grid = types.SimpleNamespace(num_x=101, dx=0.01)
    FlameletSolver.from_domain(grid, "gas", ("ox", "fu"))
    assert seen == dict(thermo="gas", lengths=[101], dx=[0.01], y_ox="ox",
                        y_fu="fu")
    FlameletSolver.from_domain([grid, types.SimpleNamespace(num_x=11,
                                                            dx=0.1)],
                               "gas", ("ox", "fu"))
    assert seen["lengths"] == [101, 11] and seen["dx"] == [0.01, 0.1]
