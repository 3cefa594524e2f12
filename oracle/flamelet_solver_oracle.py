"""CPU oracle of the steady-flamelet solver driver, one flamelet at a time.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``; the CUDA product never
imports it.

A numpy restatement of ``pyrometheus/flamelets/solver.py`` for a single
flamelet on the :class:`~oracle.flamelet_oracle.FlameletOracle` pieces
(residual, central-difference source Jacobian, block assembly, numpy
block-Thomas):

* ``_newton_update`` (``solver.py:63-101``): ``v = -J^-1 R`` through
  ``block_thomas(L, C, U, -R^T)^T``;
* ``_newton_loop_py`` (``:103-147``): at most ``maxiter`` updates, stop with
  success when ``|v| < tol`` and with failure when ``|v|`` grew; the state
  keeps the last update either way;
* ``_newton_loop_lax`` (``:149-202``): updates while ``|v| > tol`` and fewer
  than ``maxiter`` were taken;
* ``flamelet_time_step`` (``:204-323``): Crank-Nicolson residual
  ``phi - phi_prev - dt/2 (R(phi) + R(phi_prev))`` and blocks
  ``(-dt/2 L, I - dt/2 C, -dt/2 U)``, driven by the bounded loop;
* ``flamelet_time_march`` (``:387-445``): ``maxsteps`` steps, the temperature
  re-solved after each from the march's own guess;
* ``solve`` (``:476-600``): an optional steady Newton first, then up to
  ``max_attempts`` rounds of a time march followed by a steady Newton; the
  first converged round returns ``(state, T(state))``, otherwise the last
  march's ``(state, temperature)``.

``|v|`` is the Frobenius norm of the ``[S+1, N]`` update (``_state_to_array``,
``state.py:297-305``).  Besides the state and temperature, :meth:`solve`
returns a record of how the flamelet got there (``stage``: 0 for the first
steady Newton, ``k`` for time-march round ``k``, -1 for no convergence; the
Newton iteration count and last update norm of the final steady loop).
"""

from __future__ import annotations

import numpy as np

from .block_thomas_oracle import block_thomas
from .flamelet_oracle import FlameletOracle


class FlameletSolverOracle:
    def __init__(self, sol, dx, y_ox, y_fu):
        self.fo = FlameletOracle(sol)
        self.S = sol.n_species
        self.nv = self.S + 1
        self.dx = float(dx)
        self.y_ox = np.asarray(y_ox, dtype=np.float64)
        self.y_fu = np.asarray(y_fu, dtype=np.float64)

    # {{{ pieces

    def rhs(self, phi, chi, visc, t_guess, p, h_ox, h_fu):
        return self.fo.residual(phi[0], phi[1:], chi, visc, t_guess, p, h_ox,
                                h_fu, self.y_ox, self.y_fu, self.dx)

    def jac(self, phi, chi, visc, t_guess, p):
        sj = self.fo.source_jacobian_fd(phi[0], phi[1:], visc, t_guess, p)
        return self.fo.blocks(sj, chi, self.dx)

    def temperature(self, phi, t_guess):
        return self.fo.temperature(phi[0], phi[1:], t_guess)

    @staticmethod
    def newton_update(fn, jac, phi):
        r = fn(phi)
        lo, c, up = jac(phi)
        return block_thomas(lo, c, up, -r.T).T

    # }}}

    def newton_loop_py(self, phi, maxiter, tol, args):
        chi, visc, t_guess, p, h_ox, h_fu = args

        def fn(x):
            return self.rhs(x, chi, visc, t_guess, p, h_ox, h_fu)

        def jac(x):
            return self.jac(x, chi, visc, t_guess, p)

        err_prev = np.inf
        it, delta = -1, np.inf
        for it in range(maxiter):
            v = self.newton_update(fn, jac, phi)
            phi = phi + v
            delta = np.linalg.norm(v)
            if delta < tol:
                return phi, it, delta, True
            if err_prev < delta:
                return phi, it, delta, False
            err_prev = delta
        return phi, it, delta, False

    def newton_loop_lax(self, fn, jac, phi, maxiter, tol):
        it, delta = 0, np.inf
        while delta > tol and it < maxiter:
            v = self.newton_update(fn, jac, phi)
            phi = phi + v
            it += 1
            delta = np.linalg.norm(v)
        return phi, it, delta

    def time_step(self, phi, maxiter, tol, phi_prev, dt, chi, visc, t_guess,
                  p, h_ox, h_fu):
        r_prev = self.rhs(phi_prev, chi, visc, t_guess, p, h_ox, h_fu)
        eye = np.eye(self.nv)

        def fn(x):
            return (x - phi_prev) - (0.5 * dt) * (
                self.rhs(x, chi, visc, t_guess, p, h_ox, h_fu) + r_prev)

        def jac(x):
            lo, c, up = self.jac(x, chi, visc, t_guess, p)
            return (-0.5 * dt) * lo, eye - (0.5 * dt) * c, (-0.5 * dt) * up

        return self.newton_loop_lax(fn, jac, phi, maxiter, tol)

    def time_march(self, maxiter, tol, maxsteps, dt, chi, visc, t_guess, p,
                   h_ox, h_fu, phi):
        temp = t_guess
        for _ in range(maxsteps):
            phi, _, _ = self.time_step(phi, maxiter, tol, phi, dt, chi, visc,
                                       temp, p, h_ox, h_fu)
            temp = self.temperature(phi, t_guess)
        return phi, temp

    def solve(self, newton_maxiter, newton_tol, bdf_newton_maxiter,
              bdf_newton_tol, bdf_time_step, bdf_maxsteps, try_newton,
              max_attempts, chi, visc, t_guess, p, h_ox, h_fu, phi_guess):
        phi_guess = np.asarray(phi_guess, dtype=np.float64)
        if try_newton:
            phi, it, delta, ok = self.newton_loop_py(
                phi_guess, newton_maxiter, newton_tol,
                (chi, visc, t_guess, p, h_ox, h_fu))
            if ok:
                return phi, self.temperature(phi, t_guess), dict(
                    stage=0, newton_iterations=it, delta=delta)
        phi, temp = phi_guess, t_guess
        it, delta = -1, np.inf
        for attempt in range(max_attempts):
            phi, temp = self.time_march(bdf_newton_maxiter, bdf_newton_tol,
                                        bdf_maxsteps, bdf_time_step, chi,
                                        visc, temp, p, h_ox, h_fu, phi)
            phi_t, it, delta, ok = self.newton_loop_py(
                phi, newton_maxiter, newton_tol,
                (chi, visc, temp, p, h_ox, h_fu))
            if ok:
                return phi_t, self.temperature(phi_t, t_guess), dict(
                    stage=attempt + 1, newton_iterations=it, delta=delta)
        return phi, temp, dict(stage=-1, newton_iterations=it, delta=delta)
