"""CPU oracle of the compressible-EOS consistency iteration, one flamelet at
a time.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``; the CUDA product never
imports it.

A numpy restatement of ``CompressibleEOS`` in
``pyrometheus/flamelets/thermodynamic_consistency.py`` for a single
flamelet, on the :class:`~oracle.flamelet_solver_oracle.FlameletSolverOracle`
driver and the :class:`~oracle.flamelet_oracle.FlameletOracle` adjoint
gradients (their source Jacobian, ``R T`` Jacobian and pressure gradient by
central differences):

* ``evaluate_flamelet`` (``:310-398``): solve (steady Newton first) from the
  previous solution, the density / energy gradients with the previous
  temperature as the Newton guess, ``R T`` at the new temperature, and the
  PDF sums ``<p / RT>``, ``<h - RT>``;
* ``_gauss_newton_update`` (``:400-448``): ``v = (G^T G)^-1 (-G^T r)``,
  update ``(v0, v1, v1)``;
* ``_picard_update`` (``:450-526``): ``dp = rho_sim <RT> - p``, ``dh =
  (e_sim - <e>) / h_gradient``;
* ``ensure_consistency`` (``:602-706``): ``params += a v`` until ``|v| <
  tol`` (after the update) or ``maxiter`` updates.
"""

from __future__ import annotations

import numpy as np

from .flamelet_solver_oracle import FlameletSolverOracle


class CompressibleEOSOracle:
    def __init__(self, sol, dx, y_ox, y_fu, config):
        self.fs = FlameletSolverOracle(sol, dx, y_ox, y_fu)
        self.fo = self.fs.fo
        self.dx = float(dx)
        self.config = config

    def _solve(self, params, chi, visc, t_guess, phi):
        c = self.config
        p, h_ox, h_fu = params
        phi, temp, _ = self.fs.solve(
            c["newton"]["maxiter"], c["newton"]["tol"],
            c["bdf"]["newton"]["maxiter"], c["bdf"]["newton"]["tol"],
            c["bdf"]["time_step"], c["bdf"]["maxsteps"], True,
            c["max_attempts"], chi, visc, t_guess, p, h_ox, h_fu, phi)
        return phi, temp

    def enthalpy_gradient(self, phi, pdf, chi, visc, t_guess, p):
        h, y = phi[0], phi[1:]
        rt = self.fo.eos_rt(h, y, t_guess)
        sj = self.fo.source_jacobian_fd(h, y, visc, t_guess, p)
        adj, g = self.fo.enthalpy_gradient(sj, chi, self.dx, pdf)
        return rt, adj, g

    def eos_gradient(self, phi, pdf, chi, visc, t_guess, p):
        h, y = phi[0], phi[1:]
        fo = self.fo
        rt = fo.eos_rt(h, y, t_guess)
        rtj = fo.eos_rt_jacobian_fd(h, y, t_guess)
        dsdp = fo.source_pressure_gradient_fd(h, y, visc, t_guess, p)
        sj = fo.source_jacobian_fd(h, y, visc, t_guess, p)
        return fo.eos_gradient(sj, rt, rtj, dsdp, chi, self.dx, pdf, p)

    def evaluate_flamelet(self, params, pdf, chi, visc, t_guess, phi):
        p = params[0]
        phi, temp = self._solve(params, chi, visc, t_guess, phi)
        (dg, eg), _ = self.eos_gradient(phi, pdf, chi, visc, t_guess, p)
        rt = self.fo.eos_rt(phi[0], phi[1:], temp)
        density = np.sum((p / rt) * pdf)
        energy = np.sum((phi[0] - rt) * pdf)
        return phi, temp, density, energy, dg, eg

    def gauss_newton_update(self, rho_sim, e_sim, params, pdf, chi, visc,
                            t_guess, phi):
        phi, temp, density, energy, dg, eg = self.evaluate_flamelet(
            params, pdf, chi, visc, t_guess, phi)
        G = np.stack((dg, eg))
        r = np.stack((density - rho_sim, energy - e_sim))
        v = np.linalg.solve(G.T @ G, -G.T @ r)
        return phi, temp, np.array([v[0], v[1], v[1]]), r

    def picard_update(self, rho_sim, e_sim, params, pdf, chi, visc,
                      t_guess, phi):
        p = params[0]
        phi, temp = self._solve(params, chi, visc, t_guess, phi)
        rt, _, dh_b = self.enthalpy_gradient(phi, pdf, chi, visc, t_guess, p)
        density = np.sum((p / rt) * pdf)
        energy = np.sum((phi[0] - rt) * pdf)
        dp = rho_sim * np.sum(rt * pdf) - p
        dh = (e_sim - energy) / dh_b
        return (phi, temp, np.array([dp, dh, dh]),
                np.array([rho_sim - density, e_sim - energy]))

    def ensure_consistency(self, rho_sim, e_sim, params, pdf, chi, visc,
                           t_guess, phi):
        ec = self.config["eos"]
        a = ec["update_size"]
        update = {"gauss_newton": self.gauss_newton_update,
                  "picard": self.picard_update}[ec["update_method"]]
        params = np.asarray(params, dtype=np.float64)
        temp = t_guess
        residual = np.full(ec["maxiter"], np.nan)
        history = np.full((ec["maxiter"], 2), np.nan)
        it, delta = -1, np.inf
        for it in range(ec["maxiter"]):
            phi, temp, v, res = update(rho_sim, e_sim, params, pdf, chi,
                                       visc, temp, phi)
            cost = np.linalg.norm(res) ** 2
            delta = np.linalg.norm(v)
            params = params + a * v
            residual[it] = cost
            history[it] = (np.sum(phi[0] * pdf), np.sum(temp * pdf))
            if delta < ec["tol"]:
                break
        return phi, temp, params, it, delta, residual, history
