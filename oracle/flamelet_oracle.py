"""CPU oracle of the steady-flamelet residual and block Jacobian.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``; the CUDA product never
imports it.

A numpy restatement, for one flamelet on a uniform grid, of

* ``FlameletEquations.rhs`` (``pyrometheus/flamelets/equations.py:193-238``):
  ``R = chi/2 Lap(phi) + S(phi) m - BC``;
* ``FlameletEquations.jac`` (``equations.py:240-298``): central blocks
  ``chi/2 Lap_c + dS/dphi`` (zero source blocks at the two boundary
  points), lower ``chi[1:]/2 Lap_l``, upper ``chi[:-1]/2 Lap_u``;
* ``source_terms`` (``equations.py:340-385``): ``S = (v/rho, W w/rho)``
  with T from the enthalpy Newton of ``make_pyro.py:255-299`` and
  ``rho = get_density(p, T, Y)``;
* ``Laplacian.assemble_block_form`` / ``apply_operator``
  (``onedim_laplacian.py:144-212``): identity rows / dx^2 at the boundary
  points, the three-point stencil / dx^2 inside.

As in the reference, the boundary dissipation rates are used as given
(``_enforce_dirichlet_bcs`` discards the arrays it builds).  The source
Jacobian here is by central differences of the source (the reference
checks its own ``jacfwd`` Jacobian the same way, ``test/test.py:300-374``);
the golden vectors carry the autodiff one.
"""

from __future__ import annotations

import numpy as np

from .thermo_oracle import Thermochemistry


class FlameletOracle:
    def __init__(self, sol):
        self.th = Thermochemistry(sol)
        self.S = sol.n_species
        self.W = np.asarray(sol.molecular_weights, dtype=np.float64)

    def temperature(self, h, y, t_guess):
        return self.th.get_temperature_from_enthalpy(h, y, t_guess)

    def source(self, h, y, visc, t_guess, p):
        """``S = (v/rho, W w/rho)`` per point, ``[S+1, N]``."""
        h = np.atleast_1d(np.asarray(h, dtype=np.float64))
        y = np.asarray(y, dtype=np.float64).reshape(self.S, -1)
        t = self.temperature(h, y, t_guess)
        rho = self.th.get_density(p, t, y)
        w = self.th.get_net_production_rates(rho, t, y)
        return np.vstack([np.asarray(visc) / rho,
                          self.W[:, None] * w / rho])

    @staticmethod
    def laplacian(phi, dx):
        lap = np.empty_like(phi)
        lap[:, 0] = phi[:, 0] / dx ** 2
        lap[:, -1] = phi[:, -1] / dx ** 2
        lap[:, 1:-1] = (phi[:, :-2] - 2.0 * phi[:, 1:-1] + phi[:, 2:]) \
            / dx ** 2
        return lap

    def residual(self, h, y, chi, visc, t_guess, p, h_ox, h_fu, y_ox,
                 y_fu, dx):
        phi = np.vstack([h, y])
        n_x = phi.shape[1]
        src = self.source(h, y, visc, t_guess, p)
        mask = np.ones(n_x)
        mask[0] = mask[-1] = 0.0
        bc = np.zeros_like(phi)
        bc[0, 0], bc[0, -1] = h_ox, h_fu
        bc[1:, 0], bc[1:, -1] = y_ox, y_fu
        return 0.5 * chi * self.laplacian(phi, dx) + src * mask - bc

    def source_jacobian_fd(self, h, y, visc, t_guess, p, rel=1e-6):
        """Central differences of :meth:`source` w.r.t. (h, Y) per point,
        ``[N, S+1, S+1]``; steps ``rel * max(|h|, 1)`` for h and ``rel``
        for Y."""
        phi = np.vstack([h, y])
        nv, n_x = phi.shape
        jac = np.empty((n_x, nv, nv))
        for q in range(nv):
            step = rel * np.maximum(np.abs(phi[q]), 1.0) if q == 0 else \
                np.full(n_x, rel)
            xp, xm = phi.copy(), phi.copy()
            xp[q] += step
            xm[q] -= step
            fp = self.source(xp[0], xp[1:], visc, t_guess, p)
            fm = self.source(xm[0], xm[1:], visc, t_guess, p)
            jac[:, :, q] = ((fp - fm) / (2.0 * step)).T
        return jac

    @staticmethod
    def blocks(source_jac, chi, dx):
        """``(lower[N-1], central[N], upper[N-1])`` from per-point source
        Jacobians."""
        n_x, nv, _ = source_jac.shape
        eye = np.eye(nv)
        sj = source_jac.copy()
        sj[0] = 0.0
        sj[-1] = 0.0
        lap_c = np.stack([eye / dx ** 2] + [-2.0 * eye / dx ** 2] * (n_x - 2)
                         + [eye / dx ** 2])
        lap_l = np.stack([eye / dx ** 2] * (n_x - 2) + [0.0 * eye])
        lap_u = np.stack([0.0 * eye] + [eye / dx ** 2] * (n_x - 2))
        return (0.5 * chi[1:, None, None] * lap_l,
                0.5 * chi[:, None, None] * lap_c + sj,
                0.5 * chi[:-1, None, None] * lap_u)
