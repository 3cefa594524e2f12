"""CPU oracle of the steady-flamelet residual and block Jacobian.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``; the CUDA product never
imports it.

A numpy restatement, for one flamelet on a uniform grid, of

* ``FlameletEquations.rhs`` (``pyrometheus/flamelets/equations.py:167-227``):
  ``R = chi/2 Lap(phi) + S(phi) m - BC``;
* ``FlameletEquations.jac`` (``equations.py:228-282``): central blocks
  ``chi/2 Lap_c + dS/dphi`` (zero source blocks at the two boundary
  points), lower ``chi[1:]/2 Lap_l``, upper ``chi[:-1]/2 Lap_u``;
* ``FlameletEquations.jacobian_action`` (``equations.py:411-450``):
  ``chi/2 Lap(v) + dS/dphi v`` with every point's source Jacobian;
* ``source_terms`` (``equations.py:313-359``): ``S = (v/rho, W w/rho)``
  with T from the enthalpy Newton of ``make_pyro.py:255-299`` and
  ``rho = get_density(p, T, Y)``;
* ``Laplacian.assemble_block_form`` / ``apply_operator``
  (``onedim_laplacian.py:144-212``): identity rows / dx^2 at the boundary
  points, the three-point stencil / dx^2 inside.

and, for the compressible-EOS consistency layer,

* ``FlameletEquations.adjoint_operator`` (``equations.py:451-516``):
  central blocks ``Lap_c`` inside plus ``(2/chi) dS/dphi^T``, boundary
  blocks ``chi/2 Lap_c``, the Laplacian's own lower/upper blocks;
* ``local_compressible_eos_rt`` (``equations.py:518-535``): ``R T / W_mix``
  at T(h, Y), and its gradient (central differences here);
* the pressure gradient of the source (``source_gradient_wrt_pressure``,
  ``equations.py:124-134``; fourth-order central differences here);
* ``CompressibleEOS.enthalpy_gradient`` / ``eos_gradient``
  (``thermodynamic_consistency.py:105-307``): adjoint solves with
  ``block_thomas`` and the boundary-trace / trapezoidal contractions.

As in the reference, the boundary dissipation rates are used as given
(``_enforce_dirichlet_bcs`` discards the arrays it builds).  The source
Jacobian here is by central differences of the source (the reference
checks its own ``jacfwd`` Jacobian the same way, ``test/test.py:300-374``);
the golden vectors carry the autodiff one.
"""

from __future__ import annotations

import numpy as np

from .block_thomas_oracle import block_thomas
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

    def jacobian_action(self, v, h, y, chi, visc, t_guess, p, dx):
        """``chi/2 Lap(v) + dS/dphi v`` per point, ``[S+1, N]``
        (``FlameletEquations.jacobian_action``, ``equations.py:411-450``):
        unlike :meth:`blocks`, the boundary points keep their source
        Jacobians."""
        sj = self.source_jacobian_fd(h, y, visc, t_guess, p)
        return 0.5 * chi * self.laplacian(v, dx) + np.einsum("ijk,ki->ji",
                                                             sj, v)

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

    # {{{ compressible-EOS consistency (adjoint solves)

    @staticmethod
    def adjoint_blocks(source_jac, chi, dx):
        """``(lower[N-1], central[N], upper[N-1])`` of the adjoint operator
        (``equations.py:451-516``) from per-point source Jacobians."""
        n_x, nv, _ = source_jac.shape
        eye = np.eye(nv)
        src = np.zeros_like(source_jac)
        src[1:-1] = np.transpose(
            2 * source_jac[1:-1] / chi[1:-1, None, None], (0, 2, 1))
        lap_c = np.stack([eye / dx ** 2] + [-2.0 * eye / dx ** 2] * (n_x - 2)
                         + [eye / dx ** 2])
        lap_l = np.stack([eye / dx ** 2] * (n_x - 2) + [0.0 * eye])
        lap_u = np.stack([0.0 * eye] + [eye / dx ** 2] * (n_x - 2))
        central = np.concatenate([
            (0.5 * chi[0] * lap_c[0])[None], lap_c[1:-1],
            (0.5 * chi[-1] * lap_c[-1])[None]]) + src
        return lap_l, central, lap_u

    def eos_rt(self, h, y, t_guess):
        """``R T / W_mix`` per point (``equations.py:517-535``)."""
        y = np.asarray(y, dtype=np.float64).reshape(self.S, -1)
        t = self.temperature(np.atleast_1d(h), y, t_guess)
        return self.th.gas_constant * t / \
            self.th.get_mixture_molecular_weight(y)

    def eos_rt_jacobian_fd(self, h, y, t_guess, rel=1e-6):
        """Central differences of :meth:`eos_rt` w.r.t. (h, Y), ``[N,
        S+1]``."""
        phi = np.vstack([h, y])
        nv, n_x = phi.shape
        jac = np.empty((n_x, nv))
        for q in range(nv):
            step = rel * np.maximum(np.abs(phi[q]), 1.0) if q == 0 else \
                np.full(n_x, rel)
            xp, xm = phi.copy(), phi.copy()
            xp[q] += step
            xm[q] -= step
            jac[:, q] = (self.eos_rt(xp[0], xp[1:], t_guess)
                         - self.eos_rt(xm[0], xm[1:], t_guess)) / (2 * step)
        return jac

    def source_pressure_gradient_fd(self, h, y, visc, t_guess, p,
                                    rel=1e-3):
        """dS/dp per point, ``[N, S+1]``, by fourth-order central
        differences (T(h, Y) does not depend on p)."""
        dp = rel * p

        def f(q):
            return self.source(h, y, visc, t_guess, q)
        return ((f(p - 2 * dp) - 8 * f(p - dp) + 8 * f(p + dp)
                 - f(p + 2 * dp)) / (12 * dp)).T

    @staticmethod
    def _traces(a, dx):
        """Oxidizer- plus fuel-side one-sided traces of an adjoint
        enthalpy (``thermodynamic_consistency.py:159-168``)."""
        ox = (1.5 * a[0] + 2 * a[1] - 0.5 * a[2]) / dx ** 2
        fu = (1.5 * a[-1] + 2 * a[-2] - 0.5 * a[-3]) / dx ** 2
        return ox + fu

    @staticmethod
    def _trapezoid(f):
        return 0.5 * (f[0] + f[-1]) + np.sum(f[1:-1])

    def enthalpy_gradient(self, source_jac, chi, dx, pdf):
        """``(adjoint_h [S+1, N], h_gradient)``: the adjoint solve with
        right-hand side ``-e_h pdf`` and its boundary traces
        (``thermodynamic_consistency.py:105-171``)."""
        lo, c, up = self.adjoint_blocks(source_jac, chi, dx)
        nv = c.shape[1]
        rhs = np.zeros((nv, c.shape[0]))
        rhs[0] = -pdf
        adj = block_thomas(lo, c, up, rhs.T).T
        return adj, self._traces(adj[0], dx)

    def eos_gradient(self, source_jac, rt, rt_jac, ds_dp, chi, dx, pdf, p):
        """``((density_gradient[2], energy_gradient[2]), (adjoint_d,
        adjoint_e))`` (``thermodynamic_consistency.py:173-307``).
        ``rt_jac``, ``ds_dp``: ``[N, S+1]``."""
        lo, c, up = self.adjoint_blocks(source_jac, chi, dx)
        nv = c.shape[1]
        dsdp = ds_dp / (0.5 * chi[:, None])
        rhs = (p / rt ** 2) * rt_jac.T * pdf
        adj_d = block_thomas(lo, c, up, rhs.T).T
        integrand = (1 / rt) * pdf + np.einsum("ij,ji->i", dsdp, adj_d)
        dens = np.array([self._trapezoid(integrand),
                         self._traces(adj_d[0], dx)])
        unit_h = np.zeros((nv, c.shape[0]))
        unit_h[0] = 1.0
        rhs = -(unit_h - rt_jac.T) * pdf
        adj_e = block_thomas(lo, c, up, rhs.T).T
        integrand = np.einsum("ij,ji->i", dsdp, adj_e)
        ener = np.array([self._trapezoid(integrand),
                         self._traces(adj_e[0], dx)])
        return (dens, ener), (adj_d, adj_e)

    # }}}
