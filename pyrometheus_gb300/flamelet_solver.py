"""Steady-flamelet solver driver for many flamelets at once.

The counterpart of ``pyrometheus.flamelets.solver.FlameletSolver``
(``flamelets/solver.py:16-600``) over the device pieces of
:mod:`pyrometheus_gb300.flamelet`: the residual, the block Jacobian (the
analytic reactor Jacobian plus the Laplacian blocks) and the batched
block-Thomas solve.

Every flamelet of the batch follows the reference driver's control flow on
its own:

* steady Newton (``_newton_loop_py``, ``solver.py:103-147``): at most
  ``maxiter`` updates ``v = -J^-1 R``; success once ``|v| < tol``, failure
  once ``|v|`` grew over the previous update;
* Crank-Nicolson time step (``flamelet_time_step``, ``:204-323``): the
  residual ``phi - phi_prev - dt/2 (R(phi) + R(phi_prev))`` with blocks
  ``(-dt/2 L, I - dt/2 C, -dt/2 U)``, updated while ``|v| > tol`` and fewer
  than ``maxiter`` updates were taken (``_newton_loop_lax``, ``:149-202``);
* time march (``flamelet_time_march``, ``:387-445``): ``maxsteps`` steps,
  the temperature re-solved after each from the march's own guess;
* ``solve`` (``:476-600``): an optional steady Newton first; then up to
  ``max_attempts`` rounds of a march followed by a steady Newton, the first
  converged round giving ``(state, T(state))``; a flamelet that never
  converges gets its last march's ``(state, temperature)``.

``|v|`` is the Frobenius norm of a flamelet's ``[S+1, N]`` update.  The batch
keeps the set of flamelets still iterating; each iteration evaluates the
temperature, residual and blocks and runs block-Thomas over that set only
(the set is packed into its own equations and solver plan, cached while it
does not change), so converged or failed flamelets cost nothing and keep
their state.  One host synchronisation per iteration reads the per-flamelet
norms, as the reference reads ``|v|`` after each of its updates.

Where the reference's traced loops would carry nan (a temperature iteration
or a solve that breaks down), the flamelet's norm here is nan as well: it
neither converges nor counts as diverged, and ends as the reference's does
when its iteration budget runs out.  The temperature iteration inside is
bounded (500 Newton steps to ``|dT| < 1e-10``) and returns its last iterate
when it does not converge.
"""

from __future__ import annotations

import time
from typing import NamedTuple

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


class FlameletState(NamedTuple):
    """Enthalpy ``[rows]`` and mass fractions ``[S, rows]`` of a packed
    batch (``flamelets/state.py:193-231``)."""
    enthalpy: "torch.Tensor"
    mass_fractions: "torch.Tensor"


class _Args(NamedTuple):
    chi: "torch.Tensor"      # [rows]
    visc: "torch.Tensor"     # [rows]
    tg: "torch.Tensor"       # [rows] temperature guess
    p: "torch.Tensor"        # [rows] or 0-d
    h_ox: "torch.Tensor"     # [nsys]
    h_fu: "torch.Tensor"     # [nsys]


class _Subset:
    """The flamelets ``systems`` (sorted indices into the batch) packed on
    their own: equations, solver plan, row gather index and the padded
    index that sums each flamelet's rows."""

    def __init__(self, parent, systems):
        eq = parent.eq
        self.systems = systems
        self.whole = len(systems) == eq.nsys
        dev = eq.device
        if self.whole:
            self.eq = eq
            self.rows = None
            lengths = eq.lengths
        else:
            self.eq = eq.subset(systems)
            lengths = eq.lengths[systems]
            self.rows = torch.as_tensor(parent.rows_of(systems),
                                        dtype=torch.int64, device=dev)
            self.sys = torch.as_tensor(systems, dtype=torch.int64,
                                       device=dev)
        n_rows = int(np.sum(lengths))
        offs = np.concatenate([[0], np.cumsum(lengths)])
        pad = np.full((len(systems), int(lengths.max())), n_rows,
                      dtype=np.int64)
        for q, n in enumerate(lengths):
            pad[q, :n] = np.arange(offs[q], offs[q] + n)
        self.pad = torch.as_tensor(pad, device=dev)
        self.solver = self.eq.linear_solver()

    def gather(self, x):
        """Rows of ``x`` ([..., rows]) belonging to the subset."""
        return x if self.whole else x.index_select(-1, self.rows)

    def scatter(self, dst, x):
        if self.whole:
            dst.copy_(x)
        else:
            dst.index_copy_(-1, self.rows, x)

    def args(self, a: _Args) -> _Args:
        if self.whole:
            return a
        p = a.p if a.p.dim() == 0 else a.p.index_select(0, self.rows)
        return _Args(a.chi.index_select(0, self.rows),
                     a.visc.index_select(0, self.rows),
                     a.tg.index_select(0, self.rows), p,
                     a.h_ox.index_select(0, self.sys),
                     a.h_fu.index_select(0, self.sys))

    def norms(self, x):
        """Frobenius norm of each flamelet's update, ``x`` [rows, nv]."""
        sq = (x * x).sum(dim=1)
        sq = torch.cat([sq, sq.new_zeros(1)])
        return torch.sqrt(sq[self.pad].sum(dim=1)).cpu().numpy()


class FlameletSolver:
    """Batched steady-flamelet solver.

    ``FlameletSolver(thermo, lengths, dx, (y_ox, y_fu))`` mirrors the
    reference's ``FlameletSolver(domain, pyro_gas, mass_frac_bcs)`` with
    the mixture-fraction grid given per flamelet (``lengths[s]`` points of
    spacing ``dx[s]``, packed along rows as for
    :class:`~pyrometheus_gb300.flamelet.FlameletEquations`);
    :meth:`from_equations` takes an existing equations object.

    States are :class:`FlameletState` tuples or ``[S+1, rows]`` arrays;
    ``diss_rate``, ``viscous_diss`` and ``temp_guess`` are per row (or
    scalars), ``pressure`` a scalar or per row, ``h_ox``/``h_fu`` scalars or
    per flamelet.  :meth:`solve` leaves a per-flamelet record in
    :attr:`last_solve`.
    """

    def __init__(self, thermo, lengths, dx, mass_frac_bcs, device=None):
        from .flamelet import FlameletEquations
        y_ox, y_fu = mass_frac_bcs
        self._setup(FlameletEquations(thermo, lengths, dx, y_ox, y_fu,
                                      device=device))

    @classmethod
    def from_equations(cls, equations):
        self = cls.__new__(cls)
        self._setup(equations)
        return self

    @classmethod
    def from_domain(cls, domain, pyro_gas, mass_frac_bcs, device=None):
        """The reference's constructor order, ``FlameletSolver(domain,
        pyro_gas, mass_frac_bcs)`` (``solver.py:53-60``): *domain* is a
        uniform mixture-fraction grid with ``num_x`` points of spacing
        ``dx`` (the reference's ``Domain``), or a sequence of such grids,
        one flamelet each."""
        domains = domain if isinstance(domain, (list, tuple)) else [domain]
        lengths = [int(d.num_x) for d in domains]
        dx = [float(d.dx) for d in domains]
        return cls(pyro_gas, lengths, dx, mass_frac_bcs, device=device)

    def _setup(self, eq):
        self.eq = eq
        self.gov_eqns = eq
        self.num_v = eq.nv
        self.offs = np.concatenate([[0], np.cumsum(eq.lengths)])
        self._subsets = {}
        self.last_solve = None

    def subset(self, systems):
        """A solver of the flamelets *systems* alone (indices into this
        batch, packed in the order given)."""
        return FlameletSolver.from_equations(self.eq.subset(systems))

    def rows_of(self, systems):
        """The rows of the flamelets *systems*, in that order."""
        return np.concatenate([np.arange(self.offs[s], self.offs[s + 1])
                               for s in np.asarray(systems, dtype=np.int64)])

    # {{{ inputs

    def _f64(self, x):
        if torch.is_tensor(x):
            return x.to(device=self.eq.device, dtype=torch.float64)
        return torch.as_tensor(np.asarray(x, dtype=np.float64),
                               device=self.eq.device)

    def _per(self, x, n, what):
        x = self._f64(x)
        if x.dim() == 0:
            x = x.expand(n)
        if tuple(x.shape) != (n,):
            raise ValueError(f"{what} must be a scalar or have shape ({n},)")
        return x.contiguous()

    def _args(self, diss_rate, viscous_diss, temp_guess, pressure, h_ox,
              h_fu) -> _Args:
        rows, nsys = self.eq.rows, self.eq.nsys
        p = self._f64(pressure)
        if p.dim() != 0:
            p = self._per(p, rows, "pressure")
        return _Args(self._per(diss_rate, rows, "diss_rate"),
                     self._per(viscous_diss, rows, "viscous_diss"),
                     self._per(temp_guess, rows, "temp_guess").clone(), p,
                     self._per(h_ox, nsys, "h_ox"),
                     self._per(h_fu, nsys, "h_fu"))

    def _phi(self, state):
        """``[S+1, rows]`` copy of a state."""
        nv, rows = self.num_v, self.eq.rows
        if isinstance(state, tuple):
            h, Y = state
            phi = torch.cat([self._f64(h).reshape(1, -1), self._f64(Y)])
        else:
            phi = self._f64(state).clone()
        if tuple(phi.shape) != (nv, rows):
            raise ValueError(f"state must have shape {(nv, rows)}")
        return phi.contiguous()

    @staticmethod
    def _state(phi):
        return FlameletState(phi[0], phi[1:])

    def _sub(self, systems) -> _Subset:
        """The packed subset of *systems*; the few most recent ones are
        kept (a subset holds a solver workspace of one block per row)."""
        systems = np.asarray(systems, dtype=np.int64)
        key = systems.tobytes()
        sub = self._subsets.pop(key, None)
        if sub is None:
            while len(self._subsets) >= 3:
                self._subsets.pop(next(iter(self._subsets)))
            sub = _Subset(self, systems)
        self._subsets[key] = sub
        return sub

    # }}}

    # {{{ updates

    def _evaluate(self, sub, ph, a):
        """T, R [S+1, rows] and the blocks of the subset at ``ph``."""
        eq = sub.eq
        h, Y = ph[0], ph[1:]
        T = eq.temperature(h, Y, a.tg, check=False)
        R = eq.rhs(h, Y, a.chi, a.visc, a.tg, a.p, a.h_ox, a.h_fu,
                   temperature=T)
        return T, R

    def _steady_update(self, sub, ph, a):
        """``x`` [rows, nv] with ``J x = -R`` (``_newton_update``,
        ``solver.py:63-101``)."""
        T, R = self._evaluate(sub, ph, a)
        L, C, U = sub.eq.jac(ph[0], ph[1:], a.chi, a.visc, a.tg, a.p,
                             temperature=T)
        return sub.solver.solve(L, C, U, (-R).T.contiguous())

    def _cn_update(self, sub, ph, ph_prev, r_prev, dt, a):
        """The Newton update of the Crank-Nicolson residual
        (``solver.py:253-323``)."""
        T, R = self._evaluate(sub, ph, a)
        F = (ph - ph_prev) - (0.5 * dt) * (R + r_prev)
        L, C, U = sub.eq.jac(ph[0], ph[1:], a.chi, a.visc, a.tg, a.p,
                             temperature=T)
        L.mul_(-0.5 * dt)
        U.mul_(-0.5 * dt)
        C.mul_(-0.5 * dt)
        C.diagonal(dim1=1, dim2=2).add_(1.0)
        return sub.solver.solve(L, C, U, (-F).T.contiguous())

    # }}}

    # {{{ loops over a set of flamelets (in place on the batch state)

    def _newton_loop_py(self, verbosity, phi, systems, maxiter, tol, a):
        n = len(systems)
        it = np.full(n, -1, dtype=np.int64)
        delta = np.full(n, np.inf)
        ok = np.zeros(n, dtype=bool)
        err_prev = np.full(n, np.inf)
        run = np.arange(n)
        for k in range(int(maxiter)):
            if run.size == 0:
                break
            t0 = time.time()
            sub = self._sub(systems[run])
            ph = sub.gather(phi)
            x = self._steady_update(sub, ph, sub.args(a))
            ph = ph + x.T
            sub.scatter(phi, ph)
            d = sub.norms(x)
            if verbosity:
                print(f"Newton iter {k}: time: {time.time() - t0:.4e} s, "
                      f"{run.size} flamelets, max |v| = {d.max():.4e}")
            it[run] = k
            delta[run] = d
            conv = d < tol
            div = ~conv & (err_prev[run] < d)
            ok[run[conv]] = True
            err_prev[run] = d
            run = run[~(conv | div)]
        return it, delta, ok

    def _newton_loop_lax(self, phi, phi_prev, r_prev, systems, maxiter, tol,
                         dt, a):
        n = len(systems)
        it = np.zeros(n, dtype=np.int64)
        delta = np.full(n, np.inf)
        run = np.arange(n) if (np.inf > tol and 0 < maxiter) \
            else np.arange(0)
        while run.size:
            sub = self._sub(systems[run])
            ph = sub.gather(phi)
            x = self._cn_update(sub, ph, sub.gather(phi_prev),
                                sub.gather(r_prev), dt, sub.args(a))
            ph = ph + x.T
            sub.scatter(phi, ph)
            d = sub.norms(x)
            it[run] += 1
            delta[run] = d
            run = run[(d > tol) & (it[run] < maxiter)]
        return it, delta

    def _time_step(self, phi, systems, maxiter, tol, dt, a):
        phi_prev = phi.clone()
        r_prev = torch.zeros_like(phi)
        sub = self._sub(systems)
        _, R = self._evaluate(sub, sub.gather(phi), sub.args(a))
        sub.scatter(r_prev, R)
        return self._newton_loop_lax(phi, phi_prev, r_prev, systems, maxiter,
                                     tol, dt, a)

    def _time_march(self, verbosity, maxiter, tol, maxsteps, dt, a, phi,
                    systems):
        """``maxsteps`` Crank-Nicolson steps of ``systems``; returns the
        temperature ``[rows]`` (re-solved for those flamelets from the
        march's guess ``a.tg``, the guess elsewhere)."""
        temp = a.tg.clone()
        sub = self._sub(systems)
        for step in range(int(maxsteps)):
            t0 = time.time()
            self._time_step(phi, systems, maxiter, tol, dt, a._replace(
                tg=temp))
            ph = sub.gather(phi)
            sub.scatter(temp, sub.eq.temperature(
                ph[0], ph[1:], sub.gather(a.tg), check=False))
            if verbosity:
                print(f"BDF time step {step}: time: {time.time() - t0:.4e} s, "
                      f"T_max = {float(sub.gather(temp).max()):.3f} K")
        return temp

    # }}}

    # {{{ reference-shaped public methods

    def flamelet_newton_step(self, state_guess, diss_rate, viscous_diss,
                             temp_guess, pressure, h_ox, h_fu):
        """The steady Newton update of every flamelet
        (``solver.py:325-385``), as a :class:`FlameletState`."""
        a = self._args(diss_rate, viscous_diss, temp_guess, pressure, h_ox,
                       h_fu)
        sub = self._sub(np.arange(self.eq.nsys))
        x = self._steady_update(sub, self._phi(state_guess), a)
        return self._state(x.T.contiguous())

    def flamelet_time_step(self, state, newton_maxiter, newton_tol,
                           state_prev, time_step, diss_rate, viscous_diss,
                           temp_guess, pressure, h_ox, h_fu):
        """One Crank-Nicolson step from ``state_prev`` with Newton started
        at ``state`` (``solver.py:204-323``): ``(state, iterations[nsys],
        |v|[nsys])``."""
        a = self._args(diss_rate, viscous_diss, temp_guess, pressure, h_ox,
                       h_fu)
        systems = np.arange(self.eq.nsys)
        phi = self._phi(state)
        phi_prev = self._phi(state_prev)
        r_prev = torch.zeros_like(phi)
        sub = self._sub(systems)
        _, R = self._evaluate(sub, phi_prev, a)
        sub.scatter(r_prev, R)
        it, delta = self._newton_loop_lax(phi, phi_prev, r_prev, systems,
                                          newton_maxiter, newton_tol,
                                          time_step, a)
        return self._state(phi), it, delta

    def flamelet_time_march(self, verbosity, newton_maxiter, newton_tol,
                            maxsteps, time_step, diss_rate, viscous_diss,
                            temp_guess, pressure, h_ox, h_fu, state_guess):
        """``maxsteps`` Crank-Nicolson steps of every flamelet
        (``solver.py:387-445``): ``(state, temperature)``."""
        a = self._args(diss_rate, viscous_diss, temp_guess, pressure, h_ox,
                       h_fu)
        phi = self._phi(state_guess)
        temp = self._time_march(verbosity, newton_maxiter, newton_tol,
                                maxsteps, time_step, a, phi,
                                np.arange(self.eq.nsys))
        return self._state(phi), temp

    def warmup(self, warmup_fn_name, *args):
        """Run one of the solver's methods once (``solver.py:447-474``):
        here it builds the solver plans and loads the kernels."""
        if warmup_fn_name == "flamelet_newton_step":
            return self.flamelet_newton_step(*args)
        if warmup_fn_name == "flamelet_time_step":
            return self.flamelet_time_step(*args)
        raise ValueError(f"Unknown warmup function name {warmup_fn_name}")

    def solve(self, verbosity, newton_maxiter, newton_tol,
              bdf_newton_maxiter, bdf_newton_tol, bdf_time_step,
              bdf_maxsteps, try_newton, max_attempts, diss_rate,
              viscous_diss, temp_guess, pressure, h_ox, h_fu, state_guess):
        """Steady flamelets by Newton with the time-march fallback
        (``solver.py:476-600``): ``(state, temperature)``.

        :attr:`last_solve` then holds, per flamelet, ``stage`` (0: the
        first steady Newton converged; k >= 1: after time-march round k;
        -1: no convergence), ``newton_iterations`` and ``delta`` (index and
        ``|v|`` of the last update of its last steady Newton loop, -1 and
        inf when it ran none) and ``converged``."""
        nsys = self.eq.nsys
        a = self._args(diss_rate, viscous_diss, temp_guess, pressure, h_ox,
                       h_fu)
        phi0 = self._phi(state_guess)
        out_phi, out_t = phi0.clone(), a.tg.clone()
        stage = np.full(nsys, -1, dtype=np.int64)
        its = np.full(nsys, -1, dtype=np.int64)
        deltas = np.full(nsys, np.inf)
        left = np.arange(nsys)

        def finish(phi, systems, st):
            sub = self._sub(systems)
            ph = sub.gather(phi)
            sub.scatter(out_phi, ph)
            sub.scatter(out_t, sub.eq.temperature(
                ph[0], ph[1:], sub.gather(a.tg), check=False))
            stage[systems] = st

        if try_newton:
            phi = phi0.clone()
            it, d, ok = self._newton_loop_py(verbosity, phi, left,
                                             newton_maxiter, newton_tol, a)
            its[:], deltas[:] = it, d
            if ok.any():
                finish(phi, left[ok], 0)
            left = left[~ok]
            if verbosity:
                print(f"Newton: {int(ok.sum())} of {nsys} flamelets "
                      "converged")
        phi, temp = phi0.clone(), a.tg.clone()
        for attempt in range(int(max_attempts)):
            if left.size == 0:
                break
            if verbosity:
                print(f"Attempt {attempt} of BDF time marching "
                      f"({left.size} flamelets)")
            temp = self._time_march(verbosity, bdf_newton_maxiter,
                                    bdf_newton_tol, bdf_maxsteps,
                                    bdf_time_step, a._replace(tg=temp), phi,
                                    left)
            phi_t = phi.clone()
            it, d, ok = self._newton_loop_py(verbosity, phi_t, left,
                                             newton_maxiter, newton_tol,
                                             a._replace(tg=temp))
            its[left], deltas[left] = it, d
            if ok.any():
                finish(phi_t, left[ok], attempt + 1)
            left = left[~ok]
        if left.size:
            sub = self._sub(left)
            sub.scatter(out_phi, sub.gather(phi))
            sub.scatter(out_t, sub.gather(temp))
            if verbosity:
                print(f"{left.size} flamelet solutions did not converge")
        self.last_solve = dict(stage=stage, newton_iterations=its,
                               delta=deltas, converged=stage >= 0)
        return self._state(out_phi), out_t

    # }}}
