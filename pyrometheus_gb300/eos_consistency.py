"""Compressible-EOS consistency for many flamelets at once.

The counterpart of ``pyrometheus.flamelets.thermodynamic_consistency.
CompressibleEOS`` (``flamelets/thermodynamic_consistency.py:44-706``): for
each flamelet, find the pressure and boundary enthalpies ``(p, h_ox,
h_fu)`` whose steady solution, averaged under a mixture-fraction PDF, has
the density ``<p / (R T)>`` and internal energy ``<h - R T>`` a host flow
solver asks for.  Every flamelet runs the reference's outer iteration on
its own:

* ``evaluate_flamelet`` (``:310-398``): the flamelet solve (steady Newton
  first, time-march fallback) from the previous solution, then the
  adjoint gradients of the averaged density and energy with respect to
  ``p`` and the boundary enthalpy (two adjoint solves sharing one
  factorisation on the device), and the averages themselves;
* ``_gauss_newton_update`` (``:400-448``): the 2 x 2 normal equations
  ``(G^T G) v = -G^T r`` of the residual ``r = (<rho> - rho_sim, <e> -
  e_sim)``; the boundary step is applied to both ``h_ox`` and ``h_fu``;
* ``_picard_update`` (``:450-526``): ``dp = rho_sim <R T> - p`` and ``dh =
  (e_sim - <e>) / (d<h>/dh_b)`` from the enthalpy-only adjoint;
* ``ensure_consistency`` (``:602-706``): ``params += a v`` until ``|v| <
  tol`` or ``maxiter`` updates, recording ``|r|^2`` and ``(<h>, <T>)`` per
  iteration.

The batch keeps the flamelets still iterating; each outer iteration runs
the flamelet solver and the adjoint gradients over that set only (packed as
its own sub-batch), and the per-flamelet averages, 2 x 2 solves and
updates run on the host in float64 (one read of the point fields per
iteration; the solves and adjoints stay on the device).
"""

from __future__ import annotations

import time

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

from .flamelet_solver import FlameletState


class CompressibleEOS:
    """``CompressibleEOS(config, forward_solver)`` as in the reference; the
    forward solver is a :class:`~pyrometheus_gb300.flamelet_solver.
    FlameletSolver` over the batch.  ``config`` has the reference's schema:
    ``verbosity``, ``newton/{maxiter, tol}``, ``bdf/{newton/{maxiter, tol},
    time_step, maxsteps}``, ``max_attempts`` and ``eos/{update_size,
    update_method ("gauss_newton" | "picard"), maxiter, tol}``.

    ``params`` are ``[3]`` (shared) or ``[3, n_flamelets]`` rows ``(p,
    h_ox, h_fu)``; ``density_sim``/``energy_sim`` scalars or per flamelet;
    ``mixture_fraction_pdf``, ``diss_rate``, ``viscous_diss`` and
    ``temp_guess`` per row of the packed batch.
    """

    def __init__(self, config, forward_solver):
        self.config = config
        self.fwd_solver = forward_solver
        self._subs = {}

    def update_config_option(self, option_path: str, option_val):
        """``config[a][b][c] = option_val`` for ``option_path = "a/b/c"``,
        creating missing levels (``thermodynamic_consistency.py:81-104``)."""
        *parents, leaf = option_path.split("/")
        node = self.config
        for name in parents:
            child = node.setdefault(name, {})
            if not isinstance(child, dict):
                # the reference raises TypeError here too
                raise TypeError(f"config entry {name!r} on the path "
                                f"{option_path!r} is not a dict")
            node = child
        node[leaf] = option_val

    # {{{ gradients (whole batch; thermodynamic_consistency.py:105-307)

    def enthalpy_gradient(self, state, mixture_fraction_pdf, diss_rate,
                          viscous_diss, temp_guess, pressure):
        """``(rt [rows], adjoint_state_h, h_gradient [n_flamelets])``."""
        h, Y = self._hY(state)
        rt, adj, g = self.fwd_solver.gov_eqns.enthalpy_gradient(
            h, Y, diss_rate, viscous_diss, temp_guess, pressure,
            mixture_fraction_pdf)
        return rt, FlameletState(adj[0], adj[1:]), g

    def eos_gradient(self, state, mixture_fraction_pdf, diss_rate,
                     viscous_diss, temp_guess, pressure):
        """``((density_gradient, energy_gradient) [2, n_flamelets] each,
        (adjoint_state_d, adjoint_state_e))``; row 0 of a gradient is
        d/dp, row 1 d/dh at the boundaries."""
        h, Y = self._hY(state)
        (dg, eg), (ad, ae) = self.fwd_solver.gov_eqns.eos_gradient(
            h, Y, diss_rate, viscous_diss, temp_guess, pressure,
            mixture_fraction_pdf)
        return (dg, eg), (FlameletState(ad[0], ad[1:]),
                          FlameletState(ae[0], ae[1:]))

    # }}}

    def _hY(self, state):
        phi = self.fwd_solver._phi(state)
        return phi[0], phi[1:]

    # {{{ sub-batches

    def _sub(self, systems):
        """(solver, rows, flamelet of each row) of the flamelets
        *systems*; the whole batch is the forward solver itself."""
        fs = self.fwd_solver
        if len(systems) == fs.eq.nsys:
            return fs, None, np.repeat(np.arange(fs.eq.nsys), fs.eq.lengths)
        key = np.asarray(systems, dtype=np.int64).tobytes()
        sub = self._subs.pop(key, None)
        if sub is None:
            while len(self._subs) >= 2:
                self._subs.pop(next(iter(self._subs)))
            sub_fs = fs.subset(systems)
            rows = torch.as_tensor(fs.rows_of(systems), dtype=torch.int64,
                                   device=fs.eq.device)
            sub = (sub_fs, rows,
                   np.repeat(np.arange(len(systems)), sub_fs.eq.lengths))
        self._subs[key] = sub
        return sub

    @staticmethod
    def _sums(x, lengths):
        """Per-flamelet sums of a row field (numpy, flamelet by flamelet:
        the reference sums each flamelet's points with ``jnp.sum``)."""
        x = x.detach().cpu().numpy() if torch.is_tensor(x) else x
        offs = np.concatenate([[0], np.cumsum(lengths)])
        return np.array([np.sum(x[offs[s]:offs[s + 1]])
                         for s in range(len(lengths))])

    # }}}

    # {{{ one outer update of a set of flamelets

    def _forward(self, fs, p_rows, params, chi, visc, tg, state):
        c = self.config
        t0 = time.time()
        state, temp = fs.solve(
            c["verbosity"], c["newton"]["maxiter"], c["newton"]["tol"],
            c["bdf"]["newton"]["maxiter"], c["bdf"]["newton"]["tol"],
            c["bdf"]["time_step"], c["bdf"]["maxsteps"], True,
            c["max_attempts"], chi, visc, tg, p_rows, params[1], params[2],
            state)
        if c["verbosity"]:
            print(f"solve time: {time.time() - t0:.4e} s")
        return state, temp

    def _gauss_newton_update(self, fs, sys_row, density_sim, energy_sim,
                             params, pdf, chi, visc, tg, state):
        """``(state, temp, update [3, n], residual [2, n])``
        (``evaluate_flamelet`` and ``_gauss_newton_update``,
        ``thermodynamic_consistency.py:310-448``)."""
        eq = fs.gov_eqns
        dev = eq.device
        p_rows = torch.as_tensor(params[0][sys_row], device=dev)
        state, temp = self._forward(fs, p_rows, params, chi, visc, tg,
                                    state)
        h, Y = state
        t0 = time.time()
        (dg, eg), _ = eq.eos_gradient(h, Y, chi, visc, tg, p_rows, pdf)
        if self.config["verbosity"]:
            print(f"adjoint time: {time.time() - t0:.4e} s")
        rt, _ = eq.eos_rt(h, Y, temp_guess=temp, jacobian=False)
        density = self._sums((p_rows / rt) * pdf, eq.lengths)
        energy = self._sums((h - rt) * pdf, eq.lengths)
        dg, eg = dg.cpu().numpy(), eg.cpu().numpy()
        n = eq.nsys
        update = np.empty((3, n))
        residual = np.empty((2, n))
        for s in range(n):
            G = np.stack((dg[:, s], eg[:, s]))
            r = np.stack((density[s] - density_sim[s],
                          energy[s] - energy_sim[s]))
            v = np.linalg.solve(G.T @ G, -G.T @ r)
            update[:, s] = (v[0], v[1], v[1])
            residual[:, s] = r
        return state, temp, update, residual

    def _picard_update(self, fs, sys_row, density_sim, energy_sim, params,
                       pdf, chi, visc, tg, state):
        """``(state, temp, update [3, n], residual [2, n])``
        (``thermodynamic_consistency.py:450-526``)."""
        eq = fs.gov_eqns
        dev = eq.device
        p_rows = torch.as_tensor(params[0][sys_row], device=dev)
        state, temp = self._forward(fs, p_rows, params, chi, visc, tg,
                                    state)
        h, Y = state
        rt, _, dh_b = eq.enthalpy_gradient(h, Y, chi, visc, tg, p_rows, pdf)
        density = self._sums((p_rows / rt) * pdf, eq.lengths)
        energy = self._sums((h - rt) * pdf, eq.lengths)
        rt_avg = self._sums(rt * pdf, eq.lengths)
        dh_b = dh_b.cpu().numpy()
        dp = density_sim * rt_avg - params[0]
        dh = (energy_sim - energy) / dh_b
        update = np.stack((dp, dh, dh))
        residual = np.stack((density_sim - density, energy_sim - energy))
        return state, temp, update, residual

    # }}}

    def evaluate_flamelet(self, params, mixture_fraction_pdf, diss_rate,
                          viscous_diss, temp_guess, state_guess):
        """``(state, temperature, density [n], energy [n],
        density_gradient [2, n], energy_gradient [2, n])`` for the whole
        batch (``thermodynamic_consistency.py:310-398``)."""
        fs = self.fwd_solver
        eq = fs.gov_eqns
        n = eq.nsys
        params = self._params(params, n)
        sys_row = np.repeat(np.arange(n), eq.lengths)
        p_rows = torch.as_tensor(params[0][sys_row], device=eq.device)
        state, temp = self._forward(fs, p_rows, params, diss_rate,
                                    viscous_diss, temp_guess, state_guess)
        h, Y = state
        (dg, eg), _ = eq.eos_gradient(h, Y, diss_rate, viscous_diss,
                                      temp_guess, p_rows,
                                      mixture_fraction_pdf)
        rt, _ = eq.eos_rt(h, Y, temp_guess=temp, jacobian=False)
        pdf = fs._per(mixture_fraction_pdf, eq.rows, "mixture_fraction_pdf")
        density = self._sums((p_rows / rt) * pdf, eq.lengths)
        energy = self._sums((h - rt) * pdf, eq.lengths)
        return state, temp, density, energy, dg, eg

    def warmup(self, params, mixture_fraction_pdf, diss_rate, viscous_diss,
               temp_wmp, state_wmp):
        """One forward solve and both adjoint gradients
        (``thermodynamic_consistency.py:528-600``): builds the solver
        plans and loads the kernels."""
        n = self.fwd_solver.gov_eqns.nsys
        params = self._params(params, n)
        self.evaluate_flamelet(params, mixture_fraction_pdf, diss_rate,
                               viscous_diss, temp_wmp, state_wmp)
        eq = self.fwd_solver.gov_eqns
        sys_row = np.repeat(np.arange(n), eq.lengths)
        self.enthalpy_gradient(state_wmp, mixture_fraction_pdf, diss_rate,
                               viscous_diss, temp_wmp,
                               torch.as_tensor(params[0][sys_row],
                                               device=eq.device))

    @staticmethod
    def _params(params, n):
        params = np.asarray(params.cpu() if torch.is_tensor(params)
                            else params, dtype=np.float64)
        if params.shape == (3,):
            params = np.repeat(params[:, None], n, axis=1)
        if params.shape != (3, n):
            raise ValueError(f"params must have shape (3,) or (3, {n})")
        return params.copy()

    def ensure_consistency(self, density_sim, energy_sim, params,
                           mixture_fraction_pdf, diss_rate, viscous_diss,
                           temp_guess, state_guess):
        """Iterate every flamelet's ``(p, h_ox, h_fu)`` until its averaged
        density and energy match (``thermodynamic_consistency.py:602-706``).

        :returns: ``(state, temperature, params [3, n], it [n], delta [n],
            residual [maxiter, n], history [maxiter, 2, n], False)`` —
            per flamelet the index of its last update, that update's
            ``|v|``, ``|r|^2`` per iteration and ``(<h>, <T>)`` per
            iteration (nan after a flamelet stopped); the last entry is the
            reference's reserved flag.
        """
        fs = self.fwd_solver
        eq = fs.gov_eqns
        n = eq.nsys
        ec = self.config["eos"]
        a = ec["update_size"]
        method = ec["update_method"]
        if method == "gauss_newton":
            update_fn = self._gauss_newton_update
        elif method == "picard":
            update_fn = self._picard_update
        else:
            raise ValueError(f"Available {method} not implemented")
        if self.config["verbosity"]:
            print("EOS: using "
                  + ("Gauss-Newton" if method == "gauss_newton" else "Picard")
                  + " update")
        params = self._params(params, n)
        rho_sim = np.broadcast_to(np.asarray(density_sim, np.float64),
                                  (n,)).copy()
        e_sim = np.broadcast_to(np.asarray(energy_sim, np.float64),
                                (n,)).copy()
        pdf = fs._per(mixture_fraction_pdf, eq.rows, "mixture_fraction_pdf")
        chi = fs._per(diss_rate, eq.rows, "diss_rate")
        visc = fs._per(viscous_diss, eq.rows, "viscous_diss")
        temp = fs._per(temp_guess, eq.rows, "temp_guess").clone()
        phi = fs._phi(state_guess)
        maxiter = int(ec["maxiter"])
        residual = np.full((maxiter, n), np.nan)
        history = np.full((maxiter, 2, n), np.nan)
        its = np.full(n, -1, dtype=np.int64)
        deltas = np.full(n, np.inf)
        run = np.arange(n)
        for it in range(maxiter):
            if run.size == 0:
                break
            t0 = time.time()
            sub_fs, rows, sys_row = self._sub(run)

            def g(x):
                return x if rows is None else x.index_select(-1, rows)

            ph = g(phi)
            state, t_new, v, res = update_fn(
                sub_fs, sys_row, rho_sim[run], e_sim[run], params[:, run],
                g(pdf), g(chi), g(visc), g(temp),
                FlameletState(ph[0], ph[1:]))
            ph = torch.cat([state.enthalpy[None], state.mass_fractions])
            if rows is None:
                phi.copy_(ph)
                temp.copy_(t_new)
            else:
                phi.index_copy_(-1, rows, ph)
                temp.index_copy_(-1, rows, t_new)
            cost = np.array([np.linalg.norm(res[:, q]) ** 2
                             for q in range(run.size)])
            delta = np.array([np.linalg.norm(v[:, q])
                              for q in range(run.size)])
            if self.config["verbosity"]:
                print(f"EOS iteration {it}: time: {time.time() - t0:.4e} s, "
                      f"{run.size} flamelets, max residual = "
                      f"{cost.max():.4e}, max |v| = {delta.max():.4e}")
            params[:, run] = params[:, run] + a * v
            residual[it, run] = cost
            lengths = sub_fs.gov_eqns.lengths
            pdf_r = g(pdf)
            history[it, 0, run] = self._sums(state.enthalpy * pdf_r, lengths)
            history[it, 1, run] = self._sums(t_new * pdf_r, lengths)
            its[run] = it
            deltas[run] = delta
            done = delta < ec["tol"]
            if self.config["verbosity"] and done.any():
                print(f"EOS converged at iteration {it} for "
                      f"{int(done.sum())} flamelets")
            run = run[~done]
        return (FlameletState(phi[0], phi[1:]), temp, params, its, deltas,
                residual, history, False)
