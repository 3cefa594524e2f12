"""CPU oracle: a numpy restatement of pyrometheus' generated Thermochemistry.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, by
``__graft_entry__.smoke()`` (as the checker) and by ``bench.py``'s CPU
baseline leg.  The CUDA product never imports or calls it.

Parity: pinned against golden vectors produced by the reference's own code
generator (``pyrometheus/codegen/python.py``) run in the build container;
see ``tests/golden/make_golden.py`` and ``tests/test_oracle_golden.py``.

The restatement follows the reference's formulas and branch semantics, one
function per generated method, on arrays shaped like the reference's
(species-major: ``Y[S, N]``, outputs ``[S, N]`` / ``[R, N]``):

* NASA-7 ``where(T > Tmid, hi, lo)`` polynomials -- ``chem_expr.py:51-174``;
* ``log_k_eq = sum nu'' g - sum nu' g - dnu*log(p0/RT)``, irreversible slots
  ``-0.17364695002734*T`` -- ``chem_expr.py:274-302``, ``python.py:360-373``;
* Arrhenius ``exp(log A + b log T - Ta/T)`` or ``A*T**b`` when ``Ea == 0`` --
  ``chem_expr.py:310-324``;
* third-body ``[M] = sum eff_k c_k + default * sum_rest c_k`` folded into
  ``k_fwd`` -- ``chem_expr.py:327-345``, ``python.py:469-472``;
* Lindemann/Troe falloff ``k_hi * F * Pr / (1 + Pr)`` --
  ``chem_expr.py:348-420``, ``python.py:399-450``;
* rates of progress ``k_f (prod c^nu' - exp(log_k_eq) prod c^nu'')`` where
  the forward exponents pair the reactants (in their stored order) with the
  ``orders`` values (in theirs) positionally, exactly as
  ``chem_expr.py:436-446`` zips them -- ``chem_expr.py:428-460``;
* ``omega_k = sum_j nu''_kj r_j - sum_j nu'_kj r_j`` -- ``chem_expr.py:467-487``;
* forward/reverse rates and creation/destruction -- ``chem_expr.py:490-567``;
* temperature Newton with a batch-wide ``||dT||_inf < 1e-6`` stop, at most
  500 iterations, else ``RuntimeError`` -- ``python.py:375-396``; the
  ``lax.while_loop`` variants with ``||f/j||_2 > 1e-10`` --
  ``flamelets/make_pyro.py:211-299``.
"""

from __future__ import annotations

import numpy as np

GAS_CONSTANT = 8314.46261815324
ONE_ATM = 101325.0
IRREVERSIBLE_LOG_KEQ_SLOPE = -0.17364695002734


class OracleTables:
    """Dense per-mechanism tables read from a Cantera-like ``Solution``."""

    def __init__(self, sol):
        self.sol = sol
        S, R = sol.n_species, sol.n_reactions
        self.S, self.R = S, R
        self.species_names = list(sol.species_names)
        self.W = np.array(sol.molecular_weights, dtype=np.float64)
        self.invW = 1.0 / self.W
        self.t_mid = np.zeros(S)
        self.hi = np.zeros((S, 7))
        self.lo = np.zeros((S, 7))
        for k, sp in enumerate(sol.species()):
            c = np.asarray(sp.thermo.coeffs, dtype=np.float64)
            self.t_mid[k], self.hi[k], self.lo[k] = c[0], c[1:8], c[8:15]
        self.nu_r = np.zeros((R, S))
        self.nu_p = np.zeros((R, S))
        self.fwd_terms = []     # per reaction: [(k, exponent)]
        self.rev_terms = []
        self.reversible = np.zeros(R, dtype=bool)
        self.kind = []          # "arrhenius" | "three-body" | "falloff"
        self.rate = []          # Arrhenius params or (low, high, type, coeffs)
        self.eff = np.zeros((R, S))
        idx = sol.species_index
        for j, r in enumerate(sol.reactions()):
            for sp in r.reactants:
                self.nu_r[j, idx(sp)] = sol.reactant_stoich_coeff(idx(sp), j)
            for sp in r.products:
                self.nu_p[j, idx(sp)] = sol.product_stoich_coeff(idx(sp), j)
            if r.orders:
                exps = list(r.orders.values())
            else:
                exps = list(r.reactants.values())
            self.fwd_terms.append([(idx(sp), float(nu)) for sp, nu in
                                   zip(r.reactants, exps)])
            self.rev_terms.append([(idx(sp), float(nu)) for sp, nu in
                                   r.products.items()])
            self.reversible[j] = bool(r.reversible)
            if r.reaction_type.startswith("falloff"):
                self.kind.append("falloff")
                rt = r.reaction_type.split("-")[1]
                self.rate.append((_arr(r.rate.low_rate),
                                  _arr(r.rate.high_rate), rt,
                                  np.array(r.rate.falloff_coeffs,
                                           dtype=np.float64)))
            else:
                self.kind.append("three-body"
                                 if r.reaction_type == "three-body-Arrhenius"
                                 else "arrhenius")
                self.rate.append(_arr(r.rate))
            if r.third_body is not None and self.kind[-1] != "arrhenius":
                self.eff[j, :] = r.third_body.default_efficiency
                for sp, e in r.third_body.efficiencies.items():
                    if sp in sol.species_names:
                        self.eff[j, idx(sp)] = e
        self.dnu = (self.nu_p - self.nu_r).sum(axis=1)
        self.falloff_idx = [j for j, k in enumerate(self.kind)
                            if k == "falloff"]


def _arr(rate):
    a = float(rate.pre_exponential_factor)
    b = float(rate.temperature_exponent)
    ta = float(rate.activation_energy) / GAS_CONSTANT
    return (a, b, ta)


def _rate_coefficient(p, t):
    """``chem_expr.py:310-324``."""
    a, b, ta = p
    if ta == 0:
        return a * t ** b
    return np.exp(np.log(a) + b * np.log(t) - ta / t)


class Thermochemistry:
    """Numpy restatement of the generated class' kinetics/thermo methods."""

    def __init__(self, sol):
        self.tab = OracleTables(sol)
        self.num_species = self.tab.S
        self.num_reactions = self.tab.R
        self.species_names = self.tab.species_names
        self.molecular_weights = self.tab.W
        self.inv_molecular_weights = self.tab.invW
        self.gas_constant = GAS_CONSTANT
        self.one_atm = ONE_ATM

    # {{{ mixture helpers (python.py:248-311)

    def get_specific_gas_constant(self, y):
        return self.gas_constant * np.tensordot(self.tab.invW, y, 1)

    def get_mixture_molecular_weight(self, y):
        return 1.0 / np.tensordot(self.tab.invW, y, 1)

    def get_density(self, p, t, y):
        return p * self.get_mixture_molecular_weight(y) / (
            self.gas_constant * t)

    def get_pressure(self, rho, t, y):
        return rho * self.gas_constant * t / \
            self.get_mixture_molecular_weight(y)

    def get_concentrations(self, rho, y):
        return self.tab.invW[:, None] * rho * np.asarray(y).reshape(
            self.tab.S, -1)

    def get_mole_fractions(self, mmw, y):
        return self.tab.invW[:, None] * np.asarray(y).reshape(
            self.tab.S, -1) * mmw

    def get_mass_average_property(self, y, prop):
        y = np.asarray(y).reshape(self.tab.S, -1)
        return (y * prop * self.tab.invW[:, None]).sum(axis=0)

    def get_mixture_specific_heat_cp_mass(self, t, y):
        return self.gas_constant * self.get_mass_average_property(
            y, self.get_species_specific_heats_r(t))

    def get_mixture_specific_heat_cv_mass(self, t, y):
        return self.gas_constant * self.get_mass_average_property(
            y, self.get_species_specific_heats_r(t) - 1.0)

    def get_mixture_enthalpy_mass(self, t, y):
        return self.gas_constant * t * self.get_mass_average_property(
            y, self.get_species_enthalpies_rt(t))

    def get_mixture_internal_energy_mass(self, t, y):
        return self.gas_constant * t * self.get_mass_average_property(
            y, self.get_species_enthalpies_rt(t) - 1.0)

    # }}}

    # {{{ NASA-7 (chem_expr.py:51-174)

    def _nasa(self, t, fn):
        t = np.atleast_1d(np.asarray(t, dtype=np.float64))
        hi = fn(self.tab.hi[:, :, None], t[None, :])
        lo = fn(self.tab.lo[:, :, None], t[None, :])
        return np.where(t[None, :] > self.tab.t_mid[:, None], hi, lo)

    def get_species_specific_heats_r(self, t):
        return self._nasa(t, lambda c, t: c[:, 0] + c[:, 1] * t
                          + c[:, 2] * t ** 2 + c[:, 3] * t ** 3
                          + c[:, 4] * t ** 4)

    def get_species_enthalpies_rt(self, t):
        return self._nasa(t, lambda c, t: c[:, 0] + c[:, 1] / 2 * t
                          + c[:, 2] / 3 * t ** 2 + c[:, 3] / 4 * t ** 3
                          + c[:, 4] / 5 * t ** 4 + c[:, 5] / t)

    def get_species_entropies_r(self, t):
        return self._nasa(t, lambda c, t: c[:, 0] * np.log(t)
                          + c[:, 1] * t + c[:, 2] / 2 * t ** 2
                          + c[:, 3] / 3 * t ** 3 + c[:, 4] / 4 * t ** 4
                          + c[:, 6])

    def get_species_gibbs_rt(self, t):
        return self.get_species_enthalpies_rt(t) - \
            self.get_species_entropies_r(t)

    def get_species_specific_heats_r_derivative(self, t):
        return self._nasa(t, lambda c, t: c[:, 1] + 2 * c[:, 2] * t
                          + 3 * c[:, 3] * t ** 2 + 4 * c[:, 4] * t ** 3)

    def get_species_enthalpies_rt_derivative(self, t):
        return self._nasa(t, lambda c, t: c[:, 1] / 2 + 2 * c[:, 2] / 3 * t
                          + 3 * c[:, 3] / 4 * t ** 2
                          + 4 * c[:, 4] / 5 * t ** 3 - c[:, 5] / t ** 2)

    def get_species_entropies_rt_derivative(self, t):
        return self._nasa(t, lambda c, t: c[:, 0] / t + c[:, 1]
                          + c[:, 2] * t + c[:, 3] * t ** 2
                          + c[:, 4] * t ** 3)

    # }}}

    # {{{ kinetics

    def get_equilibrium_constants(self, t):
        """``python.py:360-373``; ``chem_expr.py:274-302``."""
        t = np.atleast_1d(np.asarray(t, dtype=np.float64))
        c0 = np.log(self.one_atm / (self.gas_constant * t))
        g = self.get_species_gibbs_rt(t)
        tab = self.tab
        out = np.empty((tab.R, t.size))
        for j in range(tab.R):
            if not tab.reversible[j]:
                out[j] = IRREVERSIBLE_LOG_KEQ_SLOPE * t
                continue
            sp = (tab.nu_p[j, :, None] * g).sum(axis=0, where=(
                tab.nu_p[j, :, None] != 0))
            sr = (tab.nu_r[j, :, None] * g).sum(axis=0, where=(
                tab.nu_r[j, :, None] != 0))
            out[j] = sp - sr
            if tab.dnu[j] != 0:
                out[j] -= tab.dnu[j] * c0
        return out

    def _third_body(self, j, c):
        return (self.tab.eff[j, :, None] * c).sum(axis=0)

    def get_falloff_rates(self, t, c, k_fwd):
        """Overwrites the falloff slots of *k_fwd*; ``python.py:399-450``."""
        t = np.atleast_1d(np.asarray(t, dtype=np.float64))
        for j in self.tab.falloff_idx:
            low, high, ftype, fc = self.tab.rate[j]
            k_hi = _rate_coefficient(high, t) * np.ones_like(t)
            k_lo = _rate_coefficient(low, t) * np.ones_like(t)
            pr = self._third_body(j, c) * k_lo / k_hi
            if ftype == "Troe":
                center = (1.0 - fc[0]) * np.exp(-t / fc[1]) \
                    + fc[0] * np.exp(-t / fc[2])
                if len(fc) == 4:
                    center = center + np.exp(-fc[3] / t)
                log_fc = np.log10(center)
                with np.errstate(divide="ignore", invalid="ignore"):
                    log_pr = np.log10(pr)
                    cc = -0.4 - 0.67 * log_fc
                    nn = 0.75 - 1.27 * log_fc
                    f = np.where(pr > 0,
                                 (log_pr + cc) / (nn - 0.14 * (log_pr + cc)),
                                 -1 / 0.14)
                blend = 10 ** (log_fc / (1 + f ** 2))
            elif ftype == "Lindemann":
                blend = np.ones_like(t)
            else:
                raise ValueError(f"unexpected falloff type {ftype}")
            k_fwd[j] = k_hi * (blend * pr / (1 + pr))

    def get_fwd_rate_coefficients(self, t, c):
        """``python.py:453-473``."""
        t = np.atleast_1d(np.asarray(t, dtype=np.float64))
        c = np.asarray(c).reshape(self.tab.S, -1)
        tab = self.tab
        k = np.zeros((tab.R, t.size))
        for j in range(tab.R):
            if tab.kind[j] != "falloff":
                k[j] = _rate_coefficient(tab.rate[j], t)
        self.get_falloff_rates(t, c, k)
        for j in range(tab.R):
            if tab.kind[j] == "three-body":
                k[j] *= self._third_body(j, c)
        return k

    @staticmethod
    def _prod(c, terms, n):
        out = np.ones(n)
        for k, nu in terms:
            out = out * (c[k] if nu == 1.0 else c[k] ** nu)
        return out

    def _fwd_rev_products(self, c):
        n = c.shape[1]
        pf = np.stack([self._prod(c, tm, n) for tm in self.tab.fwd_terms])
        pr = np.stack([self._prod(c, tm, n) for tm in self.tab.rev_terms])
        return pf, pr

    def get_net_rates_of_progress(self, t, c):
        """``python.py:475-484``; ``chem_expr.py:428-460``."""
        c = np.asarray(c).reshape(self.tab.S, -1)
        k = self.get_fwd_rate_coefficients(t, c)
        lk = self.get_equilibrium_constants(t)
        pf, pr = self._fwd_rev_products(c)
        rev = self.tab.reversible[:, None]
        return k * np.where(rev, pf - np.exp(lk) * pr, pf)

    def get_fwd_rates_of_progress(self, t, c):
        c = np.asarray(c).reshape(self.tab.S, -1)
        pf, _ = self._fwd_rev_products(c)
        return self.get_fwd_rate_coefficients(t, c) * pf

    def get_rev_rates_of_progress(self, t, c):
        c = np.asarray(c).reshape(self.tab.S, -1)
        k = self.get_fwd_rate_coefficients(t, c)
        lk = self.get_equilibrium_constants(t)
        _, pr = self._fwd_rev_products(c)
        return np.where(self.tab.reversible[:, None], k * np.exp(lk) * pr,
                        0.0)

    def get_net_production_rates(self, rho, t, y):
        """``python.py:486-495``; ``chem_expr.py:467-487``."""
        c = self.get_concentrations(rho, y)
        r = self.get_net_rates_of_progress(t, c)
        tab = self.tab
        return tab.nu_p.T @ r - tab.nu_r.T @ r

    def get_creation_destruction_rates(self, rho, t, y):
        """``python.py:543-562``; ``chem_expr.py:525-567``."""
        c = self.get_concentrations(rho, y)
        rf = self.get_fwd_rates_of_progress(t, c)
        rr = self.get_rev_rates_of_progress(t, c)
        tab = self.tab
        cdot = tab.nu_p.T @ rf + tab.nu_r.T @ rr
        ddot = tab.nu_r.T @ rf + tab.nu_p.T @ rr
        return cdot, ddot

    def get_creation_rates(self, rho, t, y):
        return self.get_creation_destruction_rates(rho, t, y)[0]

    def get_destruction_rates(self, rho, t, y):
        return self.get_creation_destruction_rates(rho, t, y)[1]

    # }}}

    # {{{ temperature

    def get_temperature(self, e_or_h, t_guess, y, do_energy=False):
        """``python.py:375-396``: batch-wide stop on ``||dT||_inf < 1e-6``."""
        if do_energy:
            pv, he = (self.get_mixture_specific_heat_cv_mass,
                      self.get_mixture_internal_energy_mass)
        else:
            pv, he = (self.get_mixture_specific_heat_cp_mass,
                      self.get_mixture_enthalpy_mass)
        e_or_h = np.asarray(e_or_h, dtype=np.float64)
        t = t_guess * (0 * e_or_h + 1.0)
        for _ in range(500):
            dt = (e_or_h - he(t, y)) / pv(t, y)
            t = t + dt
            if np.max(np.abs(dt)) < 1.0e-6:
                return t
        raise RuntimeError("Temperature iteration failed to converge")

    def _while_newton(self, target, y, t0, he, pv):
        """``make_pyro.py:211-253`` / ``:255-299``: iterate while
        ``||f/j||_2 > 1e-10``."""
        t = np.asarray(t0, dtype=np.float64) * np.ones_like(
            np.asarray(target, dtype=np.float64))
        for _ in range(10000):
            f = target - he(t, y)
            j = -pv(t, y)
            if not np.linalg.norm(f / j) > 1e-10:
                return t
            t = t - f / j
        raise RuntimeError("Temperature iteration failed to converge")

    def get_temperature_from_energy(self, e, y, t0):
        return self._while_newton(e, y, t0,
                                  self.get_mixture_internal_energy_mass,
                                  self.get_mixture_specific_heat_cv_mass)

    def get_temperature_from_enthalpy(self, h, y, t0):
        return self._while_newton(h, y, t0, self.get_mixture_enthalpy_mass,
                                  self.get_mixture_specific_heat_cp_mass)

    # }}}

    # {{{ mixture-averaged transport (python.py:564-641, chem_expr.py:190-267)

    def _transport(self):
        tr = getattr(self.tab.sol, "transport", None)
        if tr is None:
            raise ValueError("mechanism has no transport fits")
        return tr

    @staticmethod
    def _fit_poly(c, t):
        """``c0 + c1 ln T + c2 (ln T)^2 + c3 (ln T)^3 + c4 (ln T)^4``,
        summed left to right with the powers formed by ``**``, as the
        generated expressions of ``chem_expr.py:190-244`` evaluate."""
        lt = np.log(t)
        return (c[0] + c[1] * lt + c[2] * (lt ** 2) + c[3] * (lt ** 3)
                + c[4] * (lt ** 4))

    def get_species_viscosities(self, t):
        """``sqrt(T) * poly(ln T)^2`` -- chem_expr.py:190-205."""
        t = np.asarray(t, dtype=np.float64)
        v = self._transport().viscosity
        return np.stack([np.sqrt(t) * self._fit_poly(v[k], t) ** 2
                         for k in range(self.tab.S)])

    def get_species_thermal_conductivities(self, t):
        """``sqrt(T) * poly(ln T)`` -- chem_expr.py:208-223."""
        t = np.asarray(t, dtype=np.float64)
        c = self._transport().conductivity
        return np.stack([np.sqrt(t) * self._fit_poly(c[k], t)
                         for k in range(self.tab.S)])

    def get_species_binary_mass_diffusivities(self, t):
        """``sqrt(T) * T * poly(ln T)``, shape (S, S, N) -- chem_expr.py:
        226-244, python.py:582-593."""
        t = np.asarray(t, dtype=np.float64)
        d = self._transport().diffusivity
        S = self.tab.S
        return np.stack([np.stack([np.sqrt(t) * t * self._fit_poly(d[i, j], t)
                                   for j in range(S)]) for i in range(S)])

    def get_mixture_viscosity_mixavg(self, t, y):
        """Wilke's rule -- python.py:595-605, chem_expr.py:247-259:
        ``f_k = sum_j x_j (1 + sqrt(mu_k/mu_j sqrt(W_j/W_k)))^2 /
        sqrt(8 (1 + W_k/W_j))``, ``mu = sum_k x_k mu_k / f_k``."""
        y = np.asarray(y, dtype=np.float64).reshape(self.tab.S, -1)
        mmw = self.get_mixture_molecular_weight(y)
        x = self.get_mole_fractions(mmw, y)
        mu = self.get_species_viscosities(t)
        W = self.tab.W
        S = self.tab.S
        f = []
        for k in range(S):
            acc = 0
            for j in range(S):
                acc = acc + (x[j] * (1 + np.sqrt(
                    (mu[k] / mu[j]) * np.sqrt(W[j] / W[k]))) ** 2
                    / np.sqrt(8 * (1 + (W[k] / W[j]))))
            f.append(acc)
        return sum(x * mu / np.stack(f))

    def get_mixture_thermal_conductivity_mixavg(self, t, y):
        """``(sum x lam + 1 / sum x/lam) / 2`` -- python.py:607-613."""
        y = np.asarray(y, dtype=np.float64).reshape(self.tab.S, -1)
        mmw = self.get_mixture_molecular_weight(y)
        x = self.get_mole_fractions(mmw, y)
        lam = self.get_species_thermal_conductivities(t)
        return 0.5 * (sum(x * lam) + 1 / sum(x / lam))

    def get_species_mass_diffusivities_mixavg(self, p, t, y):
        """``(mmw - x_k W_k) / (p mmw (sum_i x_i/D_ik - x_k/D_kk))``, or
        ``D_kk / p`` where that denominator is not positive --
        python.py:615-641, chem_expr.py:262-271."""
        y = np.asarray(y, dtype=np.float64).reshape(self.tab.S, -1)
        mmw = self.get_mixture_molecular_weight(y)
        x = self.get_mole_fractions(mmw, y)
        bd = self.get_species_binary_mass_diffusivities(t)
        S = self.tab.S
        out = []
        for k in range(S):
            xs = 0
            for i in range(S):
                xs = xs + x[i] / bd[i][k]
            denom = xs - x[k] / bd[k][k]
            with np.errstate(divide="ignore", invalid="ignore"):
                out.append(np.where(np.greater(denom, 0 * t),
                                    (mmw - x[k] * self.tab.W[k])
                                    / (p * mmw * denom), bd[k][k] / p))
        return np.stack(out)

    # }}}

    # {{{ constant-pressure reactor source and its Jacobian

    def reactor_source(self, p, t, y):
        """``[dT/dt, dY/dt]`` of an adiabatic constant-pressure reactor:
        ``dY_k/dt = W_k w_k / rho``, ``dT/dt = -sum_k H_k w_k / (rho cp)``
        with molar enthalpies ``H_k = R T (h/RT)_k``."""
        t = np.atleast_1d(np.asarray(t, dtype=np.float64))
        y = np.asarray(y).reshape(self.tab.S, -1)
        rho = self.get_density(p, t, y)
        w = self.get_net_production_rates(rho, t, y)
        h_rt = self.get_species_enthalpies_rt(t)
        cp = self.get_mixture_specific_heat_cp_mass(t, y)
        tdot = -(self.gas_constant * t * (h_rt * w).sum(axis=0)) / (rho * cp)
        ydot = self.tab.W[:, None] * w / rho
        return np.concatenate([tdot[None, :], ydot], axis=0)

    def reactor_jacobian_fd(self, p, t, y, rel=1e-7, absolute_y=False):
        """Central differences of :meth:`reactor_source` w.r.t. ``(T, Y)``;
        ``[N, S+1, S+1]``.  Steps: ``rel * T`` for T; ``rel * max(|Y|,
        1e-10)`` for Y, or ``rel`` itself with *absolute_y* (the
        reference's mass-fraction steps, ``test/test.py:349-356``)."""
        t = np.atleast_1d(np.asarray(t, dtype=np.float64))
        y = np.asarray(y, dtype=np.float64).reshape(self.tab.S, -1)
        x = np.concatenate([t[None, :], y], axis=0)
        n1, n = x.shape
        jac = np.empty((n, n1, n1))
        for i in range(n1):
            if absolute_y and i > 0:
                h = np.full(n, float(rel))
            else:
                h = rel * np.maximum(np.abs(x[i]), 1e-10)
            xp, xm = x.copy(), x.copy()
            xp[i] += h
            xm[i] -= h
            fp = self.reactor_source(p, xp[0], xp[1:])
            fm = self.reactor_source(p, xm[0], xm[1:])
            jac[:, :, i] = ((fp - fm) / (2 * h)).T
        return jac

    # }}}

# vim: foldmethod=marker
