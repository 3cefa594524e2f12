"""Mixture-averaged transport fits in the form the reference's generated
class evaluates (``pyrometheus/chem_expr.py:190-244``):

* viscosity            mu_k   = sqrt(T) * (sum_n a_kn (ln T)^n)^2
* thermal conductivity lam_k  = sqrt(T) *  sum_n b_kn (ln T)^n
* binary diffusivity   D_ij p = T^1.5   *  sum_n d_ijn (ln T)^n

(degree 4, coefficients in ascending order).  The reference reads them from
a Cantera ``Solution`` through ``get_viscosity_polynomial(k)``,
``get_thermal_conductivity_polynomial(k)`` and
``get_binary_diff_coeffs_polynomial(i, j)`` (``python.py:564-590``);
:class:`pyrometheus_gb300.mechanism.Solution` exposes the same three methods
over a :class:`TransportFits`.

Cantera derives its fits from Lennard-Jones parameters with tabulated
collision integrals and polar corrections; that procedure is not restated
here.  :func:`kinetic_theory_fits` makes seeded stand-in fits of the same
form and magnitude from first-order Chapman-Enskog kinetic theory:

* mu_k  = 2.6693e-6 sqrt(W_k T) / (sigma_k^2 Omega22(T/eps_k))        [Pa s]
* D_ij p = 1.8583e-7 * 101325 * sqrt(T^3 (1/W_i + 1/W_j))
          / (sigma_ij^2 Omega11(T/eps_ij)),  sigma_ij = (sigma_i+sigma_j)/2,
          eps_ij = sqrt(eps_i eps_j)                                   [Pa m^2/s]
* lam_k = mu_k (R/W_k) (cp_k/R + 5/4)  (modified Eucken)               [W/m/K]

with the collision integrals of Neufeld, Janzen and Aziz (J. Chem. Phys.
57, 1100, 1972) and sigma in Angstrom, W in kg/kmol; each property is then
fitted by least squares in ln T over the fit range, as Cantera fits its
tabulated values.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np

GAS_CONSTANT = 8314.46261815324
ONE_ATM = 101325.0


@dataclass(frozen=True)
class TransportFits:
    """Degree-4 fits in ln T: ``viscosity`` (S, 5), ``conductivity`` (S, 5)
    and ``diffusivity`` (S, S, 5)."""

    viscosity: np.ndarray
    conductivity: np.ndarray
    diffusivity: np.ndarray

    def __post_init__(self):
        s = self.viscosity.shape[0]
        if (self.viscosity.shape != (s, 5)
                or self.conductivity.shape != (s, 5)
                or self.diffusivity.shape != (s, s, 5)):
            raise ValueError("transport fits need shapes (S,5), (S,5), "
                             "(S,S,5)")

    @property
    def symmetric(self) -> bool:
        """Whether D_ij and D_ji share one fit (true of Cantera's fits)."""
        return bool(np.array_equal(self.diffusivity,
                                   self.diffusivity.transpose(1, 0, 2)))


def omega22(tstar):
    """Reduced collision integral Omega(2,2)* (Neufeld et al. 1972)."""
    t = np.asarray(tstar, dtype=np.float64)
    return (1.16145 * t ** -0.14874 + 0.52487 * np.exp(-0.77320 * t)
            + 2.16178 * np.exp(-2.43787 * t))


def omega11(tstar):
    """Reduced collision integral Omega(1,1)* (Neufeld et al. 1972)."""
    t = np.asarray(tstar, dtype=np.float64)
    return (1.06036 * t ** -0.15610 + 0.19300 * np.exp(-0.47635 * t)
            + 1.03587 * np.exp(-1.52996 * t)
            + 1.76474 * np.exp(-3.89411 * t))


def _cp_r(thermo, t):
    c = thermo.coeffs
    a = np.where(t[:, None] > c[0], c[1:6][None, :], c[8:13][None, :])
    return a[:, 0] + t * (a[:, 1] + t * (a[:, 2] + t * (a[:, 3]
                                                          + t * a[:, 4])))


def _fit(lnt, values) -> np.ndarray:
    return np.polynomial.polynomial.polyfit(lnt, values, 4)


def kinetic_theory_fits(sol, seed: int = 0,
                        t_range: Tuple[float, float] = (300.0, 3500.0),
                        sigma: Optional[Sequence[float]] = None,
                        well_depth: Optional[Sequence[float]] = None
                        ) -> TransportFits:
    """Seeded Lennard-Jones parameters (sigma in [2.5, 4.5] Angstrom,
    growing with atom count; eps/k in [40, 600] K) unless given, then
    Chapman-Enskog properties fitted in ln T on ``t_range``."""
    rng = np.random.default_rng(seed)
    species = sol.species()
    S = len(species)
    W = np.asarray(sol.molecular_weights, dtype=np.float64)
    if sigma is None:
        atoms = np.array([sum(sp.composition.values()) for sp in species])
        sigma = 2.5 + 2.0 * (1.0 - np.exp(-atoms / 4.0)) \
            + rng.uniform(-0.2, 0.2, S)
    if well_depth is None:
        well_depth = rng.uniform(40.0, 600.0, S)
    sigma = np.asarray(sigma, dtype=np.float64)
    eps = np.asarray(well_depth, dtype=np.float64)

    t = np.geomspace(t_range[0], t_range[1], 64)
    lnt = np.log(t)
    visc = np.zeros((S, 5))
    cond = np.zeros((S, 5))
    for k, sp in enumerate(species):
        mu = 2.6693e-6 * np.sqrt(W[k] * t) / (sigma[k] ** 2
                                                * omega22(t / eps[k]))
        lam = mu * (GAS_CONSTANT / W[k]) * (_cp_r(sp.thermo, t) + 1.25)
        visc[k] = _fit(lnt, np.sqrt(mu) / t ** 0.25)
        cond[k] = _fit(lnt, lam / np.sqrt(t))
    diff = np.zeros((S, S, 5))
    for i in range(S):
        for j in range(i, S):
            sij = 0.5 * (sigma[i] + sigma[j])
            eij = np.sqrt(eps[i] * eps[j])
            dp = (1.8583e-7 * ONE_ATM
                  * np.sqrt(t ** 3 * (1.0 / W[i] + 1.0 / W[j]))
                  / (sij ** 2 * omega11(t / eij)))
            diff[i, j] = diff[j, i] = _fit(lnt, dp / t ** 1.5)
    return TransportFits(visc, cond, diff)
