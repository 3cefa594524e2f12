"""Set-up helpers for flamelet problems, as in
``pyrometheus/flamelets/utils.py``: the dissipation-rate shape and the
stoichiometric mixture fraction of a fuel/oxidizer pair.  Host code
(numpy/scipy); the inputs they make go to
:class:`~pyrometheus_gb300.flamelet_solver.FlameletSolver`."""

from __future__ import annotations

import numpy as np
from scipy.special import erfcinv

# Bilger coupling weights per element and the element weights the reference
# uses with them (``utils.py:50-100``); elements not listed weigh nothing.
_BILGER = {"C": 2.0, "H": 0.5, "O": -1.0}
_ELEMENT_WEIGHTS = {"C": 12.011, "H": 1.00794, "O": 15.999, "Ar": 39.948,
                    "N": 28.0133}


def bell_profile(z):
    """``exp(-2 erfcinv(2 z)^2)``: the counterflow shape of the scalar
    dissipation rate over the mixture fraction (``utils.py:9-27``); 1 at
    z = 1/2."""
    return np.exp(-2.0 * erfcinv(2.0 * np.asarray(z, dtype=np.float64)) ** 2)


def stoichiometric_mixture_fraction(sol, y_ox, y_fu):
    """Bilger's stoichiometric mixture fraction ``-b_ox / (b_fu - b_ox)``
    of the oxidizer and fuel mass fractions *y_ox*, *y_fu*
    (``utils.py:30-100``): ``b = sum_e w_e sum_k n_ek (W_e / W_k) Y_k`` with
    ``w_C = 2 / W_C``, ``w_H = 1 / (2 W_H)``, ``w_O = -1 / W_O``.  *sol*
    gives ``element_names``, ``molecular_weights`` and ``n_atoms``."""
    names = list(sol.element_names)
    w_s = np.asarray(sol.molecular_weights, dtype=np.float64)
    bilger = np.array([_BILGER[e] / _ELEMENT_WEIGHTS[e] if e in _BILGER
                       else 0.0 for e in names])
    elem = np.zeros((len(names), len(w_s)))
    for e, name in enumerate(names):
        for k in range(len(w_s)):
            elem[e, k] = sol.n_atoms(k, e) * (_ELEMENT_WEIGHTS[name]
                                              / w_s[k])
    beta_ox = bilger.dot(elem.dot(np.asarray(y_ox, dtype=np.float64)))
    beta_fu = bilger.dot(elem.dot(np.asarray(y_fu, dtype=np.float64)))
    return -beta_ox / (beta_fu - beta_ox)


def burke_schumann(sol, z, y_ox, y_fu, fuel=None):
    """Mass fractions ``[S, len(z)]`` of the Burke-Schumann flamelet
    (infinitely fast, complete one-step combustion) over the mixture
    fraction *z*: the mixing line ``(1 - z) y_ox + z y_fu`` with the fuel
    and O2 consumed together -- ``fuel + nu O2 -> a CO2 + b/2 H2O`` for a
    fuel C_a H_b O_c, ``nu = a + b/4 - c/2`` -- as far as the scarcer of the
    two allows (all the fuel on the lean side, all the O2 on the rich
    side).  *fuel* defaults to the fuel stream's most abundant species
    other than N2, Ar, He and O2.  The customary starting guess of a
    burning steady flamelet (the reference's notebook starts from
    equilibrium compositions, which need Cantera's solver)."""
    names = list(sol.species_names)
    w = np.asarray(sol.molecular_weights, dtype=np.float64)
    y_ox = np.asarray(y_ox, dtype=np.float64)
    y_fu = np.asarray(y_fu, dtype=np.float64)
    if fuel is None:
        skip = {"N2", "AR", "Ar", "HE", "He", "O2"}
        cand = [(y_fu[k], k) for k, n in enumerate(names) if n not in skip]
        fuel = names[max(cand)[1]]
    kf = names.index(fuel)
    ko = names.index("O2")
    el = list(sol.element_names)

    def atoms(e):
        return sol.n_atoms(kf, el.index(e)) if e in el else 0.0

    a, b, c = atoms("C"), atoms("H"), atoms("O")
    nu = a + b / 4.0 - c / 2.0
    z = np.asarray(z, dtype=np.float64)
    y = (1.0 - z)[None, :] * y_ox[:, None] + z[None, :] * y_fu[:, None]
    # moles per unit mass of fuel and O2 available, and how much burns
    n_f = y[kf] / w[kf]
    n_o = y[ko] / w[ko]
    burnt = np.minimum(n_f, n_o / nu)
    y[kf] -= burnt * w[kf]
    y[ko] -= nu * burnt * w[ko]
    for name, count in (("CO2", a), ("H2O", b / 2.0)):
        if count:
            y[names.index(name)] += count * burnt * w[names.index(name)]
    return np.maximum(y, 0.0)
