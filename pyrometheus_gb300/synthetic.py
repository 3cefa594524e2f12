"""Seeded synthetic mechanisms and thermochemical states.

The benchmark workloads are defined on synthetic Cantera-YAML mechanisms with
the shapes of the reference's fixture mechanisms (``test/mechs/sandiego.yaml``:
9 species / 24 reactions; ``test/mechs/gri30.yaml``: 53 species / 325
reactions), generated here from a seed:

* species are real chemical formulas over the requested elements, so element
  balance (and hence mass conservation of the production rates) is
  meaningful;
* NASA-7 fits: each species gets a smooth heat capacity rising from about
  2.5 to at most 7 (cp/R) over 300-3500 K; the low range is a least-squares
  quartic on [300, 1000] K and the high range a quartic on [1000, 3500] K that
  is C0/C1-continuous with it at 1000 K; the enthalpy and entropy
  integration constants (a5, a6) put a random formation enthalpy and
  standard entropy at 298.15 K and make h and s continuous at 1000 K;
* reactions are enumerated from element-balanced combinations:
  ``A + B <=> C + D`` (elementary) and ``A + M <=> B + C`` (three-body, with
  random efficiencies in [0.5, 12]) / ``A (+ M) <=> B + C`` (Troe or
  Lindemann falloff);
* Arrhenius parameters: ``A`` log-uniform in [1e6, 1e16] in cm-mol-s units
  (converted to SI by reaction order), ``b ~ U[-2, 2]``,
  ``Ea ~ U[0, 60]`` kcal/mol.  One reaction in eight (and every falloff
  low-pressure limit with probability 1/2) gets ``Ea = 0`` so the
  ``A*T**b`` branch of the reference (``chem_expr.py:319-321``) is
  exercised;
* orientation: with ``orient_temperature`` set (the benchmark mechanisms use
  1500 K), each reaction is written in the direction whose standard Gibbs
  energy change at that temperature is negative.  The random formation
  enthalpies span about 1e5 R, so a reaction written uphill has an
  equilibrium constant near e^-100 and a reverse rate coefficient
  ``k_f / K_c`` tens of decades above any forward one; a 0-D reactor on
  such a mechanism has time scales below 1e-30 s and cannot be integrated.
  Written downhill, ``k_r`` stays within a few decades of ``k_f``.

States: ``T ~ U[300, 3000]`` K, ``p`` log-uniform in [1e4, 1e6] Pa and
``Y = 0.6 e_N2 + 0.4 Dirichlet(0.5)`` (the "N2 floor of 0.6").
"""

from __future__ import annotations

import itertools
import re
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .mechanism import (Arrhenius, LindemannRate, NasaPoly2, Reaction,
                        Solution, Species, ThirdBody, TroeRate, gas_constant)
from .transport_fits import kinetic_theory_fits

#: H/O/N/Ar set with the sandiego shape (9 species).
SPECIES_9 = ["H2", "H", "O2", "O", "OH", "HO2", "H2O", "N2", "AR"]

#: C/H/O/N/Ar formulas with the gri30 shape (53 species).
SPECIES_53 = [
    "H2", "H", "O", "O2", "OH", "H2O", "HO2", "H2O2", "C", "CH", "CH2",
    "CH2(S)", "CH3", "CH4", "CO", "CO2", "HCO", "CH2O", "CH2OH", "CH3O",
    "CH3OH", "C2H", "C2H2", "C2H3", "C2H4", "C2H5", "C2H6", "HCCO", "CH2CO",
    "HCCOH", "N", "NH", "NH2", "NH3", "NNH", "NO", "NO2", "N2O", "HNO", "CN",
    "HCN", "H2CN", "HCNN", "HCNO", "HOCN", "HNCO", "NCO", "N2", "AR", "C3H7",
    "C3H8", "CH2CHO", "CH3CHO",
]

_CAL = 4184.0          # J/kmol per cal/mol
_T_LOW, _T_MID, _T_HIGH, _T_REF = 300.0, 1000.0, 3500.0, 298.15


def formula_composition(name: str) -> Dict[str, float]:
    """Element counts of a formula such as ``CH2CHO``; a trailing isomer tag
    in parentheses (``CH2(S)``) is ignored and ``AR`` means argon."""
    base = re.sub(r"\([^)]*\)$", "", name)
    if base.upper() == "AR":
        return {"Ar": 1.0}
    comp: Dict[str, float] = {}
    for el, cnt in re.findall(r"([A-Z][a-z]?)(\d*)", base):
        comp[el] = comp.get(el, 0.0) + (float(cnt) if cnt else 1.0)
    return comp


def _comp_key(comp: Dict[str, float]) -> Tuple:
    return tuple(sorted((k, v) for k, v in comp.items() if v))


def _add(a: Dict[str, float], b: Dict[str, float]) -> Dict[str, float]:
    out = dict(a)
    for k, v in b.items():
        out[k] = out.get(k, 0.0) + v
    return out


# {{{ thermo

def _nasa_fit(rng: np.random.Generator, n_atoms: int) -> NasaPoly2:
    """Random smooth cp/R(T) -> C0/C1-continuous two-range NASA-7 fit."""
    if n_atoms == 1:
        cp_max = rng.uniform(2.5, 3.0)
    else:
        cp_max = rng.uniform(3.5 + 0.5 * min(n_atoms, 4), 7.0)
    cp_min = rng.uniform(2.5, min(3.5 + 0.25 * n_atoms, cp_max))
    width = rng.uniform(400.0, 1500.0)

    def cp(t):
        x = (np.asarray(t) - _T_LOW) / width
        return cp_min + (cp_max - cp_min) * (1.0 - np.exp(-x)) \
            / (1.0 - np.exp(-(_T_HIGH - _T_LOW) / width))

    # low range: least squares quartic on [300, 1000]
    tl = np.linspace(_T_LOW, _T_MID, 64)
    low = np.polynomial.polynomial.polyfit(tl, cp(tl), 4)
    # high range: value and slope matched at Tmid, quadratic..quartic in
    # (T - Tmid) fitted by least squares on [1000, 3500]
    p_low = np.polynomial.Polynomial(low)
    v0, d0 = p_low(_T_MID), p_low.deriv()(_T_MID)
    th = np.linspace(_T_MID, _T_HIGH, 96)
    u = th - _T_MID
    resid = cp(th) - (v0 + d0 * u)
    basis = np.stack([u ** 2, u ** 3, u ** 4], axis=1)
    c234, *_ = np.linalg.lstsq(basis, resid, rcond=None)
    shifted = np.polynomial.Polynomial([v0, d0, *c234])
    # expand the (T - Tmid) polynomial into monomials of T
    high = np.zeros(5)
    for k, ck in enumerate(shifted.coef):
        for j in range(k + 1):
            high[j] += ck * _binom(k, j) * (-_T_MID) ** (k - j)

    # integration constants: formation enthalpy and entropy at 298.15 K
    if n_atoms == 1:
        hf_r = rng.uniform(25000.0, 90000.0)
    else:
        hf_r = rng.uniform(-45000.0, 45000.0)
    s0_r = rng.uniform(15.0, 35.0)

    def h_r(a, t):  # h/R without the a5 constant
        return (a[0] * t + a[1] * t ** 2 / 2 + a[2] * t ** 3 / 3
                + a[3] * t ** 4 / 4 + a[4] * t ** 5 / 5)

    def s_r(a, t):  # s/R without the a6 constant
        return (a[0] * np.log(t) + a[1] * t + a[2] * t ** 2 / 2
                + a[3] * t ** 3 / 3 + a[4] * t ** 4 / 4)

    a5_lo = hf_r - h_r(low, _T_REF)
    a6_lo = s0_r - s_r(low, _T_REF)
    a5_hi = h_r(low, _T_MID) + a5_lo - h_r(high, _T_MID)
    a6_hi = s_r(low, _T_MID) + a6_lo - s_r(high, _T_MID)
    return NasaPoly2(_T_LOW, _T_MID, _T_HIGH,
                     list(low) + [a5_lo, a6_lo],
                     list(high) + [a5_hi, a6_hi])


def _binom(n: int, k: int) -> float:
    from math import comb
    return float(comb(n, k))

# }}}


# {{{ reactions

def _arrhenius(rng, order: float, zero_ea: bool) -> Arrhenius:
    a_cgs = 10.0 ** rng.uniform(6.0, 16.0)
    a_si = a_cgs * (1e-3) ** (order - 1.0)
    b = rng.uniform(-2.0, 2.0)
    ea = 0.0 if zero_ea else rng.uniform(0.0, 60.0) * 1000.0 * _CAL
    return Arrhenius(a_si, b, ea)


def _side(d: Dict[str, float]) -> str:
    parts = []
    for k, v in d.items():
        parts.append(k if v == 1 else f"{int(v) if float(v).is_integer() else v} {k}")
    return " + ".join(parts)


def _efficiencies(rng, names: Sequence[str]) -> Dict[str, float]:
    k = int(rng.integers(1, min(6, len(names)) + 1))
    picks = rng.choice(len(names), size=k, replace=False)
    return {names[i]: float(np.round(rng.uniform(0.5, 12.0), 3))
            for i in sorted(picks)}


def enumerate_exchanges(names: Sequence[str],
                        comps: Sequence[Dict[str, float]]):
    """All element-balanced ``A + B <=> C + D`` with disjoint sides."""
    pairs: Dict[Tuple, List[Tuple[int, int]]] = {}
    for i, j in itertools.combinations_with_replacement(range(len(names)), 2):
        key = _comp_key(_add(comps[i], comps[j]))
        pairs.setdefault(key, []).append((i, j))
    out = []
    for group in pairs.values():
        for p, q in itertools.combinations(group, 2):
            if set(p) & set(q):
                continue
            out.append((p, q))
    return out


def enumerate_dissociations(names: Sequence[str],
                            comps: Sequence[Dict[str, float]]):
    """All element-balanced ``A <=> B + C`` (B, C may coincide)."""
    by_key: Dict[Tuple, List[int]] = {}
    for i, c in enumerate(comps):
        by_key.setdefault(_comp_key(c), []).append(i)
    out = []
    for i, j in itertools.combinations_with_replacement(range(len(names)), 2):
        key = _comp_key(_add(comps[i], comps[j]))
        for a in by_key.get(key, []):
            if a not in (i, j):
                out.append((a, (i, j)))
    return out


def _pick(rng, n_avail: int, n_want: int) -> np.ndarray:
    picks = [rng.permutation(n_avail)[:n_want]]
    while sum(len(p) for p in picks) < n_want:
        picks.append(rng.permutation(n_avail)[
            :n_want - sum(len(p) for p in picks)])
    return np.concatenate(picks)


def _gibbs_rt(thermo: NasaPoly2, t: float) -> float:
    """g/RT of one species from its NASA-7 fit."""
    a = thermo.high if t > thermo.t_mid else thermo.low
    h_rt = (a[0] + a[1] * t / 2 + a[2] * t ** 2 / 3 + a[3] * t ** 3 / 4
            + a[4] * t ** 4 / 5 + a[5] / t)
    s_r = (a[0] * np.log(t) + a[1] * t + a[2] * t ** 2 / 2
           + a[3] * t ** 3 / 3 + a[4] * t ** 4 / 4 + a[6])
    return float(h_rt - s_r)


def make_mechanism(species_names: Sequence[str], n_reactions: int,
                   n_three_body: int, n_troe: int, n_lindemann: int = 0,
                   seed: int = 0, irreversible_fraction: float = 0.0,
                   inert: Sequence[str] = ("AR",),
                   name: str = "synthetic",
                   orient_temperature: Optional[float] = None) -> Solution:
    """Seeded synthetic mechanism (see the module docstring)."""
    rng = np.random.default_rng(seed)
    names = list(species_names)
    comps = [formula_composition(n) for n in names]
    species = []
    for n, c in zip(names, comps):
        species.append(Species(n, c, _nasa_fit(rng, int(sum(c.values())))))
    g_rt = {sp.name: (_gibbs_rt(sp.thermo, orient_temperature)
                      if orient_temperature else 0.0) for sp in species}

    def downhill(reac, prod):
        """(reac, prod) swapped if the reaction is uphill in g at the
        orientation temperature."""
        if orient_temperature is None:
            return reac, prod
        dg = (sum(v * g_rt[k] for k, v in prod.items())
              - sum(v * g_rt[k] for k, v in reac.items()))
        return (prod, reac) if dg > 0 else (reac, prod)
    elements = []
    for c in comps:
        for el in c:
            if el not in elements:
                elements.append(el)

    reactive = [i for i, n in enumerate(names) if n not in inert]
    r_names = [names[i] for i in reactive]
    r_comps = [comps[i] for i in reactive]
    exch = enumerate_exchanges(r_names, r_comps)
    diss = enumerate_dissociations(r_names, r_comps)
    n_diss = n_three_body + n_troe + n_lindemann
    n_exch = n_reactions - n_diss
    if (n_diss and not diss) or (n_exch and not exch):
        raise ValueError("no balanced combinations for the request")
    # distinct combinations first; small species sets repeat combinations
    # (with fresh rate parameters, flagged ``duplicate`` like the duplicate
    # reactions of the fixture mechanisms)
    d_pick = _pick(rng, len(diss), n_diss)
    e_pick = _pick(rng, len(exch), n_exch)
    kinds = (["three-body"] * n_three_body + ["troe"] * n_troe
             + ["lindemann"] * n_lindemann)
    rng.shuffle(kinds)

    def spec(idx_list):
        d: Dict[str, float] = {}
        for i in idx_list:
            d[r_names[i]] = d.get(r_names[i], 0.0) + 1.0
        return d

    reactions: List[Reaction] = []
    for kind, di in zip(kinds, d_pick):
        a, (b, c) = diss[di]
        # recombination direction half the time
        if rng.random() < 0.5:
            reac, prod = spec([a]), spec([b, c])
        else:
            reac, prod = spec([b, c]), spec([a])
        reac, prod = downhill(reac, prod)
        order = sum(reac.values())
        eff = _efficiencies(rng, names)
        if kind == "three-body":
            eq = f"{_side(reac)} + M <=> {_side(prod)} + M"
            rate = _arrhenius(rng, order + 1.0, rng.random() < 0.125)
            reactions.append(Reaction(eq, reac, prod, rate, True, None,
                                      ThirdBody(eff, 1.0)))
        else:
            eq = f"{_side(reac)} (+ M) <=> {_side(prod)} (+ M)"
            high = _arrhenius(rng, order, rng.random() < 0.125)
            low = _arrhenius(rng, order + 1.0, rng.random() < 0.5)
            if kind == "troe":
                coeffs = [float(np.round(rng.uniform(0.1, 0.9), 4)),
                          float(np.round(10 ** rng.uniform(1.5, 3.0), 1)),
                          float(np.round(10 ** rng.uniform(2.8, 4.5), 1))]
                if rng.random() < 0.6:
                    coeffs.append(float(np.round(10 ** rng.uniform(3.0, 4.2),
                                                 1)))
                rate = TroeRate(low, high, coeffs)
            else:
                rate = LindemannRate(low, high)
            reactions.append(Reaction(eq, reac, prod, rate, True, None,
                                      ThirdBody(eff, 1.0)))
    for ei in e_pick:
        p, q = exch[ei]
        reac, prod = downhill(spec(p), spec(q))
        reversible = not (rng.random() < irreversible_fraction)
        arrow = "<=>" if reversible else "=>"
        eq = f"{_side(reac)} {arrow} {_side(prod)}"
        rate = _arrhenius(rng, sum(reac.values()), rng.random() < 0.125)
        reactions.append(Reaction(eq, reac, prod, rate, reversible))
    order = rng.permutation(len(reactions))
    reactions = [reactions[i] for i in order]
    # mark repeated equations as duplicates, as Cantera requires
    seen: Dict[Tuple, List[Reaction]] = {}
    for r in reactions:
        key = (_comp_key(r.reactants), _comp_key(r.products),
               r.reaction_type)
        seen.setdefault(key, []).append(r)
    for group in seen.values():
        if len(group) > 1:
            for r in group:
                r.duplicate = True
    sol = Solution(species, reactions, elements, source=f"{name}.yaml",
                   name="gas")
    # transport fits from their own generator, so the kinetics above do not
    # depend on whether fits are made
    sol.transport = kinetic_theory_fits(sol, seed=seed + 7919)
    return sol


def scaled_rates(sol: Solution, factor: float) -> Solution:
    """The mechanism with every rate coefficient multiplied by *factor*
    (the pre-exponential factors of every Arrhenius expression, both limits
    of a falloff reaction, so the falloff blending is unchanged); species,
    thermo, stoichiometry and transport fits are shared.  A small factor
    gives slow chemistry, e.g. flamelet operators dominated by diffusion."""
    def arr(a):
        return Arrhenius(a.pre_exponential_factor * factor,
                         a.temperature_exponent, a.activation_energy)

    reactions = []
    for r in sol.reactions():
        rate = r.rate
        if isinstance(rate, TroeRate):
            rate = TroeRate(arr(rate.low_rate), arr(rate.high_rate),
                            rate.falloff_coeffs)
        elif isinstance(rate, LindemannRate):
            rate = LindemannRate(arr(rate.low_rate), arr(rate.high_rate))
        else:
            rate = arr(rate)
        reactions.append(Reaction(r.equation, r.reactants, r.products, rate,
                                  r.reversible, r.orders, r.third_body,
                                  r.duplicate))
    out = Solution(sol.species(), reactions, sol.element_names,
                   source=sol.source, name=sol.name,
                   transport=sol.transport)
    return out


def config1_mechanism(seed: int = 1) -> Solution:
    """9 species (H, O, N, Ar) / 24 reversible reactions: 3 three-body,
    2 Troe falloff, 19 elementary; written downhill at 1500 K."""
    return make_mechanism(SPECIES_9, 24, 3, 2, 0, seed=seed,
                          name="synthetic9", orient_temperature=1500.0)


def config2_mechanism(seed: int = 2) -> Solution:
    """53 species (C, H, O, N, Ar) / 325 reactions: 30 three-body, 25 Troe,
    3 Lindemann, 267 elementary; written downhill at 1500 K."""
    return make_mechanism(SPECIES_53, 325, 30, 25, 3, seed=seed,
                          name="synthetic53", orient_temperature=1500.0)

# }}}


# {{{ states

def sample_states(sol: Solution, n: int, seed: int = 0,
                  t_range=(300.0, 3000.0), p_range=(1e4, 1e6),
                  n2_floor: float = 0.6, alpha: float = 0.5,
                  dilute: str = "N2"):
    """Seeded states ``(T[n], p[n], Y[S, n])`` (float64, species-major)."""
    rng = np.random.default_rng(seed)
    t = rng.uniform(t_range[0], t_range[1], size=n)
    p = np.exp(rng.uniform(np.log(p_range[0]), np.log(p_range[1]), size=n))
    y = rng.dirichlet(np.full(sol.n_species, alpha), size=n).T * (
        1.0 - n2_floor)
    y[sol.species_index(dilute)] += n2_floor
    return t, p, np.ascontiguousarray(y)


def density(sol: Solution, p, t, y):
    """Ideal-gas density ``p W / (R T)`` with ``1/W = sum_k Y_k / W_k``."""
    inv_w = (y / sol.molecular_weights[:, None]).sum(axis=0)
    return p / (gas_constant * t * inv_w)

# }}}

# vim: foldmethod=marker


# {{{ flamelets

def flamelet_profiles(sol: Solution, lengths, seed: int = 0,
                      chi_max: float = 10.0, t_peak: float = 2000.0):
    """Seeded steady-flamelet initial states on uniform mixture-fraction
    grids, packed along rows: oxidizer Y = (O2 0.233, N2 0.767), fuel
    Y = (H2 0.1, N2 0.9), linear mixing plus 1e-3 of seeded radical
    fractions inside, a hot layer T = 300 + (t_peak - 300)
    exp(-((Z - Z_p) / 0.15)^2) around a seeded Z_p in [0.2, 0.4], and a
    dissipation rate chi = chi_max exp(-((Z - 0.5) / 0.3)^2).

    Returns a dict with ``Y`` [S, rows], ``T`` [rows] (temperature profile;
    the caller turns it into the enthalpy unknown), ``chi`` [rows],
    ``dx`` [n_flamelets], ``y_ox``, ``y_fu`` [S]."""
    rng = np.random.default_rng(seed)
    S = sol.n_species
    idx = sol.species_index
    y_ox = np.zeros(S)
    y_ox[idx("O2")], y_ox[idx("N2")] = 0.233, 0.767
    y_fu = np.zeros(S)
    y_fu[idx("H2")], y_fu[idx("N2")] = 0.1, 0.9
    ys, ts, chis, dxs = [], [], [], []
    for n in np.asarray(lengths, dtype=np.int64):
        n = int(n)
        z = np.linspace(0.0, 1.0, n)
        y = (1.0 - z)[None, :] * y_ox[:, None] + z[None, :] * y_fu[:, None]
        noise = 1e-3 * rng.dirichlet(np.full(S, 0.5), size=n).T
        y[:, 1:-1] += noise[:, 1:-1]
        y /= y.sum(axis=0, keepdims=True)
        zp = rng.uniform(0.2, 0.4)
        ts.append(300.0 + (t_peak - 300.0) * np.exp(-((z - zp) / 0.15) ** 2))
        chis.append(chi_max * np.exp(-((z - 0.5) / 0.3) ** 2))
        ys.append(y)
        dxs.append(1.0 / (n - 1))
    return dict(Y=np.hstack(ys), T=np.concatenate(ts),
                chi=np.concatenate(chis), dx=np.asarray(dxs), y_ox=y_ox,
                y_fu=y_fu)

# }}}
