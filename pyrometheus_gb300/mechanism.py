"""Mechanism object model: the subset of Cantera's ``Solution`` API that the
pyrometheus code generators read.

The reference generators take a ``cantera.Solution`` and query it through a
small, fixed surface (``pyrometheus/codegen/python.py:155-199,657-687``,
``pyrometheus/chem_expr.py:51-567``):

* ``sol.species()`` -> objects with ``.name``, ``.composition`` and
  ``.thermo.coeffs`` packed ``[Tmid, hi(7), lo(7)]`` (``chem_expr.py:51-57``);
* ``sol.reactions()`` / ``sol.reaction(i)`` -> objects with ``.equation``,
  ``.reactants``, ``.products``, ``.orders``, ``.reversible``,
  ``.reaction_type`` (``"Arrhenius"``, ``"three-body-Arrhenius"``,
  ``"falloff-Troe"``, ``"falloff-Lindemann"``), ``.rate`` and
  ``.third_body``;
* ``sol.species_index``, ``sol.reactant_stoich_coeff``,
  ``sol.product_stoich_coeff``, ``sol.molecular_weights``, ``sol.n_*``.

This module provides exactly that surface from plain Python data, so the CUDA
generator accepts either a real ``cantera.Solution`` (when Cantera is
installed) or a :class:`Solution` built by :mod:`pyrometheus_gb300.yaml_mech`
or :mod:`pyrometheus_gb300.synthetic`.  All quantities are SI with kmol:
``A`` in (m^3/kmol)^(order-1)/s, activation energies in J/kmol, molecular
weights in kg/kmol.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Union

import numpy as np

#: Molar gas constant in J/(kmol K) (CODATA 2018 exact value, the value
#: Cantera exports as ``ct.gas_constant``).
gas_constant = 8314.46261815324
#: One standard atmosphere in Pa (``ct.one_atm``).
one_atm = 101325.0

#: Standard atomic weights (kg/kmol) for the elements the fixture and
#: synthetic mechanisms use; the same abridged IUPAC values Cantera tabulates.
ATOMIC_WEIGHTS: Dict[str, float] = {
    "H": 1.008,
    "He": 4.002602,
    "C": 12.011,
    "N": 14.007,
    "O": 15.999,
    "Ar": 39.95,
    "AR": 39.95,
    "E": 5.48579909065e-4,
}


def element_weight(symbol: str) -> float:
    try:
        return ATOMIC_WEIGHTS[symbol]
    except KeyError:
        cap = symbol.capitalize()
        if cap in ATOMIC_WEIGHTS:
            return ATOMIC_WEIGHTS[cap]
        raise KeyError(f"no atomic weight for element '{symbol}'") from None


class NasaPoly2:
    """Two-range NASA-7 polynomial; ``coeffs = [Tmid, hi(7), lo(7)]``
    (the packing ``chem_expr.py:53-57`` indexes)."""

    def __init__(self, t_low: float, t_mid: float, t_high: float,
                 low: Sequence[float], high: Sequence[float]):
        low = [float(v) for v in low]
        high = [float(v) for v in high]
        if len(low) != 7 or len(high) != 7:
            raise ValueError("NASA-7 ranges need 7 coefficients each")
        self.min_temp = float(t_low)
        self.max_temp = float(t_high)
        self.coeffs = np.array([float(t_mid)] + high + low, dtype=np.float64)

    @property
    def t_mid(self) -> float:
        return float(self.coeffs[0])

    @property
    def high(self) -> np.ndarray:
        return self.coeffs[1:8]

    @property
    def low(self) -> np.ndarray:
        return self.coeffs[8:15]


class Species:
    def __init__(self, name: str, composition: Dict[str, float],
                 thermo: NasaPoly2):
        self.name = name
        self.composition = dict(composition)
        self.thermo = thermo
        self.molecular_weight = float(sum(
            n * element_weight(el) for el, n in self.composition.items()))

    def __repr__(self):
        return f"<Species {self.name}>"


class Arrhenius:
    """Modified Arrhenius ``k = A T^b exp(-Ea/(R T))`` (SI, J/kmol)."""

    type = "Arrhenius"

    def __init__(self, A: float, b: float, Ea: float):
        self.pre_exponential_factor = float(A)
        self.temperature_exponent = float(b)
        self.activation_energy = float(Ea)

    def __call__(self, T):
        return (self.pre_exponential_factor * T ** self.temperature_exponent
                * np.exp(-self.activation_energy / (gas_constant * T)))


#: Cantera 3 names the elementary rate object ``ArrheniusRate``.
ArrheniusRate = Arrhenius


class FalloffRate:
    type = "falloff"

    def __init__(self, low: Arrhenius, high: Arrhenius,
                 falloff_coeffs: Sequence[float] = ()):
        self.low_rate = low
        self.high_rate = high
        self.falloff_coeffs = np.array([float(v) for v in falloff_coeffs],
                                       dtype=np.float64)


class LindemannRate(FalloffRate):
    type = "Lindemann"

    def __init__(self, low: Arrhenius, high: Arrhenius,
                 falloff_coeffs: Sequence[float] = ()):
        super().__init__(low, high, ())


class TroeRate(FalloffRate):
    """Troe falloff; ``falloff_coeffs = [A, T3, T1]`` or ``[A, T3, T1, T2]``."""

    type = "Troe"

    def __init__(self, low: Arrhenius, high: Arrhenius,
                 falloff_coeffs: Sequence[float]):
        if len(falloff_coeffs) not in (3, 4):
            raise ValueError("Troe falloff needs 3 or 4 coefficients")
        super().__init__(low, high, falloff_coeffs)


@dataclass
class ThirdBody:
    efficiencies: Dict[str, float] = field(default_factory=dict)
    default_efficiency: float = 1.0


class Reaction:
    def __init__(self, equation: str, reactants: Dict[str, float],
                 products: Dict[str, float],
                 rate: Union[Arrhenius, FalloffRate],
                 reversible: bool = True,
                 orders: Optional[Dict[str, float]] = None,
                 third_body: Optional[ThirdBody] = None,
                 duplicate: bool = False):
        self.equation = equation
        self.reactants = dict(reactants)
        self.products = dict(products)
        self.rate = rate
        self.reversible = bool(reversible)
        self.orders = dict(orders) if orders else {}
        self.third_body = third_body
        self.duplicate = bool(duplicate)
        if isinstance(rate, FalloffRate):
            if third_body is None:
                raise ValueError(f"falloff reaction '{equation}' needs a "
                                 "third body")
            self.reaction_type = f"falloff-{rate.type}"
        elif third_body is not None:
            self.reaction_type = "three-body-Arrhenius"
        else:
            self.reaction_type = "Arrhenius"

    def __repr__(self):
        return f"<Reaction {self.equation}>"


class Solution:
    """Cantera-``Solution``-like container (immutable after construction)."""

    def __init__(self, species: List[Species], reactions: List[Reaction],
                 elements: Optional[List[str]] = None, source: str = "",
                 name: str = "gas", transport=None):
        self._species = list(species)
        #: :class:`pyrometheus_gb300.transport_fits.TransportFits` or None
        self.transport = transport
        self._reactions = list(reactions)
        self.species_names = [sp.name for sp in self._species]
        if len(set(self.species_names)) != len(self.species_names):
            raise ValueError("duplicate species names")
        self._index = {n: i for i, n in enumerate(self.species_names)}
        if elements is None:
            elements = []
            for sp in self._species:
                for el in sp.composition:
                    if el not in elements:
                        elements.append(el)
        self.element_names = list(elements)
        self.source = source
        self.name = name
        for r in self._reactions:
            for sp in (list(r.reactants) + list(r.products)
                       + list(r.orders)):
                if sp not in self._index:
                    raise ValueError(f"reaction '{r.equation}' names unknown "
                                     f"species '{sp}'")
        self.molecular_weights = np.array(
            [sp.molecular_weight for sp in self._species], dtype=np.float64)

    # -- counts -----------------------------------------------------------
    @property
    def n_species(self) -> int:
        return len(self._species)

    @property
    def n_reactions(self) -> int:
        return len(self._reactions)

    @property
    def n_elements(self) -> int:
        return len(self.element_names)

    # -- lookup -----------------------------------------------------------
    def species(self, k=None):
        if k is None:
            return list(self._species)
        if isinstance(k, str):
            k = self._index[k]
        return self._species[k]

    def reactions(self) -> List[Reaction]:
        return list(self._reactions)

    def reaction(self, i: int) -> Reaction:
        return self._reactions[i]

    def species_index(self, name: str) -> int:
        try:
            return self._index[name]
        except KeyError:
            raise ValueError(f"unknown species '{name}'") from None

    def species_name(self, k: int) -> str:
        return self.species_names[k]

    def _name(self, k) -> str:
        return k if isinstance(k, str) else self.species_names[k]

    def reactant_stoich_coeff(self, k, i: int) -> float:
        return float(self._reactions[i].reactants.get(self._name(k), 0.0))

    def product_stoich_coeff(self, k, i: int) -> float:
        return float(self._reactions[i].products.get(self._name(k), 0.0))

    # -- transport fits (Cantera's MixTransport surface) -------------------
    @property
    def transport_model(self) -> str:
        return "mixture-averaged" if self.transport is not None else "none"

    def _fits(self):
        if self.transport is None:
            raise ValueError(f"mechanism '{self.source or self.name}' has no "
                             "transport fits")
        return self.transport

    def get_viscosity_polynomial(self, k: int) -> np.ndarray:
        return np.array(self._fits().viscosity[k], dtype=np.float64)

    def get_thermal_conductivity_polynomial(self, k: int) -> np.ndarray:
        return np.array(self._fits().conductivity[k], dtype=np.float64)

    def get_binary_diff_coeffs_polynomial(self, i: int, j: int
                                          ) -> np.ndarray:
        return np.array(self._fits().diffusivity[i, j], dtype=np.float64)

    def n_atoms(self, species, element) -> float:
        """Atoms of *element* (index or name) in *species* (index or
        name), as Cantera's ``Solution.n_atoms``."""
        sp = self.species(species)
        el = element if isinstance(element, str) else \
            self.element_names[element]
        return float(sp.composition.get(el, 0.0))

    # -- convenience (not part of the Cantera surface) ---------------------
    def element_matrix(self) -> np.ndarray:
        """(n_elements, n_species) atom counts."""
        m = np.zeros((self.n_elements, self.n_species))
        for k, sp in enumerate(self._species):
            for el, n in sp.composition.items():
                m[self.element_names.index(el), k] = n
        return m
