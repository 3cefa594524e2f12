"""The oracle against the reference's generator run live on the reference's
own fixture mechanisms (``test/mechs/*.yaml``).  Skipped where the reference
checkout is not present (it never is on a GPU host)."""

import os

import numpy as np
import pytest

from conftest import rel_err
from oracle import refgen
from oracle.thermo_oracle import Thermochemistry as Oracle
from pyrometheus_gb300 import synthetic
from pyrometheus_gb300.yaml_mech import load_mechanism

pytestmark = pytest.mark.skipif(not refgen.reference_available(),
                                reason="reference checkout not present")

MECHS = ["uiuc", "sandiego", "hong", "uconn32", "gri30"]


def _load(name):
    path = os.path.join(refgen.REFERENCE_ROOT, "test", "mechs",
                        f"{name}.yaml")
    try:
        return load_mechanism(path, "gas")
    except ValueError:
        return load_mechanism(path)


@pytest.mark.parametrize("mech", MECHS)
def test_oracle_matches_reference_generator(mech):
    sol = _load(mech)
    ref = refgen.reference_class(sol)()
    o = Oracle(sol)
    n = 64
    dil = "N2" if "N2" in sol.species_names else sol.species_names[-1]
    t, p, y = synthetic.sample_states(sol, n, seed=21, dilute=dil)
    rho = o.get_density(p, t, y)
    c = o.get_concentrations(rho, y)

    def arr(x):
        return np.array([np.broadcast_to(np.asarray(v, float), (n,))
                         for v in x])

    assert rel_err(o.get_fwd_rate_coefficients(t, c),
                   arr(ref.get_fwd_rate_coefficients(t, c))) < 1e-13
    cd, dd = o.get_creation_destruction_rates(rho, t, y)
    assert rel_err(o.get_net_production_rates(rho, t, y),
                   arr(ref.get_net_production_rates(rho, t, y)),
                   cd + dd) < 1e-13
    e = o.get_mixture_internal_energy_mass(t, y)
    assert np.abs(o.get_temperature(e, 1500.0, y, True)
                  - ref.get_temperature(e, 1500.0, y, True)).max() < 1e-10


@pytest.mark.parametrize("mech", ["sandiego", "gri30"])
def test_oracle_transport_matches_reference_generator(mech):
    """The reference's generated transport methods (python.py:564-641) on
    its own fixture mechanisms, with kinetic-theory fits from their
    Lennard-Jones data, against the oracle."""
    path = os.path.join(refgen.REFERENCE_ROOT, "test", "mechs",
                        f"{mech}.yaml")
    sol = load_mechanism(path, transport="kinetic-theory")
    ref = refgen.reference_class(sol)()
    o = Oracle(sol)
    n = 32
    t, p, y = synthetic.sample_states(sol, n, seed=22, dilute="N2")

    def dense(a):
        a = np.asarray(a)
        if a.dtype == object:
            return np.array([dense(v) for v in a])
        return a.astype(np.float64)

    assert np.array_equal(o.get_species_viscosities(t),
                          dense(ref.get_species_viscosities(t)))
    assert np.array_equal(o.get_species_binary_mass_diffusivities(t[:4]),
                          dense(ref.get_species_binary_mass_diffusivities(
                              t[:4])))
    assert rel_err(o.get_mixture_viscosity_mixavg(t, y),
                   dense(ref.get_mixture_viscosity_mixavg(t, y))) < 1e-14
    assert rel_err(o.get_mixture_thermal_conductivity_mixavg(t, y),
                   dense(ref.get_mixture_thermal_conductivity_mixavg(
                       t, y))) < 1e-14
    assert rel_err(o.get_species_mass_diffusivities_mixavg(p, t, y),
                   dense(ref.get_species_mass_diffusivities_mixavg(
                       p, t, y))) < 1e-13
