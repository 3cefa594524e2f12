"""Property tests of the oracle over random states (hypothesis), the
identities the reference's own tests rest on: net rates of progress equal
forward minus reverse and net production equals creation minus destruction
(``test/test.py:259-297``), mass conservation of the production rates, the
energy/enthalpy Newton inverting the mixture energy and enthalpy
(``test.py:174-209``), and the equilibrium constants' definition from the
Gibbs energies (``python.py:360-373``)."""

import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

from oracle.thermo_oracle import Thermochemistry as Oracle  # noqa: E402
from pyrometheus_gb300 import synthetic  # noqa: E402

_MECHS = {}


def _oracle(tag):
    if tag not in _MECHS:
        sol = (synthetic.config1_mechanism() if tag == "s9"
               else synthetic.config2_mechanism())
        _MECHS[tag] = (sol, Oracle(sol))
    return _MECHS[tag]


def _state(sol, seed, n=16):
    """Seeded states: T ~ U[300, 3000] K, p log-uniform in [1e4, 1e6] Pa,
    Y = 0.6 N2 + 0.4 Dirichlet(0.5)."""
    t, p, y = synthetic.sample_states(sol, n, seed=seed)
    return t, p, y


states = st.tuples(st.sampled_from(["s9", "s53"]),
                   st.integers(min_value=0, max_value=2 ** 31 - 1))


@settings(max_examples=20, deadline=None)
@given(states)
def test_rate_identities(case):
    tag, seed = case
    sol, o = _oracle(tag)
    t, p, y = _state(sol, seed)
    rho = o.get_density(p, t, y)
    c = o.get_concentrations(rho, y)
    net = o.get_net_rates_of_progress(t, c)
    fwd = o.get_fwd_rates_of_progress(t, c)
    rev = o.get_rev_rates_of_progress(t, c)
    scale = np.abs(fwd) + np.abs(rev)
    assert np.all(np.abs(net - (fwd - rev)) <= 1e-13 * scale + 1e-300)
    w = o.get_net_production_rates(rho, t, y)
    cd, dd = o.get_creation_destruction_rates(rho, t, y)
    assert np.all(np.abs(w - (cd - dd)) <= 1e-13 * (cd + dd) + 1e-300)
    mass = (o.molecular_weights[:, None] * w).sum(axis=0)
    mscale = (o.molecular_weights[:, None] * (cd + dd)).sum(axis=0)
    assert np.all(np.abs(mass) <= 1e-13 * mscale + 1e-300)


@settings(max_examples=20, deadline=None)
@given(states, st.booleans())
def test_temperature_inverts_energy_and_enthalpy(case, do_energy):
    tag, seed = case
    sol, o = _oracle(tag)
    t, p, y = _state(sol, seed)
    target = (o.get_mixture_internal_energy_mass(t, y) if do_energy
              else o.get_mixture_enthalpy_mass(t, y))
    t_back = o.get_temperature(target, 0.9 * t, y, do_energy)
    assert np.abs(t_back - t).max() < 1e-10 * np.abs(t).max()


@settings(max_examples=10, deadline=None)
@given(states)
def test_equilibrium_constants_from_gibbs_energies(case):
    """``log_k_eq = sum nu'' g - sum nu' g - dnu ln(p0 / R T)`` per
    reversible reaction (the negative natural log of Kc)."""
    tag, seed = case
    sol, o = _oracle(tag)
    t, _, _ = _state(sol, seed)
    g = o.get_species_gibbs_rt(t)
    lk = o.get_equilibrium_constants(t)
    c0 = np.log(o.one_atm / (o.gas_constant * t))
    idx = {name: k for k, name in enumerate(sol.species_names)}
    for j, r in enumerate(sol.reactions()):
        if not r.reversible:
            continue
        dg = sum(nu * g[idx[s]] for s, nu in r.products.items()) \
            - sum(nu * g[idx[s]] for s, nu in r.reactants.items())
        dnu = sum(r.products.values()) - sum(r.reactants.values())
        ref = dg - dnu * c0
        scale = (sum(abs(nu * g[idx[s]]) for s, nu in r.products.items())
                 + sum(abs(nu * g[idx[s]]) for s, nu in r.reactants.items())
                 + abs(dnu * c0))
        assert np.all(np.abs(lk[j] - ref) <= 1e-13 * scale), r.equation
