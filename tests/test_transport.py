"""Mixture-averaged transport on the CPU: the oracle against golden vectors
from the reference's own generated transport methods
(``pyrometheus/codegen/python.py:564-641``, ``tests/golden/make_golden.py``),
the kinetic-theory stand-in fits, and the ``cuda`` target's handling of
mechanisms with and without fits."""

import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_err
from oracle.thermo_oracle import Thermochemistry as Oracle
from pyrometheus_gb300 import synthetic
from pyrometheus_gb300.transport_fits import TransportFits, \
    kinetic_theory_fits
from pyrometheus_gb300.yaml_mech import dump_mechanism, load_mechanism

TAGS = ["s9", "s53"]


def transport_golden(tag):
    """The mechanism (with the stored fits attached) and the vectors."""
    d = np.load(os.path.join(GOLDEN, "transport.npz"))
    g = {k[len(tag) + 1:]: d[k] for k in d.files if k.startswith(tag + "_")}
    sol = load_mechanism(f"{tag}.yaml", text=str(g.pop("mech_yaml")))
    sol.transport = TransportFits(g.pop("fit_visc"), g.pop("fit_cond"),
                                  g.pop("fit_diff"))
    return sol, g


def diffusivity_scale(o, p, t, y):
    """|D_k| x_sum_k / denom_k: the reference subtracts x_k/D_kk from a sum
    that contains it, so its own rounding is relative to x_sum_k, not to
    the difference; the parity check is taken at that scale."""
    mmw = o.get_mixture_molecular_weight(y)
    x = o.get_mole_fractions(mmw, y)
    bd = o.get_species_binary_mass_diffusivities(t)
    xs = np.stack([sum(x[i] / bd[i][k] for i in range(o.num_species))
                   for k in range(o.num_species)])
    denom = xs - x / np.stack([bd[k][k] for k in range(o.num_species)])
    d = o.get_species_mass_diffusivities_mixavg(p, t, y)
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = np.where(denom > 0, xs / denom, 1.0)
    return np.abs(d) * np.maximum(amp, 1.0)


def test_synthetic_mechanisms_carry_the_stored_fits():
    for tag, make in (("s9", synthetic.config1_mechanism),
                      ("s53", synthetic.config2_mechanism)):
        sol, _ = transport_golden(tag)
        ref = make()
        assert dump_mechanism(ref) == dump_mechanism(sol)
        for a, b in ((ref.transport.viscosity, sol.transport.viscosity),
                     (ref.transport.conductivity,
                      sol.transport.conductivity),
                     (ref.transport.diffusivity, sol.transport.diffusivity)):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_against_reference_transport(tag):
    sol, g = transport_golden(tag)
    o = Oracle(sol)
    t, p, y = g["T"], g["P"], g["Y"]
    # species fits: the same expressions, bit for bit
    assert np.array_equal(o.get_species_viscosities(t), g["visc"])
    assert np.array_equal(o.get_species_thermal_conductivities(t),
                          g["cond"])
    nb = g["bdiff"].shape[2]
    assert np.array_equal(o.get_species_binary_mass_diffusivities(t[:nb]),
                          g["bdiff"])
    # mixture rules: mole fractions may differ in the last bit, which a
    # few roundings carry into the results
    assert rel_err(o.get_mixture_viscosity_mixavg(t, y), g["mu_mix"]) \
        < 1e-14
    assert rel_err(o.get_mixture_thermal_conductivity_mixavg(t, y),
                   g["lam_mix"]) < 1e-14
    d = o.get_species_mass_diffusivities_mixavg(p, t, y)
    assert np.all(np.abs(d - g["d_mix"])
                  <= 1e-14 * diffusivity_scale(o, p, t, y))
    # the pure-species states take the D_kk / p branch for their species
    for col, sp in ((-1, "N2"), (-2, "H2")):
        k = sol.species_index(sp)
        dkk = o.get_species_binary_mass_diffusivities(t[col:][:1])[k][k][0]
        assert d[k, col] == dkk / p[col]


def test_kinetic_theory_fits_are_physical():
    sol = synthetic.config2_mechanism()
    fits = kinetic_theory_fits(sol, seed=3)
    S = sol.n_species
    assert fits.viscosity.shape == (S, 5) and fits.symmetric
    t = np.geomspace(300.0, 3500.0, 50)
    lt = np.log(t)
    powers = np.stack([lt ** n for n in range(5)])
    mu = np.sqrt(t) * (fits.viscosity @ powers) ** 2
    lam = np.sqrt(t) * (fits.conductivity @ powers)
    dp = t ** 1.5 * (fits.diffusivity.reshape(-1, 5) @ powers)
    # gas-phase magnitudes: mu ~ 1e-5 Pa s, lam ~ 0.01-1 W/m/K,
    # D ~ 1e-5 m^2/s at 1 atm
    assert 1e-6 < mu.min() and mu.max() < 1e-3
    assert 1e-3 < lam.min() and lam.max() < 5.0
    d_atm = dp / 101325.0
    assert 1e-7 < d_atm.min() and d_atm.max() < 1e-1
    # viscosity rises with temperature for every species
    assert np.all(np.diff(mu, axis=1) > 0)


def test_mechanism_without_fits():
    from pyrometheus_gb300.codegen.cuda import CudaCodeGenerator
    sol = synthetic.config1_mechanism()
    bare = load_mechanism("bare.yaml", text=dump_mechanism(sol))
    assert bare.transport is None and bare.transport_model == "none"
    with pytest.raises(ValueError):
        bare.get_viscosity_polynomial(0)
    src = CudaCodeGenerator.generate("bare", bare)
    assert "PYRO_HAS_TRANSPORT" not in src
    assert '#include "transport.cuh"' in src
    with pytest.raises(ValueError):
        Oracle(bare).get_species_viscosities(np.array([1000.0]))


def test_generated_transport_tables():
    from pyrometheus_gb300.codegen.cuda import CudaCodeGenerator
    sol = synthetic.config1_mechanism()
    S = sol.n_species
    src = CudaCodeGenerator.generate("s9", sol)
    assert "#define PYRO_HAS_TRANSPORT 1" in src
    assert "#define PYRO_TR_SYM 1" in src
    # symmetric fits: one record per unordered pair
    assert f"k_tr_diff[{S * (S + 1) // 2 * 5}]" in src
    assert f"k_tr_wilke[{S * S}]" in src
    # a non-symmetric set keeps every ordered pair
    tr = sol.transport
    diff = tr.diffusivity.copy()
    diff[0, 1, 0] *= 1.0 + 1e-9
    sol.transport = TransportFits(tr.viscosity, tr.conductivity, diff)
    src = CudaCodeGenerator.generate("s9", sol)
    assert "#define PYRO_TR_SYM 0" in src
    assert f"k_tr_diff[{S * S * 5}]" in src


def test_yaml_lennard_jones_fits():
    """Kinetic-theory fits from a YAML mechanism's species transport data
    (diameter, well-depth); none unless requested; a species without the
    data is an error."""
    text = dump_mechanism(synthetic.config1_mechanism())
    sol = load_mechanism("m.yaml", text=text)
    assert sol.transport is None
    lines, out, in_species = text.splitlines(), [], False
    for ln in lines:
        out.append(ln)
        if not ln.startswith((" ", "-")):
            in_species = ln.startswith("species:")
        if in_species and ln.startswith("- name: "):
            out += ["  transport:", "    model: gas",
                    "    geometry: linear", "    diameter: 3.0",
                    "    well-depth: 100.0"]
    lj = "\n".join(out) + "\n"
    sol = load_mechanism("m.yaml", text=lj, transport="kinetic-theory")
    S = sol.n_species
    assert sol.transport.viscosity.shape == (S, 5)
    assert sol.transport.symmetric
    t = np.array([1000.0])
    mu = Oracle(sol).get_species_viscosities(t)
    assert np.all((mu > 1e-6) & (mu < 1e-3))
    with pytest.raises(ValueError):
        load_mechanism("m.yaml", text=text, transport="kinetic-theory")
    with pytest.raises(ValueError):
        load_mechanism("m.yaml", text=lj, transport="cantera")
