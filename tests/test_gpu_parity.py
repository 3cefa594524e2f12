"""CUDA path against the golden vectors and the CPU oracle.

Tolerances follow the parity contract: 1e-12 relative per element
(production rates and net rates of progress measured against the
creation + destruction scale, so equilibrium cancellation does not produce
false failures), temperatures within 1e-10 K.  All calls go through the
generated library's C ABI (via the drop-in ``Thermochemistry`` class)."""

import numpy as np
import pytest

from conftest import GOLDEN_SETS, load_golden, rel_err

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_T = 1e-10


def _cuda_class(sol):
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from pyrometheus_gb300 import get_thermochem_class
    return get_thermochem_class(sol)


def _np(x):
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else \
        np.asarray(x)


@pytest.fixture(params=GOLDEN_SETS)
def golden_cuda(request):
    sol, g = load_golden(request.param)
    return sol, g, _cuda_class(sol)()


def test_species_and_mixture_properties(golden_cuda):
    sol, g, th = golden_cuda
    t, y = g["T"], g["Y"]
    for key, fn in (("cp_r", th.get_species_specific_heats_r),
                    ("h_rt", th.get_species_enthalpies_rt),
                    ("s_r", th.get_species_entropies_r),
                    ("dcp_r", th.get_species_specific_heats_r_derivative),
                    ("dh_rt", th.get_species_enthalpies_rt_derivative),
                    ("ds_r", th.get_species_entropies_rt_derivative)):
        # dimensionless thermo crosses zero (h/RT, s/R derivatives): relative
        # above 1, absolute below, like the reference's absolute criterion
        # (test/test.py:125-171)
        assert rel_err(_np(fn(t)), g[key], 1.0) < TOL, key
    # g = h - s carries the cancellation of its two terms: compare at the
    # scale of |h| + |s|
    gg = _np(th.get_species_gibbs_rt(t))
    assert np.all(np.abs(gg - g["g_rt"])
                  <= TOL * (np.abs(g["h_rt"]) + np.abs(g["s_r"])))
    assert rel_err(_np(th.get_mixture_molecular_weight(y)), g["mmw"]) < TOL
    assert rel_err(_np(th.get_pressure(g["rho"], t, y)), g["pressure"]) < TOL
    assert rel_err(_np(th.get_density(g["P"], t, y)), g["rho"]) < TOL
    for key, fn in (("cp_mass", th.get_mixture_specific_heat_cp_mass),
                    ("cv_mass", th.get_mixture_specific_heat_cv_mass),
                    ("h_mass", th.get_mixture_enthalpy_mass),
                    ("e_mass", th.get_mixture_internal_energy_mass)):
        assert rel_err(_np(fn(t, y)), g[key]) < TOL, key
    assert rel_err(_np(th.get_concentrations(g["rho"], y)), g["conc"]) < TOL


def test_kinetics(golden_cuda):
    sol, g, th = golden_cuda
    t, c, rho, y = g["T"], g["conc"], g["rho"], g["Y"]
    lk = _np(th.get_equilibrium_constants(t))
    scale = np.abs(g["g_rt"]).max(axis=0)
    assert np.all(np.abs(lk - g["log_k_eq"]) <= TOL * 10 * scale)
    assert rel_err(_np(th.get_fwd_rate_coefficients(t, c)), g["k_fwd"]) < TOL
    assert rel_err(_np(th.get_fwd_rates_of_progress(t, c)), g["r_fwd"]) < TOL
    assert rel_err(_np(th.get_rev_rates_of_progress(t, c)), g["r_rev"]) < TOL
    s_r = np.abs(g["r_fwd"]) + np.abs(g["r_rev"])
    assert rel_err(_np(th.get_net_rates_of_progress(t, c)), g["r_net"],
                   s_r) < TOL
    s = g["cdot"] + g["ddot"]
    assert rel_err(_np(th.get_net_production_rates(rho, t, y)), g["wdot"],
                   s) < TOL
    cd, dd = th.get_creation_destruction_rates(rho, t, y)
    assert rel_err(_np(cd), g["cdot"]) < TOL
    assert rel_err(_np(dd), g["ddot"]) < TOL
    assert rel_err(_np(th.get_creation_rates(rho, t, y)), g["cdot"]) < TOL


def test_temperature(golden_cuda):
    sol, g, th = golden_cuda
    y = g["Y"]
    te = _np(th.get_temperature(g["e_mass"], 1500.0, y, True))
    th_ = _np(th.get_temperature(g["h_mass"], 1500.0, y, False))
    assert np.abs(te - g["T_from_e"]).max() < TOL_T
    assert np.abs(th_ - g["T_from_h"]).max() < TOL_T
    if "T_from_e_guess09" in g:
        # the reference's temperature test starts from 0.9 T
        # (test/test.py:196-199)
        t9 = _np(th.get_temperature(g["e_mass"], 0.9 * g["T"], y, True))
        assert np.abs(t9 - g["T_from_e_guess09"]).max() < TOL_T


def test_falloff_rates_in_place(golden_cuda):
    sol, g, th = golden_cuda
    t, c = g["T"], g["conc"]
    k = torch.zeros((sol.n_reactions, t.size), dtype=torch.float64,
                    device="cuda")
    assert th.get_falloff_rates(t, c, k) is None
    idx = [j for j, r in enumerate(sol.reactions())
           if r.reaction_type.startswith("falloff")]
    if idx:
        assert rel_err(_np(k)[idx], g["k_fwd"][idx]) < TOL


@pytest.mark.parametrize("name,n", [("synthetic9", 65536),
                                    ("synthetic53", 16384)])
def test_large_batch_against_oracle(name, n):
    from oracle.thermo_oracle import Thermochemistry as Oracle
    from pyrometheus_gb300 import synthetic
    sol, _ = load_golden(name)
    th = _cuda_class(sol)()
    orc = Oracle(sol)
    t, p, y = synthetic.sample_states(sol, n, seed=99)
    rho = orc.get_density(p, t, y)
    e = orc.get_mixture_internal_energy_mass(t, y)
    cd, dd = orc.get_creation_destruction_rates(rho, t, y)
    w_ref = orc.get_net_production_rates(rho, t, y)
    w, tn = th.get_net_production_rates_and_temperature(p, t, y, e, 1500.0)
    assert rel_err(_np(w), w_ref, cd + dd) < TOL
    assert np.abs(_np(tn) - t).max() < TOL_T
    # fused == unfused calls
    rho_d = th.get_density(p, t, y)
    w2 = th.get_net_production_rates(rho_d, t, y)
    t2 = th.get_temperature(e, 1500.0, y, do_energy=True)
    assert torch.equal(w, w2)
    assert np.abs(_np(tn) - _np(t2)).max() < 1e-12 * 3000


def test_layouts_and_edge_sizes():
    from oracle.thermo_oracle import Thermochemistry as Oracle
    from pyrometheus_gb300 import synthetic
    sol, _ = load_golden("synthetic9")
    th = _cuda_class(sol)()
    orc = Oracle(sol)
    for n in (1, 31, 33, 65537):
        t, p, y = synthetic.sample_states(sol, n, seed=n)
        rho = orc.get_density(p, t, y)
        cd, dd = orc.get_creation_destruction_rates(rho, t, y)
        ref = orc.get_net_production_rates(rho, t, y)
        assert rel_err(_np(th.get_net_production_rates(rho, t, y)), ref,
                       cd + dd) < TOL
        # strided species-major input: leading dimension > n
        pad = torch.zeros((sol.n_species, n + 7), dtype=torch.float64,
                          device="cuda")
        pad[:, :n] = torch.as_tensor(y, device="cuda")
        assert rel_err(_np(th.get_net_production_rates(rho, t, pad[:, :n])),
                       ref, cd + dd) < TOL
    # broadcast scalars (the reference accepts scalars for T and rho)
    t, p, y = synthetic.sample_states(sol, 64, seed=5)
    w = th.get_net_production_rates(0.5, 1500.0, y)
    ref = orc.get_net_production_rates(0.5, np.full(64, 1500.0), y)
    cd, dd = orc.get_creation_destruction_rates(0.5, np.full(64, 1500.0), y)
    assert rel_err(_np(w), ref, cd + dd) < TOL
    # a single state (1-D composition) returns 1-D outputs
    w1 = th.get_net_production_rates(0.5, 1500.0, y[:, 0])
    assert tuple(w1.shape) == (sol.n_species,)
    assert rel_err(_np(w1), ref[:, 0], (cd + dd)[:, 0]) < TOL
    # empty batch
    w0 = th.get_net_production_rates(np.zeros(0), np.zeros(0),
                                     np.zeros((sol.n_species, 0)))
    assert tuple(w0.shape) == (sol.n_species, 0)


def test_newton_failure_raises_like_reference():
    sol, g = load_golden("synthetic9")
    th = _cuda_class(sol)()
    e = g["e_mass"].copy()
    e[3] = np.nan
    with pytest.raises(RuntimeError,
                       match="Temperature iteration failed to converge"):
        th.get_temperature(e, 1500.0, g["Y"], True)
    # the context stays usable
    te = th.get_temperature(g["e_mass"], 1500.0, g["Y"], True)
    assert np.abs(_np(te) - g["T_from_e"]).max() < TOL_T
