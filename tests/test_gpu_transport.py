"""Mixture-averaged transport kernels (``csrc/transport.cuh``) through the
generated library's C ABI, against golden vectors from the reference's
generated transport methods (``pyrometheus/codegen/python.py:564-641``) and
against the CPU oracle.

Tolerance 1e-12 relative, taken at the scale the reference's own rounding
has: a degree-4 fit in ln T is compared at the size of its largest terms
(``sum |c_n| (ln T)^n``), and a mixture diffusivity at ``|D_k| x_sum_k /
denom_k`` (the reference subtracts ``x_k/D_kk`` from a sum that contains
it)."""

import ctypes

import numpy as np
import pytest

from test_transport import diffusivity_scale, transport_golden

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _cuda_class(sol):
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from pyrometheus_gb300 import get_thermochem_class
    return get_thermochem_class(sol)


def _np(x):
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else \
        np.asarray(x)


def _abs_fit(c, t):
    """sum_n |c_n| (ln T)^n for fits c[..., 5] at temperatures t[N]."""
    lt = np.log(np.asarray(t, dtype=np.float64))
    powers = np.stack([np.abs(lt) ** n for n in range(5)])
    return np.abs(c) @ powers


def _check_species(sol, th, t, visc=None, cond=None, bdiff=None):
    tr = sol.transport
    sq = np.sqrt(t)
    if visc is not None:
        got = _np(th.get_species_viscosities(t))
        scale = 2.0 * sq * _abs_fit(tr.viscosity, t) ** 2
        assert np.all(np.abs(got - visc) <= TOL * np.maximum(scale,
                                                             np.abs(visc)))
    if cond is not None:
        got = _np(th.get_species_thermal_conductivities(t))
        scale = sq * _abs_fit(tr.conductivity, t)
        assert np.all(np.abs(got - cond) <= TOL * np.maximum(scale,
                                                             np.abs(cond)))
    if bdiff is not None:
        nb = bdiff.shape[2]
        got = _np(th.get_species_binary_mass_diffusivities(t[:nb]))
        scale = (sq * t)[:nb] * _abs_fit(tr.diffusivity, t[:nb])
        assert np.all(np.abs(got - bdiff) <= TOL * np.maximum(scale,
                                                              np.abs(bdiff)))


def _check_mixture(o, th, p, t, y, mu, lam, dmix):
    got_mu = _np(th.get_mixture_viscosity_mixavg(t, y))
    got_lam = _np(th.get_mixture_thermal_conductivity_mixavg(t, y))
    got_d = _np(th.get_species_mass_diffusivities_mixavg(p, t, y))
    assert np.all(np.abs(got_mu - mu) <= TOL * np.abs(mu))
    assert np.all(np.abs(got_lam - lam) <= TOL * np.abs(lam))
    assert np.all(np.abs(got_d - dmix) <= TOL * diffusivity_scale(o, p, t, y))
    # the fused call runs the same per-quantity arithmetic
    f_mu, f_lam, f_d = th.get_transport_mixavg(p, t, y)
    assert np.array_equal(_np(f_mu), got_mu)
    assert np.array_equal(_np(f_lam), got_lam)
    assert np.array_equal(_np(f_d), got_d)


@pytest.mark.parametrize("tag", ["s9", "s53"])
def test_against_reference_goldens(tag):
    from oracle.thermo_oracle import Thermochemistry as Oracle
    sol, g = transport_golden(tag)
    th = _cuda_class(sol)()
    assert th.has_transport
    t, p, y = g["T"], g["P"], g["Y"]
    _check_species(sol, th, t, g["visc"], g["cond"], g["bdiff"])
    _check_mixture(Oracle(sol), th, p, t, y, g["mu_mix"], g["lam_mix"],
                   g["d_mix"])
    # pure N2 / pure H2: their own diffusivity is D_kk / p
    d = _np(th.get_species_mass_diffusivities_mixavg(p, t, y))
    for col, sp in ((-1, "N2"), (-2, "H2")):
        k = sol.species_index(sp)
        assert abs(d[k, col] - g["d_mix"][k, col]) <= \
            TOL * abs(g["d_mix"][k, col])


def test_against_oracle_on_a_batch():
    from oracle.thermo_oracle import Thermochemistry as Oracle
    from pyrometheus_gb300 import synthetic
    sol = synthetic.config2_mechanism()
    o = Oracle(sol)
    th = _cuda_class(sol)()
    t, p, y = synthetic.sample_states(sol, 3000, seed=77)
    _check_species(sol, th, t, o.get_species_viscosities(t),
                   o.get_species_thermal_conductivities(t),
                   o.get_species_binary_mass_diffusivities(t[:40]))
    _check_mixture(o, th, p, t, y, o.get_mixture_viscosity_mixavg(t, y),
                   o.get_mixture_thermal_conductivity_mixavg(t, y),
                   o.get_species_mass_diffusivities_mixavg(p, t, y))
    # a scalar pressure broadcasts to every state
    d1 = _np(th.get_species_mass_diffusivities_mixavg(2e5, t, y))
    d2 = _np(th.get_species_mass_diffusivities_mixavg(np.full(3000, 2e5), t,
                                                      y))
    assert np.array_equal(d1, d2)


def test_non_symmetric_fits():
    """A fit set with D_ij != D_ji runs the kernel's all-pairs loop."""
    from oracle.thermo_oracle import Thermochemistry as Oracle
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.transport_fits import TransportFits
    sol = synthetic.config1_mechanism()
    tr = sol.transport
    diff = tr.diffusivity.copy()
    diff[0, 3] *= 1.01
    diff[5, 2] *= 0.98
    sol.transport = TransportFits(tr.viscosity, tr.conductivity, diff)
    th = _cuda_class(sol)()
    info = ctypes.c_int(), ctypes.c_int()
    assert th._lib.pyro_transport_info(ctypes.byref(info[0]),
                                       ctypes.byref(info[1])) == 0
    assert info[0].value == 1 and info[1].value == 0
    o = Oracle(sol)
    t, p, y = synthetic.sample_states(sol, 500, seed=78)
    _check_species(sol, th, t, bdiff=o.get_species_binary_mass_diffusivities(
        t[:20]))
    _check_mixture(o, th, p, t, y, o.get_mixture_viscosity_mixavg(t, y),
                   o.get_mixture_thermal_conductivity_mixavg(t, y),
                   o.get_species_mass_diffusivities_mixavg(p, t, y))


def test_extreme_fit_values_take_the_exact_division_path():
    """Pair values outside [2^-200, 2^200] make the grouped reciprocal
    (one division for four pairs) fall back to one division per pair; the
    result still matches the reference's per-pair division."""
    from oracle.thermo_oracle import Thermochemistry as Oracle
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.transport_fits import TransportFits
    sol = synthetic.config1_mechanism()
    tr = sol.transport
    diff = tr.diffusivity.copy()
    for i, j, f in ((2, 5, 1e230), (1, 7, 1e-230)):
        diff[i, j] *= f
        diff[j, i] *= f
    sol.transport = TransportFits(tr.viscosity, tr.conductivity, diff)
    th = _cuda_class(sol)()
    o = Oracle(sol)
    t, p, y = synthetic.sample_states(sol, 300, seed=79)
    got = _np(th.get_species_mass_diffusivities_mixavg(p, t, y))
    ref = o.get_species_mass_diffusivities_mixavg(p, t, y)
    assert np.all(np.isfinite(got))
    assert np.all(np.abs(got - ref) <= TOL * diffusivity_scale(o, p, t, y))


def test_shapes_scalars_and_empty():
    from pyrometheus_gb300 import synthetic
    sol = synthetic.config1_mechanism()
    th = _cuda_class(sol)()
    S = sol.n_species
    assert tuple(th.get_species_viscosities(1200.0).shape) == (S,)
    assert tuple(th.get_species_binary_mass_diffusivities(1200.0).shape) \
        == (S, S)
    y = np.full(S, 1.0 / S)
    mu, lam, d = th.get_transport_mixavg(1e5, 1200.0, y)
    assert mu.dim() == 0 and lam.dim() == 0 and tuple(d.shape) == (S,)
    empty = th.get_species_viscosities(np.zeros(0))
    assert tuple(empty.shape) == (S, 0)
    mu0 = th.get_mixture_viscosity_mixavg(np.zeros(0), np.zeros((S, 0)))
    assert tuple(mu0.shape) == (0,)


def test_mechanism_without_fits_is_unsupported():
    from pyrometheus_gb300 import synthetic
    from pyrometheus_gb300.yaml_mech import dump_mechanism, load_mechanism
    bare = load_mechanism("bare.yaml",
                          text=dump_mechanism(synthetic.config1_mechanism()))
    th = _cuda_class(bare)()
    assert not th.has_transport
    with pytest.raises(ValueError):
        th.get_species_viscosities(np.array([1000.0]))
    t = torch.full((4,), 1000.0, dtype=torch.float64, device="cuda")
    out = torch.empty((bare.n_species, 4), dtype=torch.float64,
                      device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert th._lib.pyro_species_transport(0, t.data_ptr(), 1,
                                          out.data_ptr(), 4, 4, stream) == 4
