"""Generate the golden vectors in this folder from the reference itself.

Run with ``PYRO_REFERENCE_ROOT`` set to the root of a reference checkout::

    PYRO_REFERENCE_ROOT=<checkout> python tests/golden/make_golden.py [fixtures]

For each mechanism below it

1. builds the mechanism -- seeded synthetic ones with
   :mod:`pyrometheus_gb300.synthetic`, and the reference's own test
   fixtures (``test/mechs/{uiuc,sandiego,hong,uconn32,gri30}.yaml``, the
   set ``test/CMakeLists.txt:9`` runs every backend on) through the YAML
   loader -- and stores its Cantera-YAML text in SI units (so the tests
   rebuild exactly the same mechanism without the checkout);
2. renders the reference's ``PythonCodeGenerator`` class for it
   (``oracle/refgen.py``: the reference's generator with stand-ins for its
   uninstalled Cantera/pymbolic/mako dependencies);
3. evaluates the reference's generated methods with numpy on seeded states
   and stores inputs and outputs;
4. evaluates the same generated class on torch CPU float64 tensors and
   differentiates the constant-pressure reactor source with
   ``torch.func.jacfwd`` -- the stand-in for the reference's
   ``jax.jacfwd`` over its generated class (``test/test.py:335-347``,
   ``flamelets/equations.py:124-129``, ``examples/free_flame/reactors.py:125``).

The outputs are small ``.npz`` files; this script is the only thing that
writes them.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refgen  # noqa: E402
from pyrometheus_gb300 import synthetic  # noqa: E402
from pyrometheus_gb300.mechanism import gas_constant  # noqa: E402
from pyrometheus_gb300.yaml_mech import dump_mechanism  # noqa: E402


def quirks_mechanism():
    """Small mechanism exercising irreversible reactions, explicit reaction
    orders and a zero default efficiency."""
    sol = synthetic.make_mechanism(synthetic.SPECIES_9, 18, 3, 2, 1, seed=7,
                                   irreversible_fraction=0.35,
                                   name="quirks9")
    rng = np.random.default_rng(70)
    n_orders = 0
    for r in sol.reactions():
        if not r.reversible and n_orders < 3:
            r.orders = {sp: float(np.round(rng.uniform(0.3, 1.7), 2))
                        for sp in r.reactants}
            n_orders += 1
    tb = [r for r in sol.reactions()
          if r.reaction_type == "three-body-Arrhenius"]
    tb[0].third_body.default_efficiency = 0.0
    return sol


def edge_states(sol, n, seed):
    t, p, y = synthetic.sample_states(sol, n, seed=seed)
    # the strict T > Tmid branch (chem_expr.py:54) at exactly Tmid,
    # the ends of the range, and exact zeros in the composition
    t[0], t[1], t[2] = 1000.0, 300.0, 3000.0
    y[:, 3] = 0.0
    y[sol.species_index("N2"), 3] = 1.0
    zero = [k for k in range(sol.n_species) if k % 3 == 1]
    y[zero, 4] = 0.0
    y[:, 4] /= y[:, 4].sum()
    return t, p, y


class _TorchNS:
    """``pyro_np`` namespace mapping the generated code's calls to torch."""

    def __init__(self):
        import torch
        self.torch = torch
        self.linalg = torch.linalg

    def __getattr__(self, name):
        return getattr(self.torch, name)


def torch_reference(cls):
    import torch

    class TorchThermo(cls):
        def _pyro_make_array(self, res_list):
            ts = [x if isinstance(x, torch.Tensor) else torch.tensor(
                float(x), dtype=torch.float64) for x in res_list]
            ts = torch.broadcast_tensors(*ts)
            return torch.stack(ts)

        def _pyro_norm(self, argument, normord):
            return torch.linalg.norm(argument, normord)

    return TorchThermo(_TorchNS())


def reactor_jacobian(cls, p, t, y):
    """``jacfwd`` of ``[dT/dt, dY/dt]`` (adiabatic, constant p) w.r.t.
    ``(T, Y)`` through the reference's generated methods."""
    import torch
    from torch.func import jacfwd, vmap
    th = torch_reference(cls)
    mw = torch.tensor(th.molecular_weights, dtype=torch.float64)

    def source(x, pres):
        temp, mass = x[0], x[1:]
        rho = th.get_density(pres, temp, mass)
        w = th.get_net_production_rates(rho, temp, mass)
        h_rt = th.get_species_enthalpies_rt(temp)
        cp = th.get_mixture_specific_heat_cp_mass(temp, mass)
        tdot = -(th.gas_constant * temp * (h_rt * w).sum()) / (rho * cp)
        return torch.cat([tdot[None], mw * w / rho])

    x = torch.tensor(np.concatenate([t[None, :], y], axis=0).T)
    pres = torch.tensor(p)
    jac = vmap(jacfwd(source), in_dims=(0, 0))(x, pres)
    val = vmap(source, in_dims=(0, 0))(x, pres)
    return jac.numpy(), val.numpy().T


def reactor_states(sol, fuel, stoich_ratio, n_samples, t_end):
    """States along an adiabatic constant-pressure ignition from 1500 K and
    one atmosphere, with the fuel/O2/N2 mole fractions of the reference's
    kinetics tests (``test/test.py:228-238``: equivalence ratio 1,
    oxidizer-to-diluent ratio 0.21), sampled at the first integrator steps
    where the temperature has risen by 0, 1/n, ..., (n-1)/n of its rise up
    to *t_end*.  The trajectory comes from SciPy's BDF on the oracle's
    source terms (vectorised over the difference Jacobian's columns); it
    only supplies realistic compositions (radical pools, near-equilibrium
    products)."""
    from scipy.integrate import solve_ivp

    from oracle.thermo_oracle import Thermochemistry as Oracle
    orc = Oracle(sol)
    S = sol.n_species
    x = np.zeros(S)
    i_fu, i_ox = sol.species_index(fuel), sol.species_index("O2")
    i_di = sol.species_index("N2")
    x[i_fu] = 0.21 / (stoich_ratio + 0.21)
    x[i_ox] = stoich_ratio * x[i_fu]
    x[i_di] = (1.0 - 0.21) * x[i_ox] / 0.21
    x /= x.sum()
    mw = np.asarray(sol.molecular_weights, dtype=np.float64)
    y0 = x * mw / np.dot(x, mw)
    p0 = 101325.0

    def rhs(_, s):
        s = s.reshape(S + 1, -1)
        t, y = s[0], np.maximum(s[1:], 0.0)
        rho = orc.get_density(p0, t, y)
        w = orc.get_net_production_rates(rho, t, y)
        h = orc.get_species_enthalpies_rt(t) * gas_constant * t
        cp = orc.get_mixture_specific_heat_cp_mass(t, y)
        return np.vstack([-(h * w).sum(axis=0) / (rho * cp),
                          mw[:, None] * w / rho])

    traj = solve_ivp(rhs, (0.0, t_end), np.concatenate([[1500.0], y0]),
                     method="BDF", rtol=1e-7, atol=1e-13, vectorized=True)
    if traj.status != 0:
        raise RuntimeError(f"ignition on {sol.source}: {traj.message}")
    rise = traj.y[0] - traj.y[0, 0]
    picks = [int(np.argmax(rise >= k / n_samples * rise[-1]))
             for k in range(n_samples)]
    states = traj.y[:, picks]
    y = np.maximum(states[1:], 0.0)
    y /= y.sum(axis=0, keepdims=True)
    return states[0].copy(), np.full(n_samples, p0), y


def fixture_states(sol, fuel, stoich_ratio, t_end, n_reactor, n_random,
                   seed):
    """The state families of the reference's tests (``test/test.py``):
    ignition-trajectory states, seeded random states with edge cases
    (T = Tmid, 300 K, 3000 K, exact zeros), equal mass fractions at ten
    temperatures in [500, 3000] K (``:56-60``), and every pure species at
    those temperatures (``:191-200``); pressure one atmosphere except for
    the random states."""
    S = sol.n_species
    t_r, p_r, y_r = reactor_states(sol, fuel, stoich_ratio, n_reactor,
                                   t_end)
    t_e, p_e, y_e = edge_states(sol, n_random, seed)
    temps = np.linspace(500.0, 3000.0, 10)
    t_u, y_u = temps.copy(), np.full((S, 10), 1.0 / S)
    t_p = np.tile(temps, S)
    y_p = np.repeat(np.eye(S), 10, axis=1)
    t = np.concatenate([t_r, t_e, t_u, t_p])
    p = np.concatenate([p_r, p_e, np.full(10 + 10 * S, 101325.0)])
    y = np.ascontiguousarray(np.concatenate([y_r, y_e, y_u, y_p], axis=1))
    return t, p, y


def golden(sol, n, seed, n_jac, fname, states=None):
    cls = refgen.reference_class(sol)
    ref = cls()
    if states is None:
        t, p, y = edge_states(sol, n, seed)
    else:
        t, p, y = states
        n = t.size
    mmw = ref.get_mixture_molecular_weight(y)
    rho = p * mmw / (gas_constant * t)
    c = np.array(list(ref.get_concentrations(rho, y)))

    def arr(x):
        return np.array([np.broadcast_to(np.asarray(v, dtype=np.float64),
                                         (n,)) for v in x])

    out = dict(
        T=t, P=p, Y=y, rho=rho, conc=c,
        mmw=np.asarray(mmw),
        pressure=np.asarray(ref.get_pressure(rho, t, y)),
        cp_r=arr(ref.get_species_specific_heats_r(t)),
        h_rt=arr(ref.get_species_enthalpies_rt(t)),
        s_r=arr(ref.get_species_entropies_r(t)),
        g_rt=arr(ref.get_species_gibbs_rt(t)),
        dcp_r=arr(ref.get_species_specific_heats_r_derivative(t)),
        dh_rt=arr(ref.get_species_enthalpies_rt_derivative(t)),
        ds_r=arr(ref.get_species_entropies_rt_derivative(t)),
        cp_mass=np.asarray(ref.get_mixture_specific_heat_cp_mass(t, y)),
        cv_mass=np.asarray(ref.get_mixture_specific_heat_cv_mass(t, y)),
        h_mass=np.asarray(ref.get_mixture_enthalpy_mass(t, y)),
        e_mass=np.asarray(ref.get_mixture_internal_energy_mass(t, y)),
        log_k_eq=arr(ref.get_equilibrium_constants(t)),
        k_fwd=arr(ref.get_fwd_rate_coefficients(t, c)),
        r_net=arr(ref.get_net_rates_of_progress(t, c)),
        r_fwd=arr(ref.get_fwd_rates_of_progress(t, c)),
        r_rev=arr(ref.get_rev_rates_of_progress(t, c)),
        wdot=arr(ref.get_net_production_rates(rho, t, y)),
        cdot=arr(ref.get_creation_rates(rho, t, y)),
        ddot=arr(ref.get_destruction_rates(rho, t, y)),
    )
    e = out["e_mass"]
    h = out["h_mass"]
    out["T_from_e"] = np.asarray(ref.get_temperature(e, 1500.0, y, True))
    out["T_from_h"] = np.asarray(ref.get_temperature(h, 1500.0, y, False))
    # the reference's own guess in its temperature test (test/test.py:197)
    out["T_from_e_guess09"] = np.asarray(
        ref.get_temperature(e, 0.9 * t, y, True))
    jac, src = reactor_jacobian(cls, p[:n_jac], t[:n_jac], y[:, :n_jac])
    out["jac"] = jac
    out["reactor_source"] = src
    out["mech_yaml"] = np.array(dump_mechanism(sol))
    np.savez_compressed(os.path.join(HERE, fname), **out)
    print(f"wrote {fname}: S={sol.n_species} R={sol.n_reactions} N={n} "
          f"jac={n_jac}")


def golden_block_thomas(fname="block_thomas.npz"):
    """Systems of the benchmark's kind (diagonally dominant random blocks,
    uneven lengths) solved by the reference's own block_thomas."""
    from oracle.block_thomas_oracle import make_systems
    bt = refgen.reference_block_thomas()
    out = {}
    for tag, nv, nsys, nmin, nmax, seed in (("nv4", 4, 5, 1, 9, 31),
                                            ("nv10", 10, 4, 2, 40, 32),
                                            ("nv54", 54, 2, 3, 12, 33)):
        lengths, lo, c, up, b = make_systems(nsys, nv, nmin, nmax, seed)
        x = np.empty_like(b)
        r0 = 0
        for n in lengths:
            n = int(n)
            x[r0:r0 + n] = bt(lo[r0:r0 + n - 1], c[r0:r0 + n],
                              up[r0:r0 + n - 1], b[r0:r0 + n])
            r0 += n
        for k, v in (("lengths", lengths), ("L", lo), ("C", c), ("U", up),
                     ("b", b), ("x", x)):
            out[f"{tag}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, fname), **out)
    print(f"wrote {fname}")


def _enthalpy_newton(th, h, y, t0, fixed_iters=None):
    """T with h_mix(T, Y) = h: the Newton iteration of the reference's
    ``get_temperature_from_enthalpy`` (``flamelets/make_pyro.py:255-299``:
    T -= f / j with f = h - h_mix(T), j = -cp_mix(T), until
    ||f / j||_2 <= 1e-10), on the reference's generated class ``th``.  With
    *fixed_iters* it runs that many steps instead (forward-mode autodiff
    cannot follow a data-dependent loop exit; past convergence the steps
    change nothing)."""
    t = t0
    for it in range(fixed_iters or 500):
        f = h - th.get_mixture_enthalpy_mass(t, y)
        j = -th.get_mixture_specific_heat_cp_mass(t, y)
        if fixed_iters is None and np.linalg.norm(f / j) <= 1e-10:
            return t
        t = t - f / j
    if fixed_iters is None:
        raise RuntimeError("enthalpy Newton did not converge")
    return t


def flamelet_case(sol, n_x, seed):
    """A seeded flamelet on a uniform mixture-fraction grid: air-like
    oxidizer, diluted-H2 fuel, a hot layer near Z = 0.3 and small radical
    fractions, with random dissipation rates and viscous heating."""
    rng = np.random.default_rng(seed)
    cls = refgen.reference_class(sol)
    ref = cls()
    S = sol.n_species
    idx = sol.species_index
    z = np.linspace(0.0, 1.0, n_x)
    dx = float(z[1] - z[0])
    y_ox = np.zeros(S)
    y_ox[idx("O2")], y_ox[idx("N2")] = 0.233, 0.767
    y_fu = np.zeros(S)
    y_fu[idx("H2")], y_fu[idx("N2")] = 0.1, 0.9
    y = (1.0 - z)[None, :] * y_ox[:, None] + z[None, :] * y_fu[:, None]
    noise = 1e-3 * rng.dirichlet(np.full(S, 0.5), size=n_x).T
    y[:, 1:-1] += noise[:, 1:-1]
    y /= y.sum(axis=0, keepdims=True)
    t = 350.0 + 1650.0 * np.exp(-((z - 0.3) / 0.2) ** 2)
    h = np.asarray(ref.get_mixture_enthalpy_mass(t, y), dtype=np.float64)
    t_guess = t * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, size=n_x))
    chi = 5.0 + 20.0 * rng.random(n_x)
    visc = 1e3 * rng.random(n_x)
    return dict(z=z, dx=np.asarray(dx), y_ox=y_ox, y_fu=y_fu, Y=y, T=t,
                h=h, T_guess=t_guess, chi=chi, visc=visc,
                P=np.asarray(1e5), h_ox=np.asarray(h[0]),
                h_fu=np.asarray(h[-1])), cls, ref


def flamelet_residual_and_blocks(sol, case, cls, ref):
    """The reference's ``FlameletEquations.rhs`` and ``jac``
    (``flamelets/equations.py:167-318``) with its Laplacian block form
    (``onedim_laplacian.py:144-180``) and source terms
    (``equations.py:340-420``), evaluated with the reference's generated
    class: numpy for the residual, torch + ``jacfwd`` (the stand-in for
    the reference's ``jax.vmap(jax.jacfwd(local_source_terms))``) for the
    per-point source Jacobian.  The assembly (masks, boundary rows,
    dissipation scaling) is restated here because the reference's
    ``equations.py`` imports JAX, which is not installed.  As in the
    reference, the boundary dissipation rates are used as given
    (``_enforce_dirichlet_bcs`` builds new arrays with ``.at[].set`` and
    discards them)."""
    import torch
    from torch.func import jacfwd, vmap
    S = sol.n_species
    nv = S + 1
    y, h, dx = case["Y"], case["h"], float(case["dx"])
    n_x = y.shape[1]
    p = float(case["P"])
    chi, visc = case["chi"], case["visc"]
    mw = np.asarray(ref.molecular_weights, dtype=np.float64)
    # residual (numpy)
    t = _enthalpy_newton(ref, h, y, case["T_guess"])
    rho = np.asarray(ref.get_density(p, t, y))
    w = np.array([np.broadcast_to(np.asarray(v, dtype=np.float64), (n_x,))
                  for v in ref.get_net_production_rates(rho, t, y)])
    src = np.vstack([visc / rho, mw[:, None] * w / rho])
    phi = np.vstack([h, y])
    lap = np.empty_like(phi)
    lap[:, 0] = phi[:, 0] / dx ** 2
    lap[:, -1] = phi[:, -1] / dx ** 2
    lap[:, 1:-1] = (phi[:, :-2] - 2.0 * phi[:, 1:-1] + phi[:, 2:]) / dx ** 2
    mask = np.ones(n_x)
    mask[0] = mask[-1] = 0.0
    bc = np.zeros_like(phi)
    bc[0, 0], bc[0, -1] = float(case["h_ox"]), float(case["h_fu"])
    bc[1:, 0], bc[1:, -1] = case["y_ox"], case["y_fu"]
    resid = 0.5 * chi * lap + src * mask - bc
    # per-point source Jacobian (torch, jacfwd)
    th = torch_reference(cls)
    mwt = torch.tensor(mw)

    def local(x, vd, tg, pres):
        hh, yy = x[0], x[1:]
        tt = _enthalpy_newton(th, hh, yy, tg, fixed_iters=40)
        rr = th.get_density(pres, tt, yy)
        ww = th.get_net_production_rates(rr, tt, yy)
        return torch.cat([(vd / rr)[None], mwt * ww / rr])

    xs = torch.tensor(phi.T.copy())
    sj = vmap(jacfwd(local), in_dims=(0, 0, 0, None))(
        xs, torch.tensor(visc), torch.tensor(case["T_guess"]),
        torch.tensor(p)).numpy()
    eye = np.eye(nv)
    sj[0] = 0.0
    sj[-1] = 0.0
    lap_c = np.stack([eye / dx ** 2] + [-2.0 * eye / dx ** 2] * (n_x - 2)
                     + [eye / dx ** 2])
    lap_l = np.stack([eye / dx ** 2] * (n_x - 2) + [0.0 * eye])
    lap_u = np.stack([0.0 * eye] + [eye / dx ** 2] * (n_x - 2))
    central = 0.5 * chi[:, None, None] * lap_c + sj
    lower = 0.5 * chi[1:, None, None] * lap_l
    upper = 0.5 * chi[:-1, None, None] * lap_u
    return dict(T_solved=t, resid=resid, src=src, L=lower, C=central,
                U=upper)


def golden_flamelet(fname="flamelet.npz"):
    out = {}
    for tag, sol, n_x, seed in (
            ("s9", synthetic.config1_mechanism(), 12, 41),
            ("s53", synthetic.config2_mechanism(), 5, 42)):
        case, cls, ref = flamelet_case(sol, n_x, seed)
        case.update(flamelet_residual_and_blocks(sol, case, cls, ref))
        case["mech_yaml"] = np.array(dump_mechanism(sol))
        for k, v in case.items():
            out[f"{tag}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, fname), **out)
    print(f"wrote {fname}")


def eos_adjoint(sol, case, cls, ref, pdf):
    """The reference's compressible-EOS adjoint pieces for one flamelet:
    ``FlameletEquations.adjoint_operator`` (``equations.py:451-516``),
    ``compressible_eos_rt`` and its ``jacfwd`` (``:517-535``,
    ``:136-147``), ``source_gradient_wrt_pressure`` (``:130-134``) and
    ``CompressibleEOS.enthalpy_gradient`` / ``eos_gradient``
    (``thermodynamic_consistency.py:105-307``).  The generated class
    evaluates the chemistry (torch + ``jacfwd`` standing in for the
    reference's ``jax.vmap(jax.jacfwd(...))``), the reference's own
    ``block_thomas`` (numpy ``lax.scan`` stand-in, ``oracle/refgen.py``)
    solves; the assembly and contractions are restated from the
    reference's JAX modules, which cannot be imported here."""
    import torch
    from torch.func import jacfwd, vmap
    S = sol.n_species
    nv = S + 1
    y, h, dx = case["Y"], case["h"], float(case["dx"])
    n_x = y.shape[1]
    p = float(case["P"])
    chi, visc, tg = case["chi"], case["visc"], case["T_guess"]
    mw = np.asarray(ref.molecular_weights, dtype=np.float64)
    th = torch_reference(cls)
    mwt = torch.tensor(mw)

    def local(x, vd, tgi, pres):
        hh, yy = x[0], x[1:]
        tt = _enthalpy_newton(th, hh, yy, tgi, fixed_iters=40)
        rr = th.get_density(pres, tt, yy)
        ww = th.get_net_production_rates(rr, tt, yy)
        return torch.cat([(vd / rr)[None], mwt * ww / rr])

    def local_rt(x, tgi):
        hh, yy = x[0], x[1:]
        tt = _enthalpy_newton(th, hh, yy, tgi, fixed_iters=40)
        return th.gas_constant * tt / th.get_mixture_molecular_weight(yy)

    xs = torch.tensor(np.vstack([h, y]).T.copy())
    args = (xs, torch.tensor(visc), torch.tensor(tg), torch.tensor(p))
    sj = vmap(jacfwd(local), in_dims=(0, 0, 0, None))(*args).numpy()
    ds_dp = vmap(jacfwd(local, argnums=3), in_dims=(0, 0, 0, None))(
        *args).numpy()
    rt_jac = vmap(jacfwd(local_rt), in_dims=(0, 0))(
        xs, torch.tensor(tg)).numpy()
    t = _enthalpy_newton(ref, h, y, tg)
    rt = np.asarray(ref.gas_constant * t
                    / ref.get_mixture_molecular_weight(y))
    # adjoint operator
    eye = np.eye(nv)
    lap_c = np.stack([eye / dx ** 2] + [-2.0 * eye / dx ** 2] * (n_x - 2)
                     + [eye / dx ** 2])
    lap_l = np.stack([eye / dx ** 2] * (n_x - 2) + [0.0 * eye])
    lap_u = np.stack([0.0 * eye] + [eye / dx ** 2] * (n_x - 2))
    zeros = np.zeros((1, nv, nv))
    src = np.concatenate([zeros, np.transpose(
        2 * sj[1:-1] / chi[1:-1, None, None], (0, 2, 1)), zeros])
    central = np.concatenate([
        (0.5 * chi[0] * lap_c[0])[None], lap_c[1:-1],
        (0.5 * chi[-1] * lap_c[-1])[None]]) + src
    bt = refgen.reference_block_thomas()

    def traces(a):
        ox = (1.5 * a[0] + 2 * a[1] - 0.5 * a[2]) / dx ** 2
        fu = (1.5 * a[-1] + 2 * a[-2] - 0.5 * a[-3]) / dx ** 2
        return ox + fu

    def trapezoid(f):
        return 0.5 * (f[0] + f[-1]) + np.sum(f[1:-1])

    unit_h = np.zeros((nv, n_x))
    unit_h[0] = 1.0
    adj_h = np.asarray(bt(lap_l, central, lap_u, (-unit_h * pdf).T)).T
    dsdp = ds_dp / (0.5 * chi[:, None])
    rhs_d = (p / rt ** 2) * rt_jac.T * pdf
    adj_d = np.asarray(bt(lap_l, central, lap_u, rhs_d.T)).T
    integ = (1 / rt) * pdf + np.einsum("ij,ji->i", dsdp, adj_d)
    dens = np.array([trapezoid(integ), traces(adj_d[0])])
    rhs_e = -(unit_h - rt_jac.T) * pdf
    adj_e = np.asarray(bt(lap_l, central, lap_u, rhs_e.T)).T
    integ = np.einsum("ij,ji->i", dsdp, adj_e)
    ener = np.array([trapezoid(integ), traces(adj_e[0])])
    return dict(pdf=pdf, src_jac_all=sj, ds_dp=ds_dp, rt=rt, rt_jac=rt_jac,
                adj_L=lap_l, adj_C=central, adj_U=lap_u, adj_h=adj_h,
                h_gradient=np.asarray(traces(adj_h[0])), adj_d=adj_d,
                adj_e=adj_e, density_gradient=dens, energy_gradient=ener)


def golden_eos_adjoint(fname="eos_adjoint.npz"):
    """Two cases per mechanism: the benchmark mechanism (stiff: its adjoint
    operators have condition numbers of 1e15 and more, so gradients are
    compared stage by stage), and the same mechanism with every rate
    scaled down (``synthetic.scaled_rates``: 1e-12 and 1e-30), whose
    diffusion-dominated adjoint systems are well conditioned, for
    end-to-end gradient comparisons."""
    out = {}
    for tag, sol, n_x, seed in (
            ("s9", synthetic.config1_mechanism(), 12, 41),
            ("s53", synthetic.config2_mechanism(), 8, 43),
            ("s9slow", synthetic.scaled_rates(synthetic.config1_mechanism(),
                                              1e-12), 12, 44),
            ("s53slow", synthetic.scaled_rates(
                synthetic.config2_mechanism(), 1e-30), 8, 45)):
        case, cls, ref = flamelet_case(sol, n_x, seed)
        z = case["z"]
        pdf = 1e-3 + z ** 1.5 * (1.0 - z) ** 2.5
        pdf = pdf / pdf.sum()
        case.update(eos_adjoint(sol, case, cls, ref, pdf))
        case["mech_yaml"] = np.array(dump_mechanism(sol))
        for k, v in case.items():
            out[f"{tag}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, fname), **out)
    print(f"wrote {fname}")


def golden_transport(fname="transport.npz"):
    """The reference's generated transport methods (``python.py:564-641``)
    on the synthetic mechanisms' kinetic-theory fits.  The last two states
    are pure N2 and pure H2 (the ``denom > 0`` branch of
    ``get_species_mass_diffusivities_mixavg`` goes to ``D_kk / p``)."""
    def dense(a):
        a = np.asarray(a)
        if a.dtype == object:
            return np.array([dense(v) for v in a])
        return a.astype(np.float64)

    out = {}
    for tag, sol, n, n_bd, seed in (
            ("s9", synthetic.config1_mechanism(), 64, 16, 51),
            ("s53", synthetic.config2_mechanism(), 32, 3, 52)):
        ref = refgen.reference_class(sol)()
        t, p, y = edge_states(sol, n, seed)
        for col, sp in ((-1, "N2"), (-2, "H2")):
            y[:, col] = 0.0
            y[sol.species_index(sp), col] = 1.0
        tr = sol.transport
        case = dict(
            T=t, P=p, Y=y,
            fit_visc=tr.viscosity, fit_cond=tr.conductivity,
            fit_diff=tr.diffusivity,
            visc=dense(ref.get_species_viscosities(t)),
            cond=dense(ref.get_species_thermal_conductivities(t)),
            bdiff=dense(ref.get_species_binary_mass_diffusivities(
                t[:n_bd])),
            mu_mix=dense(ref.get_mixture_viscosity_mixavg(t, y)),
            lam_mix=dense(ref.get_mixture_thermal_conductivity_mixavg(t,
                                                                      y)),
            d_mix=dense(ref.get_species_mass_diffusivities_mixavg(p, t, y)),
            mech_yaml=np.array(dump_mechanism(sol)))
        for k, v in case.items():
            out[f"{tag}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, fname), **out)
    print(f"wrote {fname}")


# the reference's fixture mechanisms with the fuel and O2/fuel mole ratio
# its kinetics tests use for each (test/test.py:212-217, 377-383), the end
# of the ignition run (s; past 99 % of the temperature rise) and how many
# golden states go to the Jacobian
FIXTURES = (("uiuc", "C2H4", 3.0, 1e-3, 16),
            ("sandiego", "H2", 0.5, 1e-3, 16),
            ("hong", "H2", 0.5, 1e-3, 16),
            ("uconn32", "C2H4", 3.0, 1e-3, 12),
            ("gri30", "CH4", 2.0, 2e-3, 12))


def load_fixture(name):
    from pyrometheus_gb300.yaml_mech import load_mechanism
    path = os.path.join(refgen.REFERENCE_ROOT, "test", "mechs",
                        f"{name}.yaml")
    try:
        return load_mechanism(path, "gas")
    except ValueError:
        return load_mechanism(path)


def golden_fixtures(names=None):
    for k, (name, fuel, stoich, t_end, n_jac) in enumerate(FIXTURES):
        if names and name not in names:
            continue
        sol = load_fixture(name)
        states = fixture_states(sol, fuel, stoich, t_end, n_jac, 32, 60 + k)
        golden(sol, 0, 0, n_jac, f"ref_{name}.npz", states)


def main():
    if not refgen.reference_available():
        raise SystemExit("reference checkout not found: set "
                         "PYRO_REFERENCE_ROOT")
    if sys.argv[1:2] == ["fixtures"]:
        golden_fixtures(sys.argv[2:])
        return
    golden(synthetic.config1_mechanism(), 256, 11, 24, "synthetic9.npz")
    golden(synthetic.config2_mechanism(), 48, 12, 6, "synthetic53.npz")
    golden(quirks_mechanism(), 128, 13, 12, "quirks9.npz")
    golden_block_thomas()
    golden_flamelet()
    golden_transport()
    golden_eos_adjoint()
    golden_fixtures()


if __name__ == "__main__":
    main()
