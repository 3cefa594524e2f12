"""The CUDA flamelet assembly (``FlameletEquations`` on the GPU) against
the golden vectors (reference-generated chemistry and autodiff) and the
oracle, single and packed, plus one Newton correction through the batched
block-Thomas solver."""

import numpy as np
import pytest

from test_flamelet import TAGS, _golden, _resid_scale, _source_part

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _eqs(sol, lengths, dx, y_ox, y_fu):
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from pyrometheus_gb300 import get_thermochem_class
    from pyrometheus_gb300.flamelet import FlameletEquations
    th = get_thermochem_class(sol)()
    return FlameletEquations(th, lengths, dx, y_ox, y_fu)


def _row_err(j, ref):
    scale = np.abs(ref).max(axis=2, keepdims=True)
    scale = np.where(scale == 0, 1.0, scale)
    return (np.abs(j - ref) / scale).max()


@pytest.mark.parametrize("tag", TAGS)
def test_residual_and_blocks_against_golden(tag):
    sol, d = _golden(tag)
    n_x = d["h"].shape[0]
    eq = _eqs(sol, [n_x], float(d["dx"]), d["y_ox"], d["y_fu"])
    args = (d["h"], torch.as_tensor(d["Y"]), d["chi"], d["visc"],
            d["T_guess"], float(d["P"]))
    R = eq.rhs(*args, float(d["h_ox"]), float(d["h_fu"])).cpu().numpy()
    assert np.all(np.abs(R - d["resid"]) <= 1e-12 * _resid_scale(d))
    L, C, U = (x.cpu().numpy() for x in eq.jac(*args))
    assert np.array_equal(L[:-1], d["L"]) and np.array_equal(U[:-1],
                                                             d["U"])
    assert not L[-1].any() and not U[-1].any()
    assert _row_err(C, d["C"]) < 1e-10
    assert _row_err(C - (d["C"] - _source_part(d)), _source_part(d)) < 1e-10


def test_packed_flamelets_match_oracle():
    """Three flamelets of different lengths in one call: each slice of the
    packed residual matches the oracle on that flamelet alone."""
    from oracle.flamelet_oracle import FlameletOracle
    sol, d = _golden("s9")
    rng = np.random.default_rng(9)
    lengths = [7, 12, 4]
    dxs = [1.0 / (n - 1) for n in lengths]
    hs, ys, chis, viscs, tgs = [], [], [], [], []
    for n in lengths:
        z = np.linspace(0.0, 1.0, n)
        y = np.interp(z, np.linspace(0, 1, d["Y"].shape[1]),
                      np.arange(d["Y"].shape[1]))
        idx = np.clip(np.round(y).astype(int), 0, d["Y"].shape[1] - 1)
        ys.append(d["Y"][:, idx])
        hs.append(d["h"][idx])
        tgs.append(d["T_solved"][idx] * (1 + 0.01 * rng.uniform(-1, 1, n)))
        chis.append(5 + 10 * rng.random(n))
        viscs.append(100 * rng.random(n))
    eq = _eqs(sol, lengths, dxs, d["y_ox"], d["y_fu"])
    h_ox = np.array([h[0] for h in hs])
    h_fu = np.array([h[-1] for h in hs])
    R = eq.rhs(np.concatenate(hs), torch.as_tensor(np.hstack(ys)),
               np.concatenate(chis), np.concatenate(viscs),
               np.concatenate(tgs), 2e5, h_ox, h_fu).cpu().numpy()
    orc = FlameletOracle(sol)
    r0 = 0
    for s, n in enumerate(lengths):
        ref = orc.residual(hs[s], ys[s], chis[s], viscs[s], tgs[s], 2e5,
                           h_ox[s], h_fu[s], d["y_ox"], d["y_fu"], dxs[s])
        got = R[:, r0:r0 + n]
        scale = np.abs(ref).max(axis=1, keepdims=True) + 1e-300
        assert np.abs(got - ref).max() <= 1e-11 * scale.max(), s
        r0 += n


def test_newton_correction_solves_the_linear_system():
    sol, d = _golden("s9")
    n_x = d["h"].shape[0]
    eq = _eqs(sol, [n_x, n_x], float(d["dx"]), d["y_ox"], d["y_fu"])
    h = np.concatenate([d["h"], d["h"]])
    Y = torch.as_tensor(np.hstack([d["Y"], d["Y"]]))
    chi = np.concatenate([d["chi"], d["chi"]])
    visc = np.concatenate([d["visc"], d["visc"]])
    tg = np.concatenate([d["T_guess"], d["T_guess"]])
    hb = np.array([d["h_ox"], d["h_ox"]]), np.array([d["h_fu"], d["h_fu"]])
    dphi, R, T = eq.newton_step(h, Y, chi, visc, tg, float(d["P"]), *hb)
    L, C, U = (x.cpu().numpy() for x in eq.jac(h, Y, chi, visc, tg,
                                                float(d["P"])))
    x = dphi.cpu().numpy().T           # [rows, nv]
    b = -R.cpu().numpy().T
    for r0 in (0, n_x):
        sl = slice(r0, r0 + n_x)
        Ls, Cs, Us, xs, bs = L[sl], C[sl], U[sl], x[sl], b[sl]
        ax = np.einsum("nij,nj->ni", Cs, xs)
        ax[:-1] += np.einsum("nij,nj->ni", Us[:-1], xs[1:])
        ax[1:] += np.einsum("nij,nj->ni", Ls[:-1], xs[:-1])
        scale = (np.abs(Cs).sum(axis=2).max() * np.abs(xs).max()
                 + np.abs(bs).max())
        assert np.abs(ax - bs).max() <= 1e-11 * scale
    # both copies of the flamelet get the same correction
    assert np.allclose(x[:n_x], x[n_x:], rtol=1e-12, atol=0)


def _lap(v, dx):
    lap = np.empty_like(v)
    lap[:, 0] = v[:, 0] / dx ** 2
    lap[:, -1] = v[:, -1] / dx ** 2
    lap[:, 1:-1] = (v[:, :-2] - 2.0 * v[:, 1:-1] + v[:, 2:]) / dx ** 2
    return lap


@pytest.mark.parametrize("tag", ["s9", "s53", "s9slow", "s53slow"])
def test_jacobian_action_against_reference_autodiff(tag):
    """The device ``jacobian_action`` (``equations.py:411-450``) against
    chi/2 Lap(v) + dS/dphi v with the golden per-point source Jacobians of
    every point -- jacfwd through the reference's generated class and its
    enthalpy Newton, the boundary points included -- and against the
    oracle's ``jacobian_action`` (central differences)."""
    import os

    from conftest import GOLDEN
    from oracle.flamelet_oracle import FlameletOracle
    from pyrometheus_gb300.yaml_mech import load_mechanism
    g = np.load(os.path.join(GOLDEN, "eos_adjoint.npz"))
    d = {k[len(tag) + 1:]: g[k] for k in g.files
         if k.startswith(tag + "_")}
    sol = load_mechanism(f"{tag}.yaml", text=str(d["mech_yaml"]))
    n_x = d["h"].shape[0]
    dx = float(d["dx"])
    eq = _eqs(sol, [n_x], dx, d["y_ox"], d["y_fu"])
    v = np.random.default_rng(3).standard_normal((sol.n_species + 1, n_x))
    args = (d["h"], torch.as_tensor(d["Y"]), d["chi"], d["visc"],
            d["T_guess"], float(d["P"]))
    A = eq.jacobian_action(torch.as_tensor(v), *args).cpu().numpy()
    sj = d["src_jac_all"]
    terms = np.abs(0.5 * d["chi"] * _lap(v, dx)) + np.einsum(
        "ijk,ki->ji", np.abs(sj), np.abs(v))
    ref = 0.5 * d["chi"] * _lap(v, dx) + np.einsum("ijk,ki->ji", sj, v)
    # at the scale of the terms summed (the source Jacobian's rows span
    # many decades), as for the blocks
    assert np.all(np.abs(A - ref) <= 1e-10 * terms.max(axis=1,
                                                       keepdims=True))
    # boundary points keep their source Jacobians: the action there is
    # not just chi/2 v/dx^2
    assert np.abs(A[:, [0, -1]] - (0.5 * d["chi"] * _lap(v, dx))[:, [0, -1]]
                  ).max() > 0
    if tag.endswith("slow"):
        # central differences resolve the slow-chemistry source Jacobians
        # (the stiff ones, entries to 1e14, only the autodiff pins)
        fo = FlameletOracle(sol)
        ref_fd = fo.jacobian_action(v, d["h"], d["Y"], d["chi"], d["visc"],
                                    d["T_guess"], float(d["P"]), dx)
        assert np.all(np.abs(A - ref_fd) <= 1e-6 * terms.max(
            axis=1, keepdims=True))


@pytest.mark.parametrize("tag", TAGS)
def test_public_source_terms_eos_and_boundary_conditions(tag):
    """``equation_of_state``, ``source_terms`` and ``boundary_conditions``
    (``equations.py:284-409``) against the golden values from the
    reference's generated class."""
    sol, d = _golden(tag)
    n_x = d["h"].shape[0]
    eq = _eqs(sol, [n_x], float(d["dx"]), d["y_ox"], d["y_fu"])
    Y = torch.as_tensor(d["Y"])
    rho, T = eq.equation_of_state(d["h"], Y, d["T_guess"], float(d["P"]))
    assert np.abs(T.cpu().numpy() - d["T_solved"]).max() < 1e-10
    sh, sy = eq.source_terms(d["h"], Y, d["visc"], d["T_guess"],
                             float(d["P"]))
    src = np.vstack([sh.cpu().numpy()[None], sy.cpu().numpy()])
    scale = np.abs(d["src"]).max(axis=1, keepdims=True)
    assert np.all(np.abs(src - d["src"]) <= 1e-12 * scale)
    bh, by = eq.boundary_conditions(float(d["h_ox"]), float(d["h_fu"]))
    bh, by = bh.cpu().numpy(), by.cpu().numpy()
    assert bh[0] == float(d["h_ox"]) and bh[-1] == float(d["h_fu"])
    assert not bh[1:-1].any() and not by[:, 1:-1].any()
    assert np.array_equal(by[:, 0], d["y_ox"])
    assert np.array_equal(by[:, -1], d["y_fu"])
