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
