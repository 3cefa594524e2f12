"""The compressible-EOS consistency pieces on the GPU: the adjoint operator
(``pyro_flamelet_adjoint_blocks``), ``R T`` and its gradient
(``pyro_flamelet_eos_rt``), the block-Thomas re-solve with kept factors
(``pyro_block_thomas_resolve``) and the batched adjoint enthalpy / EOS
gradients of ``FlameletEquations``, against golden vectors restated from
the reference (``pyrometheus/flamelets/equations.py:451-535``,
``thermodynamic_consistency.py:105-307``) and the oracle.

The source Jacobian inside the adjoint operator is the analytic one
(matched to the reference's forward-mode one at 1e-10 per row, as in the
flamelet Jacobian tests).  The benchmark mechanisms are so stiff that
their adjoint operators have condition numbers of 1e15 and more (a 1e-13
change of the Jacobian moves the gradients by O(1), in the reference as
here), so for them each later stage is checked on the GPU's own inputs at
its own rounding level; the slow-chemistry variants, whose adjoint systems
are well conditioned, are compared end to end."""

import numpy as np
import pytest

from test_eos_adjoint import TAGS, eos_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _eqs(sol, lengths, dx, y_ox, y_fu):
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from pyrometheus_gb300 import get_thermochem_class
    from pyrometheus_gb300.flamelet import FlameletEquations
    th = get_thermochem_class(sol)()
    return FlameletEquations(th, lengths, dx, y_ox, y_fu)


def _np(x):
    return x.detach().cpu().numpy()


def _args(g):
    return (g["h"], torch.as_tensor(g["Y"]), g["chi"], g["visc"],
            g["T_guess"], float(g["P"]))


@pytest.mark.parametrize("tag", TAGS)
def test_adjoint_operator_and_rt(tag):
    sol, g = eos_golden(tag)
    n_x = g["h"].shape[0]
    dx = float(g["dx"])
    eq = _eqs(sol, [n_x], dx, g["y_ox"], g["y_fu"])
    L, C, U = (_np(x) for x in eq.adjoint_operator(*_args(g)))
    assert np.array_equal(L[:-1], g["adj_L"])
    assert np.array_equal(U[:-1], g["adj_U"])
    assert not L[-1].any() and not U[-1].any()
    # boundary rows exactly; interior element (a, b) is (2/chi) dS_b/dphi_a
    # (+ the Laplacian on the diagonal): compared at 1e-10 of the source
    # Jacobian's row b (the flamelet Jacobian's criterion) plus a few ulps
    # of the element itself
    assert np.array_equal(C[0], g["adj_C"][0])
    assert np.array_equal(C[-1], g["adj_C"][-1])
    ref = g["adj_C"][1:-1]
    rows = np.abs(g["src_jac_all"][1:-1]).max(axis=2)        # [n, b]
    scale = (2.0 / g["chi"][1:-1])[:, None, None] * rows[:, None, :]
    tol = 1e-10 * scale + 4 * np.finfo(float).eps * np.abs(ref)
    assert np.all(np.abs(C[1:-1] - ref) <= tol)
    rt, rtj = eq.eos_rt(g["h"], torch.as_tensor(g["Y"]), g["T_guess"])
    assert np.all(np.abs(_np(rt) - g["rt"]) <= 1e-12 * np.abs(g["rt"]))
    ref = g["rt_jac"].T
    scale = np.abs(ref).max(axis=0, keepdims=True)
    assert np.all(np.abs(_np(rtj) - ref) <= 1e-11 * scale)


@pytest.mark.parametrize("tag", TAGS)
def test_source_gradient_wrt_pressure(tag):
    """Forward-mode dS/dp (homogeneity of the rates in the concentrations
    and [M]) against the golden forward-mode derivative through the
    reference's generated class, per point at 1e-10 of its largest entry;
    the reactor-level derivative against the VJP kernel's pressure
    cotangent for unit cotangents."""
    sol, g = eos_golden(tag)
    n_x = g["h"].shape[0]
    eq = _eqs(sol, [n_x], float(g["dx"]), g["y_ox"], g["y_fu"])
    got = _np(eq.source_gradient_wrt_pressure(
        g["h"], torch.as_tensor(g["Y"]), g["visc"], g["T_guess"],
        float(g["P"])))
    ref = g["ds_dp"]
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(got - ref) <= 1e-10 * scale), \
        float((np.abs(got - ref) / scale).max())
    th = eq.th
    T = eq.temperature(g["h"], torch.as_tensor(g["Y"]), g["T_guess"])
    Y = torch.as_tensor(g["Y"], device="cuda")
    p = float(g["P"])
    dfdp = _np(th.get_reactor_source_dp(p, T, Y))
    nv = dfdp.shape[0]
    for k in range(nv):
        cot = torch.zeros((nv, n_x), dtype=torch.float64, device="cuda")
        cot[k] = 1.0
        _, _, gp = th.get_reactor_vjp(p, T, Y, cot)
        gp = _np(gp)
        assert np.all(np.abs(dfdp[k] - gp) <= 1e-10 * np.abs(dfdp).max(
            axis=0) + 1e-300), k


@pytest.mark.parametrize("nv,kernel", [(10, "cta"), (10, "small"),
                                       (54, "cta")])
def test_resolve_matches_fresh_solves(nv, kernel):
    """Right-hand sides solved with the kept factors equal full solves."""
    from oracle.block_thomas_oracle import make_systems, solve_packed
    from pyrometheus_gb300.flamelet import BlockThomasSolver
    lengths, lo, c, up, b = make_systems(12, nv, n_min=3, n_max=40, seed=nv)
    rows = int(np.sum(lengths))
    rng = np.random.default_rng(5)
    extra = rng.standard_normal((5, rows, nv))
    dev = torch.device("cuda")
    L = torch.as_tensor(lo, device=dev).contiguous()
    C = torch.as_tensor(c, device=dev).contiguous()
    U = torch.as_tensor(up, device=dev).contiguous()
    bt = BlockThomasSolver(nv, lengths, device=dev, kernel=kernel)
    with pytest.raises(RuntimeError):
        bt.resolve(L, U, torch.as_tensor(extra[0], device=dev))
    x0 = bt.solve(L, C, U, torch.as_tensor(b, device=dev).contiguous())
    X = bt.resolve(L, U, torch.as_tensor(extra, device=dev).contiguous())
    x1 = bt.resolve(L, U, torch.as_tensor(extra[2], device=dev))
    bt.check_status()
    X = _np(X)
    assert np.array_equal(_np(x1), X[2])
    for q in range(5):
        ref = solve_packed(lengths, lo, c, up, extra[q])
        assert np.abs(X[q] - ref).max() <= 1e-10 * np.abs(ref).max()
    ref = solve_packed(lengths, lo, c, up, b)
    assert np.abs(_np(x0) - ref).max() <= 1e-10 * np.abs(ref).max()


def _backward_error(L, C, U, x, b):
    """Normwise backward error of x for the packed single system."""
    from oracle.block_thomas_oracle import dense_matrix
    A = dense_matrix(L[:-1], C, U[:-1])
    xf, bf = x.reshape(-1), b.reshape(-1)
    r = A @ xf - bf
    return np.abs(r).max() / (np.abs(A).sum(axis=1).max()
                              * np.abs(xf).max() + np.abs(bf).max())


@pytest.mark.parametrize("tag", TAGS)
def test_gradient_stages(tag):
    """Every stage on the GPU's own inputs: the three adjoint solves by
    their backward error against the GPU's adjoint blocks (the stiff
    mechanisms' operators are too ill-conditioned for a forward-error
    comparison), the boundary traces and the trapezoidal pressure
    integrals against the reference's formulas on the GPU's adjoint
    states, with the golden forward-mode dS/dp."""
    from oracle.flamelet_oracle import FlameletOracle
    sol, g = eos_golden(tag)
    n_x = g["h"].shape[0]
    dx = float(g["dx"])
    p = float(g["P"])
    eq = _eqs(sol, [n_x], dx, g["y_ox"], g["y_fu"])
    rt, adj_h, hg = eq.enthalpy_gradient(*_args(g), g["pdf"])
    (dens, ener), (adj_d, adj_e) = eq.eos_gradient(*_args(g), g["pdf"])
    L, C, U = (_np(x) for x in eq.adjoint_operator(*_args(g)))
    rtg, rtj = (_np(x) for x in eq.eos_rt(g["h"], torch.as_tensor(g["Y"]),
                                         g["T_guess"]))
    pdf = g["pdf"]
    nv = C.shape[1]
    unit_h = np.zeros((nv, n_x))
    unit_h[0] = 1.0
    for adj, rhs in ((adj_h, -unit_h * pdf),
                     (adj_d, (p / rtg ** 2) * rtj * pdf),
                     (adj_e, -(unit_h - rtj) * pdf)):
        assert _backward_error(L, C, U, _np(adj).T, rhs.T) < 1e-13
    fo = FlameletOracle(sol)
    for got, adj in ((hg[0], adj_h), (dens[1, 0], adj_d),
                     (ener[1, 0], adj_e)):
        a = _np(adj)[0]
        ref = fo._traces(a, dx)
        mag = (np.abs(a[:3]).sum() + np.abs(a[-3:]).sum()) * 2 / dx ** 2
        assert abs(float(got) - ref) <= 1e-13 * mag
    dsdp = g["ds_dp"] / (0.5 * g["chi"][:, None])
    for got, adj, base in ((dens[0, 0], adj_d, pdf / g["rt"]),
                           (ener[0, 0], adj_e, 0.0 * pdf)):
        terms = np.einsum("ij,ji->i", dsdp, _np(adj))
        integ = base + terms
        ref = 0.5 * (integ[0] + integ[-1]) + integ[1:-1].sum()
        mag = np.abs(base).sum() + np.abs(dsdp * _np(adj).T).sum()
        assert abs(float(got) - ref) <= 1e-11 * mag, (float(got), ref)
    assert tuple(rt.shape) == (n_x,)


@pytest.mark.parametrize("tag", ["s9slow", "s53slow"])
def test_gradients_end_to_end(tag):
    """Slow chemistry (well-conditioned adjoint systems): the batched
    gradients and adjoint states against the reference-derived golden
    values."""
    sol, g = eos_golden(tag)
    n_x = g["h"].shape[0]
    eq = _eqs(sol, [n_x], float(g["dx"]), g["y_ox"], g["y_fu"])
    _, adj_h, hg = eq.enthalpy_gradient(*_args(g), g["pdf"])
    (dens, ener), (adj_d, adj_e) = eq.eos_gradient(*_args(g), g["pdf"])
    errs = {}
    for k, got, ref in (("h_gradient", _np(hg)[0], g["h_gradient"]),
                        ("density", _np(dens)[:, 0], g["density_gradient"]),
                        ("energy", _np(ener)[:, 0], g["energy_gradient"])):
        errs[k] = float(np.max(np.abs(got - ref) / np.abs(ref)))
    for k, got, ref in (("adj_h", adj_h, g["adj_h"]),
                        ("adj_d", adj_d, g["adj_d"]),
                        ("adj_e", adj_e, g["adj_e"])):
        errs[k] = float(np.abs(_np(got) - ref).max() / np.abs(ref).max())
    assert max(errs.values()) < 1e-8, errs


def test_packed_flamelets_match_single():
    """Flamelets packed in one call give each flamelet's gradients as when
    it is solved alone."""
    sol, g = eos_golden("s9")
    n = g["h"].shape[0]
    dx = float(g["dx"])
    lengths = [n, n, n]
    rng = np.random.default_rng(3)
    scale = [1.0, 1.3, 0.7]
    h = np.concatenate([g["h"]] * 3)
    Y = np.concatenate([g["Y"]] * 3, axis=1)
    chi = np.concatenate([g["chi"] * s for s in scale])
    visc = np.concatenate([g["visc"]] * 3)
    tg = np.concatenate([g["T_guess"]] * 3)
    pdf = np.concatenate([g["pdf"] * (1 + 0.1 * rng.random(n))
                          for _ in range(3)])
    eq = _eqs(sol, lengths, dx, g["y_ox"], g["y_fu"])
    (dens, ener), _ = eq.eos_gradient(h, torch.as_tensor(Y), chi, visc, tg,
                                      float(g["P"]), pdf)
    _, _, hg = eq.enthalpy_gradient(h, torch.as_tensor(Y), chi, visc, tg,
                                    float(g["P"]), pdf)
    for s in range(3):
        sl = slice(s * n, (s + 1) * n)
        one = _eqs(sol, [n], dx, g["y_ox"], g["y_fu"])
        (d1, e1), _ = one.eos_gradient(g["h"], torch.as_tensor(g["Y"]),
                                       chi[sl], g["visc"], g["T_guess"],
                                       float(g["P"]), pdf[sl])
        _, _, h1 = one.enthalpy_gradient(g["h"], torch.as_tensor(g["Y"]),
                                         chi[sl], g["visc"], g["T_guess"],
                                         float(g["P"]), pdf[sl])
        assert np.array_equal(_np(dens[:, s]), _np(d1[:, 0]))
        assert np.array_equal(_np(ener[:, s]), _np(e1[:, 0]))
        assert float(hg[s]) == float(h1[0])
