"""Reactor-source Jacobian (warp-per-state kernel) and VJP (thread-per-state
kernel) against the reference's autodiff Jacobian (``torch.func.jacfwd``
through the reference-generated class, stored in the golden vectors), against
central finite differences of the oracle, and against each other.

The reference checks its JAX Jacobian against central differences with an
order-of-convergence criterion (``test/test.py:300-374``: EOC > 1.95 over
delta in {1e-5, 1e-6, 1e-7}); the same criterion is applied here."""

import numpy as np
import pytest

from conftest import GOLDEN_SETS, load_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# Jacobian entries are sums of terms of both signs; compare each row at the
# scale of its largest entry
TOL_ROW = 1e-11


def _cls(sol):
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from pyrometheus_gb300 import get_thermochem_class
    return get_thermochem_class(sol)


def _row_err(j, ref):
    """Row-scaled max error over rows whose reference entries are finite
    (fractional reaction orders at exactly zero concentration have an
    infinite derivative in both)."""
    finite = np.isfinite(ref).all(axis=2, keepdims=True)
    ref = np.where(finite, ref, 0.0)
    j = np.where(finite, j, 0.0)
    scale = np.abs(ref).max(axis=2, keepdims=True)
    scale = np.where(scale == 0, 1.0, scale)
    return (np.abs(j - ref) / scale).max()


@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_source_and_jacobian_against_reference_autodiff(name):
    sol, g = load_golden(name)
    th = _cls(sol)()
    n = g["jac"].shape[0]
    p, t, y = g["P"][:n], g["T"][:n], g["Y"][:, :n]
    src = th.get_reactor_source(p, t, y).cpu().numpy()
    ref = g["reactor_source"]
    assert np.abs(src - ref).max() <= 1e-12 * np.abs(ref).max()
    jac = th.get_reactor_jacobian(p, t, y).cpu().numpy()
    assert _row_err(jac, g["jac"]) < TOL_ROW
    # the non-finite entries are non-finite in both
    assert np.array_equal(np.isfinite(jac), np.isfinite(g["jac"])) or \
        not np.isfinite(g["jac"]).all()


@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_fused_source_and_jacobian(name):
    """One pass for the source and its Jacobian (the primal and tangents of
    the reference's jacfwd): the same Jacobian as the Jacobian-only entry
    point bit for bit, and the source against the reference's golden one
    and the source kernel."""
    sol, g = load_golden(name)
    th = _cls(sol)()
    n = g["jac"].shape[0]
    p, t, y = g["P"][:n], g["T"][:n], g["Y"][:, :n]
    f, jac = th.get_reactor_source_and_jacobian(p, t, y)
    # fractional orders at zero concentration give non-finite entries in
    # both (equal_nan compares those too)
    assert np.array_equal(jac.cpu().numpy(),
                          th.get_reactor_jacobian(p, t, y).cpu().numpy(),
                          equal_nan=True)
    ref = g["reactor_source"]
    f = f.cpu().numpy()
    assert np.abs(f - ref).max() <= 1e-12 * np.abs(ref).max()
    f_sep = th.get_reactor_source(p, t, y).cpu().numpy()
    assert np.abs(f - f_sep).max() <= 1e-13 * np.abs(f_sep).max()
    # into caller buffers, with a leading dimension beyond N
    nc = sol.n_species + 1
    fb = torch.full((nc, n + 5), float("nan"), dtype=torch.float64,
                    device="cuda")
    jb = torch.empty((n, nc, nc), dtype=torch.float64, device="cuda")
    th.get_reactor_source_and_jacobian(p, t, y, out=(fb[:, :n], jb))
    assert np.array_equal(fb[:, :n].cpu().numpy(), f, equal_nan=True)
    assert torch.isnan(fb[:, n:]).all()
    assert np.array_equal(jb.cpu().numpy(), jac.cpu().numpy(),
                          equal_nan=True)


@pytest.mark.parametrize("name", ["synthetic9", "ref_sandiego", "ref_uiuc",
                                  "ref_hong", "synthetic53"])
def test_batch_tails_and_independence(name):
    """Each state's Jacobian is its own group's work: batches of 1, 2, 3,
    5, 7 and 13 states (a warp's last groups past the batch, at four
    states per warp for the small mechanisms) give bit for bit the rows a
    larger batch gives for the same states, and the source of the same
    pass likewise."""
    sol, g = load_golden(name)
    th = _cls(sol)()
    n = g["jac"].shape[0]
    p, t, y = g["P"][:n], g["T"][:n], g["Y"][:, :n]
    full = th.get_reactor_jacobian(p, t, y).cpu().numpy()
    ffull, _ = th.get_reactor_source_and_jacobian(p, t, y)
    ffull = ffull.cpu().numpy()
    for m in (1, 2, 3, 5, 7, 13):
        if m > n:
            continue
        for start in (0, n - m):
            sl = slice(start, start + m)
            jm = th.get_reactor_jacobian(p[sl], t[sl], y[:, sl])
            jm = jm.cpu().numpy().reshape(m, *full.shape[1:])
            assert np.array_equal(jm, full[sl], equal_nan=True), (m, start)
            fm, _ = th.get_reactor_source_and_jacobian(p[sl], t[sl],
                                                       y[:, sl])
            fm = fm.cpu().numpy().reshape(ffull.shape[0], m)
            assert np.array_equal(fm, ffull[:, sl], equal_nan=True)


@pytest.mark.parametrize("which", ["wide9", "mid18"])
def test_small_and_mid_size_mechanisms(which):
    """Mechanisms on the sub-warp state groups outside the golden sets: 9
    species with 60 reactions (8-lane groups, 44 states per CTA after
    rounding to whole warps) and 18 species with 40 reactions (16-lane
    groups, two states per warp).  Central differences of the oracle
    source converge to the CUDA Jacobian at second order, and sub-batches
    give the same rows bit for bit."""
    from oracle.thermo_oracle import Thermochemistry as Oracle
    from pyrometheus_gb300 import synthetic
    if which == "wide9":
        sol = synthetic.make_mechanism(synthetic.SPECIES_9, 60, 6, 4, 2,
                                       seed=5, name="wide9",
                                       orient_temperature=1500.0)
    else:
        sol = synthetic.make_mechanism(
            list(synthetic.SPECIES_53[:17]) + ["N2"], 40, 5, 3, 1, seed=7,
            name="mid18", orient_temperature=1500.0)
    th = _cls(sol)()
    orc = Oracle(sol)
    t, p, y = synthetic.sample_states(sol, 45, seed=9)
    full = th.get_reactor_jacobian(p, t, y).cpu().numpy()
    for m in (1, 3, 13):
        jm = th.get_reactor_jacobian(p[-m:], t[-m:], y[:, -m:])
        jm = jm.cpu().numpy().reshape(m, *full.shape[1:])
        assert np.array_equal(jm, full[-m:], equal_nan=True)
    errs = []
    deltas = [1e-3, 1e-4, 1e-5]
    for rel in deltas:
        jfd = orc.reactor_jacobian_fd(p[:2], t[:2], y[:, :2], rel=rel,
                                      absolute_y=True)
        errs.append(np.linalg.norm(full[:2] - jfd) / np.linalg.norm(full[:2]))
    order = np.polyfit(np.log(deltas), np.log(errs), 1)[0]
    assert order > 1.95, (errs, order)


def test_jacobian_order_of_convergence_like_reference():
    """Central differences of the oracle source converge to the CUDA
    Jacobian at second order (test/test.py:360-374)."""
    from oracle.thermo_oracle import Thermochemistry as Oracle
    sol, g = load_golden("synthetic9")
    th = _cls(sol)()
    orc = Oracle(sol)
    p, t, y = g["P"][5:7], g["T"][5:7], g["Y"][:, 5:7]
    jac = th.get_reactor_jacobian(p, t, y).cpu().numpy()
    errs = []
    deltas = [1e-3, 1e-4, 1e-5]
    for rel in deltas:
        jfd = orc.reactor_jacobian_fd(p, t, y, rel=rel, absolute_y=True)
        errs.append(np.linalg.norm(jac - jfd) / np.linalg.norm(jac))
    order = np.polyfit(np.log(deltas), np.log(errs), 1)[0]
    assert order > 1.95, (errs, order)


def test_vjp_matches_jacobian_transpose():
    from pyrometheus_gb300 import synthetic
    sol, _ = load_golden("synthetic53")
    th = _cls(sol)()
    n = 257
    t, p, y = synthetic.sample_states(sol, n, seed=3)
    rng = np.random.default_rng(4)
    v = rng.standard_normal((sol.n_species + 1, n))
    jac = th.get_reactor_jacobian(p, t, y).cpu().numpy()
    gT, gY, gp = th.get_reactor_vjp(p, t, y, v)
    vj = np.einsum("in,nij->nj", v, jac)
    scale = (np.abs(v).T[:, :, None] * np.abs(jac)).sum(axis=1)
    # entries far below their row's largest one come out of cancelling
    # terms of the row's size (the dT/dt row sums H_k times dw_k/dY), so
    # both computations carry an absolute error of a few ulps of the row
    # scale there: allow 1e-15 of sum_i |v_i| max_j |J_ij| on top
    floor = 1e-15 * (np.abs(v).T * np.abs(jac).max(axis=2)).sum(axis=1)
    got = np.concatenate([gT.cpu().numpy()[None, :], gY.cpu().numpy()]).T
    assert np.all(np.abs(got - vj) <= 1e-12 * scale + floor[:, None])
    # dp through finite differences of the source
    fp = th.get_reactor_source(p * (1 + 1e-6), t, y).cpu().numpy()
    fm = th.get_reactor_source(p * (1 - 1e-6), t, y).cpu().numpy()
    dfdp = (fp - fm) / (2e-6 * p)
    gp_fd = (v * dfdp).sum(axis=0)
    gps = gp.cpu().numpy()
    assert np.all(np.abs(gps - gp_fd) <= 1e-6 * np.abs(v * dfdp).sum(axis=0))


def test_autograd_function():
    from pyrometheus_gb300 import synthetic
    sol, _ = load_golden("synthetic9")
    th = _cls(sol)()
    n = 64
    t, p, y = synthetic.sample_states(sol, n, seed=8)
    T = torch.tensor(t, device="cuda", requires_grad=True)
    Y = torch.tensor(y, device="cuda", requires_grad=True)
    P = torch.tensor(p, device="cuda", requires_grad=True)
    f = th.reactor_source(P, T, Y)
    v = torch.randn_like(f)
    (f * v).sum().backward()
    gT, gY, gp = th.get_reactor_vjp(p, t, y, v)
    assert torch.allclose(T.grad, gT, rtol=0, atol=0)
    assert torch.allclose(Y.grad, gY, rtol=0, atol=0)
    assert torch.allclose(P.grad, gp, rtol=0, atol=0)
