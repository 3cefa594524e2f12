"""The reactor server on the GPU, on both integrator paths (the fused
per-cell kernel and the batched tensor path): a request's result is
bit-identical alone and in a mix (per-cell integration), agrees with a
tight CPU BDF integration of the oracle's source, the two paths agree with
each other, and a non-finite cell fails on its own without disturbing the
others."""

import numpy as np
import pytest

from conftest import load_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _server(budget=2e8, fused=True):
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from pyrometheus_gb300 import get_thermochem_class
    from pyrometheus_gb300.serving import ReactorServer
    s9, _ = load_golden("synthetic9")
    s53, _ = load_golden("synthetic53")
    th = {"s9": get_thermochem_class(s9)(), "s53": get_thermochem_class(s53)()}
    return (ReactorServer.from_thermos(th, budget, fused=fused),
            {"s9": s9, "s53": s53})


def _reqs(mechs, seed, n_req, cells=(1, 40)):
    from pyrometheus_gb300.serving import poisson_requests
    reqs = poisson_requests(1e4, 1.0, mechs, seed=seed, cells=cells,
                            t_end=1e-4)
    return reqs[:n_req]


@pytest.mark.parametrize("fused", [True, False])
def test_alone_and_in_mix_are_identical(fused):
    server, mechs = _server(fused=fused)
    reqs = _reqs(mechs, seed=1, n_req=6)
    target = reqs[2]
    import copy
    alone = copy.deepcopy(target)
    alone.arrival = 0.0
    server.run([alone], time_limit=120.0)
    assert alone.status == "done"
    server2, _ = _server(fused=fused)
    mix = [copy.deepcopy(r) for r in reqs]
    for r in mix:
        r.arrival *= 1e-3
    server2.run(mix, time_limit=300.0)
    got = [r for r in mix if r.rid == target.rid][0]
    assert got.status == "done"
    assert np.array_equal(got.T, alone.T) and np.array_equal(got.Y, alone.Y)
    assert np.array_equal(got.steps, alone.steps)


@pytest.mark.parametrize("fused", [True, False])
def test_accuracy_against_cpu_bdf(fused):
    scipy_integrate = pytest.importorskip("scipy.integrate")
    from oracle.thermo_oracle import Thermochemistry as Oracle
    server, mechs = _server(fused=fused)
    sol = mechs["s9"]
    orc = Oracle(sol)
    reqs = _reqs({"s9": sol}, seed=3, n_req=1, cells=(3, 3))
    r = reqs[0]
    r.arrival = 0.0
    server.run([r], time_limit=120.0)
    assert r.status == "done"
    for c in range(r.n):
        x0 = np.concatenate([[r.T0[c]], r.Y0[:, c]])

        def rhs(t, x):
            return orc.reactor_source(r.pressure, x[:1], x[1:, None])[:, 0]

        ref = scipy_integrate.solve_ivp(rhs, (0.0, r.t_end), x0,
                                        method="BDF", rtol=1e-11,
                                        atol=1e-16)
        assert ref.success
        xe = ref.y[:, -1]
        assert abs(r.T[c] - xe[0]) <= 1e-5 * xe[0]
        assert np.abs(r.Y[:, c] - xe[1:]).max() <= 1e-5 * np.abs(xe[1:]).max()


def test_accuracy_53_species_against_cpu_bdf():
    """A reacting 53-species request (C2H4/O2/N2, the mixture the serving
    benchmark uses on that mechanism) on the server's default path for it
    (the batched path: analytic Jacobian, batched LU) against a tight SciPy
    BDF integration of the oracle's source, at the 9-species test's
    tolerance; the cells have reacted by then (temperature and composition
    moved well beyond it)."""
    scipy_integrate = pytest.importorskip("scipy.integrate")
    from oracle.thermo_oracle import Thermochemistry as Oracle
    from pyrometheus_gb300.serving import poisson_requests
    server, mechs = _server(fused=None)
    sol = mechs["s53"]
    assert not server.pools["s53"].fused
    orc = Oracle(sol)
    r = poisson_requests(1e4, 1.0, {"s53": sol}, seed=11, cells=(2, 2),
                         t_end=2e-5, fuels={"s53": ("C2H4", 1.0 / 3.0)})[0]
    r.T0 = np.array([1500.0, 1750.0])
    r.arrival = 0.0
    server.run([r], time_limit=300.0)
    assert r.status == "done"

    def rhs(t, x):
        x = x.reshape(sol.n_species + 1, -1)
        return orc.reactor_source(r.pressure, x[0], x[1:])

    for c in range(r.n):
        x0 = np.concatenate([[r.T0[c]], r.Y0[:, c]])
        ref = scipy_integrate.solve_ivp(rhs, (0.0, r.t_end), x0,
                                        method="BDF", rtol=1e-11,
                                        atol=1e-16, vectorized=True)
        assert ref.success
        xe = ref.y[:, -1]
        assert np.abs(xe[1:] - x0[1:]).max() > 1e-4     # it reacted
        assert abs(r.T[c] - xe[0]) <= 1e-5 * xe[0]
        assert np.abs(r.Y[:, c] - xe[1:]).max() <= 1e-5 * np.abs(xe[1:]).max()


def test_fused_and_batched_paths_agree():
    """Same requests through both paths: the fused kernel forms its
    Jacobian by differences, the batched path analytically, so the step
    sequences differ; both must land within the integration tolerance."""
    import copy
    got = {}
    for fused in (True, False):
        server, mechs = _server(fused=fused)
        reqs = _reqs(mechs, seed=7, n_req=3, cells=(2, 6))
        for r in reqs:
            r.arrival = 0.0
        server.run([copy.deepcopy(r) for r in reqs], time_limit=300.0)
        got[fused] = {r.rid: r for r in server.done}
    for rid, a in got[True].items():
        b = got[False][rid]
        assert a.status == "done" and b.status == "done"
        assert np.abs(a.T - b.T).max() <= 1e-5 * np.abs(b.T).max()
        assert np.abs(a.Y - b.Y).max() <= 1e-6


def test_nonfinite_cell_fails_alone():
    server, mechs = _server()
    reqs = _reqs(mechs, seed=5, n_req=3)
    bad = reqs[1]
    bad.T0 = bad.T0.copy()
    bad.T0[0] = np.nan
    for r in reqs:
        r.arrival = 0.0
    server.run(reqs, time_limit=300.0)
    st = {r.rid: r.status for r in reqs}
    assert st[bad.rid].startswith("failed")
    assert all(st[r.rid] == "done" for r in reqs if r is not bad)
