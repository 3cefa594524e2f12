"""The reactor integrator's numerics on the CPU: ``ReactorPool`` driven by
the oracle backend (numpy source, central-difference Jacobian, LAPACK LU)
against SciPy's variable-order BDF at much tighter tolerances, plus the
starting-step and failure paths.  The GPU tests drive the same pool code
with the CUDA backend."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
scipy_integrate = pytest.importorskip("scipy.integrate")


def _pool(sol, cap=8, **kw):
    from oracle.reactor_backend import OracleReactorBackend
    from pyrometheus_gb300.serving import ReactorPool
    return ReactorPool(OracleReactorBackend(sol), cap, **kw)


def _request(sol, n, t_end, seed=1):
    from pyrometheus_gb300.serving import poisson_requests
    r = poisson_requests(100.0, 1.0, {"m": sol}, seed=seed, cells=(n, n),
                         t_end=t_end)[0]
    r.arrival = 0.0
    return r


def _run(pool, limit=200000):
    it = 0
    while bool(pool.active.any()) and it < limit:
        pool.step()
        it += 1
    return it


def test_bdf2_against_scipy_bdf():
    from oracle.thermo_oracle import Thermochemistry as Oracle
    from pyrometheus_gb300 import synthetic
    sol = synthetic.config1_mechanism()
    orc = Oracle(sol)
    pool = _pool(sol)
    r = _request(sol, 2, 1e-5)
    slots = pool.admit(r)
    _run(pool)
    T, Y, steps, failed = pool.results(slots)
    assert not failed.any() and (steps > 10).all()
    for c in range(r.n):
        x0 = np.concatenate([[r.T0[c]], r.Y0[:, c]])
        ref = scipy_integrate.solve_ivp(
            lambda t, x: orc.reactor_source(r.pressure, x[:1],
                                            x[1:, None])[:, 0],
            (0.0, r.t_end), x0, method="BDF", rtol=1e-11, atol=1e-16)
        assert ref.success
        assert abs(T[c] - ref.y[0, -1]) <= 1e-6 * ref.y[0, -1]
        assert np.abs(Y[:, c] - ref.y[1:, -1]).max() <= 1e-6
        # mass is conserved by the element-balanced mechanism
        assert abs(Y[:, c].sum() - 1.0) <= 1e-10


def test_starting_step_is_positive_and_bounded():
    from pyrometheus_gb300 import synthetic
    sol = synthetic.config1_mechanism()
    pool = _pool(sol)
    r = _request(sol, 3, 1e-3, seed=4)
    slots = pool.admit(r)
    h0 = pool.h[torch.as_tensor(slots)].numpy()
    assert np.all(h0 > 0) and np.all(h0 <= r.t_end)
    assert np.all(pool.jstale[torch.as_tensor(slots)].numpy())


def test_nonfinite_cell_fails_alone():
    from pyrometheus_gb300 import synthetic
    sol = synthetic.config1_mechanism()
    ref_pool, pool = _pool(sol), _pool(sol)
    r = _request(sol, 2, 2e-6, seed=6)
    ref_slots = ref_pool.admit(r)
    _run(ref_pool)
    bad = _request(sol, 2, 2e-6, seed=6)
    bad.T0 = bad.T0.copy()
    bad.T0[0] = np.nan
    slots = pool.admit(bad)
    _run(pool)
    T, Y, steps, failed = pool.results(slots)
    Tr, Yr, sr, fr = ref_pool.results(ref_slots)
    assert failed[0] and not failed[1] and not fr.any()
    # numpy's vectorised exp/log may round a lane differently when another
    # lane of the same vector holds a NaN, so on the CPU the neighbour is
    # compared to tolerance; the GPU test checks bitwise identity
    assert abs(T[1] - Tr[1]) <= 1e-9 * Tr[1]
    assert np.abs(Y[:, 1] - Yr[:, 1]).max() <= 1e-9
