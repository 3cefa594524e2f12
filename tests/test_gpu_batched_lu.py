"""Batched LU kernels (warp per system) and the per-cell norm kernel on the
GPU, through the C ABI, against LAPACK (``scipy.linalg``) and numpy."""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
scipy_linalg = pytest.importorskip("scipy.linalg")
pytestmark = pytest.mark.gpu


def _libs():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from pyrometheus_gb300 import native
    return native.batched_lu_lib(), native.reactor_step_lib()


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("nv", [1, 10, 33, 54, 64])
def test_factor_and_solve_against_lapack(nv):
    lu, _ = _libs()
    n = 301
    rng = np.random.default_rng(nv)
    A = rng.standard_normal((n, nv, nv)) + np.eye(nv) * rng.uniform(
        0.0, 3.0, size=(n, 1, 1))
    b = rng.standard_normal((nv, n))          # species-major right sides
    mask = (rng.random(n) < 0.8).astype(np.uint8)
    M = torch.as_tensor(A, device="cuda").contiguous()
    piv = torch.zeros((n, nv), dtype=torch.int32, device="cuda")
    mk = torch.as_tensor(mask, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lu.pyro_batched_lu_factor(M.data_ptr(), piv.data_ptr(),
                                     mk.data_ptr(), n, nv, st.data_ptr(),
                                     _stream()) == 0
    B = torch.as_tensor(b, device="cuda").contiguous()
    X = torch.full_like(B, 7.0)
    assert lu.pyro_batched_lu_solve(
        M.data_ptr(), piv.data_ptr(), mk.data_ptr(), B.data_ptr(), 1, n,
        X.data_ptr(), 1, n, n, nv, _stream()) == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    Mh, ph, Xh = M.cpu().numpy(), piv.cpu().numpy(), X.cpu().numpy()
    for s in range(n):
        if not mask[s]:
            assert np.array_equal(Mh[s], A[s]) and np.all(Xh[:, s] == 7.0)
            continue
        lu_ref, piv_ref = scipy_linalg.lu_factor(A[s])
        assert np.array_equal(ph[s], piv_ref)
        assert np.abs(Mh[s] - lu_ref).max() <= 1e-12 * np.abs(lu_ref).max()
        x_ref = np.linalg.solve(A[s], b[:, s])
        cond = np.linalg.cond(A[s])
        assert np.abs(Xh[:, s] - x_ref).max() <= \
            1e-13 * cond * np.abs(x_ref).max() + 1e-300


def test_solve_in_place_row_major_and_singular_flag():
    lu, _ = _libs()
    n, nv = 64, 12
    rng = np.random.default_rng(3)
    A = rng.standard_normal((n, nv, nv)) + 4.0 * np.eye(nv)
    A[5, :, 3] = 0.0                          # a zero column: singular
    b = rng.standard_normal((n, nv))          # row-major right sides
    M = torch.as_tensor(A, device="cuda").contiguous()
    piv = torch.zeros((n, nv), dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lu.pyro_batched_lu_factor(M.data_ptr(), piv.data_ptr(), None, n,
                                     nv, st.data_ptr(), _stream()) == 0
    B = torch.as_tensor(b, device="cuda").contiguous()
    assert lu.pyro_batched_lu_solve(M.data_ptr(), piv.data_ptr(), None,
                                    B.data_ptr(), nv, 1, B.data_ptr(), nv, 1,
                                    n, nv, _stream()) == 0
    torch.cuda.synchronize()
    assert int(st.item()) & 1
    X = B.cpu().numpy()
    for s in range(n):
        if s == 5:
            continue
        x_ref = np.linalg.solve(A[s], b[s])
        assert np.abs(X[s] - x_ref).max() <= 1e-12 * np.abs(x_ref).max()


def test_wrms_columns_fixed_order():
    _, rs = _libs()
    nv, n = 54, 1000
    rng = np.random.default_rng(5)
    v = rng.standard_normal((nv, n))
    w = rng.uniform(0.5, 2.0, size=(nv, n))
    V = torch.as_tensor(v, device="cuda")
    W = torch.as_tensor(w, device="cuda")
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    assert rs.pyro_wrms_columns(V.data_ptr(), n, W.data_ptr(), n, nv, n,
                                out.data_ptr(), _stream()) == 0
    ref = np.sqrt(((v / w) ** 2).mean(axis=0))
    got = out.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-14 * ref.max()
    # a column's value does not depend on the batch around it
    out1 = torch.empty(1, dtype=torch.float64, device="cuda")
    V1, W1 = V[:, 17:18].contiguous(), W[:, 17:18].contiguous()
    assert rs.pyro_wrms_columns(V1.data_ptr(), 1, W1.data_ptr(), 1, nv, 1,
                                out1.data_ptr(), _stream()) == 0
    torch.cuda.synchronize()
    assert float(out1.item()) == float(got[17])
