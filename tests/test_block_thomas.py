"""Batched block-Thomas: the oracle against the reference's own
``block_thomas`` (golden vectors from ``flamelets/linear_solver.py`` run in
the build container) and against a dense solve; the CUDA solver against
both (``-m gpu``)."""

import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.block_thomas_oracle import (block_thomas, dense_matrix,
                                        make_systems, solve_packed)

TAGS = ["nv4", "nv10", "nv54"]


def _golden(tag):
    g = np.load(os.path.join(GOLDEN, "block_thomas.npz"))
    return [g[f"{tag}_{k}"] for k in ("lengths", "L", "C", "U", "b", "x")]


def _rel(x, ref):
    return np.abs(x - ref).max() / np.abs(ref).max()


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_matches_reference_block_thomas(tag):
    """The oracle's solve against the reference's on its golden systems, to
    cond(A)·eps (cond up to 3e4): the two solve the diagonal blocks through
    the platform's LAPACK, whose rounding differs between machines (1e-13
    at nv = 54 on an Arm build, below 1e-14 on x86)."""
    lengths, L, C, U, b, x = _golden(tag)
    assert _rel(solve_packed(lengths, L, C, U, b), x) < 1e-12


def _two_ended(lengths, L, C, U, b):
    """The segmented kernels' recurrences in numpy: per system, rows 0 ..
    m-1 eliminated downwards (S_i = C'_i^-1 U_i), rows N-1 .. m+1 upwards
    (S^_i = C^_i^-1 L_{i-1}), the middle row m = N // 2 solved with both
    couplings, then x outwards from it."""
    x = np.empty_like(b)
    r0 = 0
    for n in lengths:
        n = int(n)
        m = n >> 1
        S, t = {}, {}
        for i in range(m):
            cp, bp = C[r0 + i].copy(), b[r0 + i].copy()
            if i:
                cp -= L[r0 + i - 1] @ S[i - 1]
                bp -= L[r0 + i - 1] @ t[i - 1]
            S[i], t[i] = (np.linalg.solve(cp, U[r0 + i]),
                          np.linalg.solve(cp, bp))
        for k in range(n - 1 - m):
            i = n - 1 - k
            cp, bp = C[r0 + i].copy(), b[r0 + i].copy()
            if k:
                cp -= U[r0 + i] @ S[i + 1]
                bp -= U[r0 + i] @ t[i + 1]
            S[i], t[i] = (np.linalg.solve(cp, L[r0 + i - 1]),
                          np.linalg.solve(cp, bp))
        cm, bm = C[r0 + m].copy(), b[r0 + m].copy()
        if m >= 1:
            cm -= L[r0 + m - 1] @ S[m - 1]
            bm -= L[r0 + m - 1] @ t[m - 1]
        if m + 1 <= n - 1:
            cm -= U[r0 + m] @ S[m + 1]
            bm -= U[r0 + m] @ t[m + 1]
        x[r0 + m] = xp = np.linalg.solve(cm, bm)
        for i in range(m - 1, -1, -1):
            x[r0 + i] = xp = t[i] - S[i] @ xp
        xp = x[r0 + m]
        for i in range(m + 1, n):
            x[r0 + i] = xp = t[i] - S[i] @ xp
        r0 += n
    return x


@pytest.mark.parametrize("nv", [1, 3, 10])
def test_two_ended_recurrence_equals_top_down(nv):
    """The elimination order of the segmented kernels (from both ends to
    the middle row) reaches the reference's top-down solution
    (linear_solver.py:6-103) on uneven systems of 1 to 40 rows."""
    lengths, L, C, U, b = make_systems(60, nv, 1, 40, seed=70 + nv)
    assert (lengths <= 3).any()
    ref = solve_packed(lengths, L, C, U, b)
    assert _rel(_two_ended(lengths, L, C, U, b), ref) < 1e-13


def test_oracle_against_dense_solve():
    lengths, L, C, U, b = make_systems(1, 6, 5, 5, seed=3)
    n = int(lengths[0])
    x = block_thomas(L[:n - 1], C, U[:n - 1], b)
    xd = np.linalg.solve(dense_matrix(L[:n - 1], C, U[:n - 1]),
                         b.reshape(-1)).reshape(n, -1)
    assert _rel(x, xd) < 1e-13


torch = pytest.importorskip("torch")


def _cuda():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")


def _solve_cuda(lengths, L, C, U, b, threads=None, use_graph=False,
                kernel=None):
    from pyrometheus_gb300.flamelet import BlockThomasSolver
    dev = torch.device("cuda")
    t = [torch.as_tensor(a, device=dev).contiguous() for a in (L, C, U, b)]
    solver = BlockThomasSolver(C.shape[1], lengths, threads=threads,
                               use_graph=use_graph, kernel=kernel)
    x = solver.solve(*t)
    solver.check_status()
    return x.cpu().numpy(), solver, t


PLANS = [("cta", 32), ("cta", 64), ("cta", 128), ("small", 32),
         ("small", 64), ("seg", 32)]


@pytest.mark.gpu
@pytest.mark.parametrize("tag", TAGS)
@pytest.mark.parametrize("plan", PLANS)
def test_cuda_block_thomas_golden(tag, plan):
    _cuda()
    lengths, L, C, U, b, x = _golden(tag)
    kernel, threads = plan
    if kernel in ("small", "seg") and C.shape[1] > 16:
        pytest.skip(f"the {kernel!r} kernel takes nv <= 16")
    got, _, _ = _solve_cuda(lengths, L, C, U, b, threads=threads,
                            kernel=kernel)
    assert _rel(got, x) < 1e-12


def _residual(L, C, U, b, x):
    """Normwise backward error of one system,
    ||A x - b||_inf / (||A||_inf ||x||_inf + ||b||_inf)."""
    r = np.einsum("nij,nj->ni", C, x) - b
    r[:-1] += np.einsum("nij,nj->ni", U[:-1], x[1:])
    r[1:] += np.einsum("nij,nj->ni", L[:-1], x[:-1])
    rows = np.abs(C).sum(axis=2)
    rows[:-1] += np.abs(U[:-1]).sum(axis=2)
    rows[1:] += np.abs(L[:-1]).sum(axis=2)
    return np.abs(r).max() / (rows.max() * np.abs(x).max()
                              + np.abs(b).max())


@pytest.mark.gpu
@pytest.mark.parametrize("nv,kernel", [(10, "cta"), (10, "small"),
                                       (10, "seg"), (1, "seg"), (3, "seg"),
                                       (8, "seg"), (16, "seg"),
                                       (54, "cta")])
def test_cuda_block_thomas_uneven_batch(nv, kernel):
    """Against the reference algorithm on long systems.  The two round
    differently (right-looking LU and sequential Schur updates here,
    LAPACK's recursive getrf and BLAS there), so x agrees only to about
    cond(A)·eps: these random systems have cond(A) of 1e4 to 3e4, which puts
    the forward difference near 1e-11 at nv=54.  The test therefore checks
    x at 1e-10 and the normwise backward error against the reference's own
    (block elimination is not backward stable to eps: the reference itself
    reaches about 1e-13 at nv=54), within a factor of 16."""
    _cuda()
    lengths, L, C, U, b = make_systems(37 if nv == 54 else 300, nv, 1, 200,
                                       seed=nv)
    ref = solve_packed(lengths, L, C, U, b)
    got, solver, t = _solve_cuda(lengths, L, C, U, b, kernel=kernel)
    r0 = 0
    for n in lengths:
        n = int(n)
        sl = slice(r0, r0 + n)
        assert _rel(got[sl], ref[sl]) < 1e-10
        be_got = _residual(L[sl], C[sl], U[sl], b[sl], got[sl])
        be_ref = _residual(L[sl], C[sl], U[sl], b[sl], ref[sl])
        assert be_got <= 16.0 * max(be_ref, nv * 1.1e-16)
        r0 += n


@pytest.mark.gpu
@pytest.mark.parametrize("nv", [3, 10, 16])
@pytest.mark.parametrize("ctas", [1, 3])
def test_seg_segments_take_systems_in_turn(nv, ctas):
    """The segmented kernel with a grid far smaller than the batch: one or
    three CTAs of four warps, so every lane segment runs tens of sweeps of
    uneven lengths one after another (each segment taking the next sweep of
    the order when its own is done), lengths 1 to 90 (one- and two-row
    systems, whose sweeps are empty, included); in a CUDA graph, replayed
    with new right-hand sides, then two more through the re-solve."""
    _cuda()
    from pyrometheus_gb300.flamelet import BlockThomasSolver
    lengths, L, C, U, b = make_systems(300, nv, 1, 90, seed=40 + nv)
    assert (lengths == 1).any()
    ref = solve_packed(lengths, L, C, U, b)
    dev = torch.device("cuda")
    t = [torch.as_tensor(a, device=dev).contiguous() for a in (L, C, U, b)]
    solver = BlockThomasSolver(nv, lengths, kernel="seg", ctas=ctas,
                               use_graph=True)
    got = solver.solve(*t).cpu().numpy()
    solver.check_status()
    assert _rel(got, ref) < 1e-10
    b2 = np.random.default_rng(nv).standard_normal(b.shape)
    t[3].copy_(torch.as_tensor(b2))
    got2 = solver.solve(*t).cpu().numpy()
    assert _rel(got2, solve_packed(lengths, L, C, U, b2)) < 1e-10
    # two more right-hand sides from the kept factors
    B = np.random.default_rng(nv + 1).standard_normal((2,) + b.shape)
    X = solver.resolve(t[0], t[2], torch.as_tensor(B, device=dev))
    X = X.cpu().numpy()
    for c in range(2):
        assert _rel(X[c], solve_packed(lengths, L, C, U, B[c])) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("nv", [5, 10])
def test_seg_resolve_through_the_abi_with_a_padded_stride(nv):
    """pyro_block_thomas_seg then pyro_block_thomas_seg_resolve through
    the C ABI: four right-hand sides 7 doubles apart beyond their packed
    size (the padding untouched), each against the oracle's solve."""
    _cuda()
    import ctypes

    from pyrometheus_gb300 import native
    lib = native.block_thomas_lib()
    lengths, L, C, U, b = make_systems(70, nv, 1, 60, seed=60 + nv)
    rows = int(lengths.sum())
    dev = torch.device("cuda")
    t = [torch.as_tensor(a, device=dev).contiguous() for a in (L, C, U, b)]
    offs = torch.as_tensor(np.concatenate([[0], np.cumsum(lengths)]),
                           dtype=torch.int64, device=dev)
    order = torch.as_tensor(np.argsort(-lengths, kind="stable"),
                            dtype=torch.int32, device=dev)
    work = torch.empty(int(lib.pyro_block_thomas_work_doubles(nv, rows)),
                       dtype=torch.float64, device=dev)
    counter = torch.zeros(1, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    x = torch.empty_like(t[3])
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.pyro_block_thomas_seg(
        *[a.data_ptr() for a in t], x.data_ptr(), offs.data_ptr(),
        order.data_ptr(), len(lengths), nv, work.data_ptr(),
        counter.data_ptr(), status.data_ptr(), 0, sp) == 0
    stride = rows * nv + 7
    rng = np.random.default_rng(nv)
    B = torch.as_tensor(rng.standard_normal(4 * stride), device=dev)
    X = torch.full((4 * stride,), 7.5, dtype=torch.float64, device=dev)
    assert lib.pyro_block_thomas_seg_resolve(
        t[0].data_ptr(), t[2].data_ptr(), B.data_ptr(), X.data_ptr(), 4,
        stride, offs.data_ptr(), order.data_ptr(), len(lengths), nv,
        work.data_ptr(), counter.data_ptr(), status.data_ptr(), sp) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    Bh, Xh = B.cpu().numpy(), X.cpu().numpy()
    for c in range(4):
        bc = Bh[c * stride:c * stride + rows * nv].reshape(rows, nv)
        xc = Xh[c * stride:c * stride + rows * nv].reshape(rows, nv)
        assert _rel(xc, solve_packed(lengths, L, C, U, bc)) < 1e-10
        assert np.all(Xh[c * stride + rows * nv:(c + 1) * stride] == 7.5)


@pytest.mark.gpu
def test_cuda_graph_replay_and_single_system_api():
    _cuda()
    from pyrometheus_gb300.flamelet import block_thomas as bt_gpu
    lengths, L, C, U, b = make_systems(64, 10, 16, 64, seed=5)
    ref = solve_packed(lengths, L, C, U, b)
    got, solver, t = _solve_cuda(lengths, L, C, U, b, use_graph=True)
    assert _rel(got, ref) < 1e-12
    # replay with new right-hand sides in the same buffers
    b2 = np.random.default_rng(6).standard_normal(b.shape)
    t[3].copy_(torch.as_tensor(b2))
    x2 = solver.solve(*t).cpu().numpy()
    assert _rel(x2, solve_packed(lengths, L, C, U, b2)) < 1e-12
    # the reference's single-system signature
    n = int(lengths[0])
    xs = bt_gpu(L[:n - 1], C[:n], U[:n - 1], b[:n]).cpu().numpy()
    assert _rel(xs, ref[:n]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["cta", "small", "seg"])
def test_empty_systems_are_skipped_and_flagged(kernel):
    """A system with an empty row range is skipped with status bit 1 and
    writes nothing.  The empty systems sit right after non-empty ones in
    the packing (offsets 0, 5, 5, 12, 12, 20), so a kernel that ran their
    backward sweep anyway would overwrite the last row of the system before
    them, inside the buffers: that row must still hold its solution.  The
    re-solve with the kept factors skips them the same way."""
    _cuda()
    import ctypes

    from pyrometheus_gb300 import native
    lib = native.block_thomas_lib()
    nv = 10
    real = np.array([5, 7, 8])
    lengths = np.array([5, 0, 7, 0, 8])
    rows = int(real.sum())
    rng = np.random.default_rng(18)
    L, C, U = (rng.standard_normal((rows, nv, nv)) for _ in range(3))
    C += 10.0 * np.eye(nv)
    b = rng.standard_normal((rows, nv))
    ref = solve_packed(real, L, C, U, b)
    dev = torch.device("cuda")
    t = [torch.as_tensor(a, device=dev).contiguous() for a in (L, C, U, b)]
    offs = torch.as_tensor(np.concatenate([[0], np.cumsum(lengths)]),
                           dtype=torch.int64, device=dev)
    # the empty systems first, where a longest-first order would not put
    # them
    order = torch.as_tensor([1, 3, 4, 2, 0], dtype=torch.int32, device=dev)
    work = torch.empty(int(lib.pyro_block_thomas_work_doubles(nv, rows)),
                       dtype=torch.float64, device=dev)
    counter = torch.zeros(1, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    x = torch.full_like(t[3], float("nan"))
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = [a.data_ptr() for a in t] + [x.data_ptr(), offs.data_ptr(),
                                        order.data_ptr(), 5, nv,
                                        work.data_ptr()]
    if kernel == "cta":
        st = lib.pyro_block_thomas(*args, counter.data_ptr(),
                                   status.data_ptr(), 64, 0, sp)
    elif kernel == "small":
        st = lib.pyro_block_thomas_small(*args, status.data_ptr(), 32, sp)
    else:
        st = lib.pyro_block_thomas_seg(*args, counter.data_ptr(),
                                       status.data_ptr(), 0, sp)
    assert st == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 2
    assert _rel(x.cpu().numpy(), ref) < 1e-12
    # re-solve with the kept factors: the same skip and flag
    b2 = torch.as_tensor(rng.standard_normal((rows, nv)), device=dev)
    x2 = torch.full_like(b2, float("nan"))
    status.zero_()
    resolve = (lib.pyro_block_thomas_seg_resolve if kernel == "seg"
               else lib.pyro_block_thomas_resolve)
    assert resolve(
        t[0].data_ptr(), t[2].data_ptr(), b2.data_ptr(), x2.data_ptr(), 1,
        0, offs.data_ptr(), order.data_ptr(), 5, nv, work.data_ptr(),
        counter.data_ptr(), status.data_ptr(), sp) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 2
    ref2 = solve_packed(real, L, C, U, b2.cpu().numpy())
    assert _rel(x2.cpu().numpy(), ref2) < 1e-12


@pytest.mark.gpu
def test_seg_kernel_workspace_serves_resolve_and_matches_cta():
    """The several-systems-per-warp kernel keeps its two-ended factors, S |
    t blocks and pivots in the workspace: re-solves from it (its own
    re-solve, three right-hand sides in one call) equal fresh solves, and
    its solution equals the CTA kernel's to rounding."""
    _cuda()
    from pyrometheus_gb300.flamelet import BlockThomasSolver
    lengths, L, C, U, b = make_systems(97, 10, 1, 90, seed=23)
    dev = torch.device("cuda")
    t = [torch.as_tensor(a, device=dev).contiguous() for a in (L, C, U, b)]
    seg = BlockThomasSolver(10, lengths, kernel="seg")
    cta = BlockThomasSolver(10, lengths, kernel="cta", threads=64)
    xs = seg.solve(*t).cpu().numpy()
    xc = cta.solve(*t).cpu().numpy()
    seg.check_status()
    assert _rel(xs, xc) < 1e-13
    rng = np.random.default_rng(24)
    B = torch.as_tensor(rng.standard_normal((3,) + b.shape), device=dev)
    X = seg.resolve(t[0], t[2], B).cpu().numpy()
    for c in range(3):
        ref = solve_packed(lengths, L, C, U, B[c].cpu().numpy())
        assert _rel(X[c], ref) < 1e-12
