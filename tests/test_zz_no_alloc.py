"""The no-allocation block-Thomas entry point (``pyro_block_thomas_noalloc``).

It exists for callers that cannot allocate device memory when they need the
solve -- applications that hand all device memory to their own pool at
start-up and forbid allocation inside a time step, or real-time loops that
cannot take an allocation's latency or failure mid-step -- and keeps its
scratch in a fixed static array of the library.  Here it is called
through the C ABI and compared with ``pyro_block_thomas`` (caller-provided
workspace) on two calls in a row, at the block-Thomas tests' tolerance.
This file is collected last on purpose."""

import ctypes

import numpy as np
import pytest

from oracle.block_thomas_oracle import make_systems

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
PYRO_ERR_CAPACITY = 5


def _lib():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    from pyrometheus_gb300 import native
    lib = ctypes.CDLL(native.build_block_thomas())
    lib.pyro_block_thomas.restype = I
    lib.pyro_block_thomas.argtypes = [P, P, P, P, P, P, P, I, I, P, P, P, I,
                                      I, P]
    lib.pyro_block_thomas_noalloc.restype = I
    lib.pyro_block_thomas_noalloc.argtypes = [P, P, P, P, P, P, P, I, I,
                                              I64, P, I, I, P]
    lib.pyro_block_thomas_noalloc_max_rows.restype = I64
    lib.pyro_block_thomas_noalloc_max_rows.argtypes = [I]
    lib.pyro_block_thomas_work_doubles.restype = I64
    lib.pyro_block_thomas_work_doubles.argtypes = [I, I64]
    return lib


def _device_systems(nsys, nv, seed):
    lengths, L, C, U, b = make_systems(nsys, nv, 1, 120, seed=seed)
    dev = torch.device("cuda")
    t = [torch.as_tensor(a, device=dev).contiguous() for a in (L, C, U, b)]
    offs = torch.as_tensor(np.concatenate([[0], np.cumsum(lengths)]),
                           dtype=torch.int64, device=dev)
    order = torch.as_tensor(np.argsort(-lengths, kind="stable"),
                            dtype=torch.int32, device=dev)
    return lengths, t, offs, order


@pytest.mark.parametrize("nv", [10, 54])
def test_noalloc_matches_allocating_entry_point_twice(nv):
    lib = _lib()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    nsys = 40 if nv == 10 else 4
    for call, seed in enumerate((11, 12)):
        lengths, (L, C, U, b), offs, order = _device_systems(nsys, nv, seed)
        rows = int(lengths.sum())
        assert rows <= lib.pyro_block_thomas_noalloc_max_rows(nv)
        threads = 32 if nv <= 12 else 128
        # existing entry point: caller-provided workspace and counter
        work = torch.empty(int(lib.pyro_block_thomas_work_doubles(nv, rows)),
                           dtype=torch.float64, device="cuda")
        counter = torch.zeros(1, dtype=torch.int32, device="cuda")
        st_ref = torch.zeros(1, dtype=torch.int32, device="cuda")
        x_ref = torch.empty_like(b)
        assert lib.pyro_block_thomas(
            L.data_ptr(), C.data_ptr(), U.data_ptr(), b.data_ptr(),
            x_ref.data_ptr(), offs.data_ptr(), order.data_ptr(), nsys, nv,
            work.data_ptr(), counter.data_ptr(), st_ref.data_ptr(), threads,
            0, sp) == 0
        # no-allocation entry point
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        x = torch.full_like(b, float("nan"))
        assert lib.pyro_block_thomas_noalloc(
            L.data_ptr(), C.data_ptr(), U.data_ptr(), b.data_ptr(),
            x.data_ptr(), offs.data_ptr(), order.data_ptr(), nsys, nv, rows,
            st.data_ptr(), threads, 0, sp) == 0
        torch.cuda.synchronize()
        assert int(st.item()) == 0 and int(st_ref.item()) == 0
        xr, xn = x_ref.cpu().numpy(), x.cpu().numpy()
        assert np.isfinite(xn).all()
        assert np.abs(xn - xr).max() <= 1e-12 * np.abs(xr).max(), call


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib()
    nv = 54
    too_many = int(lib.pyro_block_thomas_noalloc_max_rows(nv)) + 1
    # rejected on the host before any device memory is touched
    st = lib.pyro_block_thomas_noalloc(1, 1, 1, 1, 1, 1, 1, 1, nv, too_many,
                                       None, 128, 0, None)
    assert st == PYRO_ERR_CAPACITY


def test_noalloc_skips_systems_past_the_stated_rows():
    """If the host's total_rows is smaller than the packed offsets say, the
    systems reaching past it are skipped (status bit 1) instead of writing
    past the static scratch; the others still match the allocating entry
    point and the skipped rows of x keep what they held."""
    lib = _lib()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    nv, nsys = 10, 6
    lengths, (L, C, U, b), offs, order = _device_systems(nsys, nv, 31)
    rows = int(lengths.sum())
    head = rows - int(lengths[-1])
    work = torch.empty(int(lib.pyro_block_thomas_work_doubles(nv, rows)),
                       dtype=torch.float64, device="cuda")
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    x_ref = torch.empty_like(b)
    assert lib.pyro_block_thomas(
        L.data_ptr(), C.data_ptr(), U.data_ptr(), b.data_ptr(),
        x_ref.data_ptr(), offs.data_ptr(), order.data_ptr(), nsys, nv,
        work.data_ptr(), counter.data_ptr(), None, 32, 0, sp) == 0
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    x = torch.full_like(b, float("nan"))
    assert lib.pyro_block_thomas_noalloc(
        L.data_ptr(), C.data_ptr(), U.data_ptr(), b.data_ptr(),
        x.data_ptr(), offs.data_ptr(), order.data_ptr(), nsys, nv, head,
        st.data_ptr(), 32, 0, sp) == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 2
    xr, xn = x_ref.cpu().numpy(), x.cpu().numpy()
    assert np.abs(xn[:head] - xr[:head]).max() <= \
        1e-12 * np.abs(xr[:head]).max()
    assert np.isnan(xn[head:]).all()
