"""The table-driven exponential (Tang 1989) and logarithm (Tang 1990) and
the Newton-Raphson reciprocal of csrc/pyro_math.cuh against CUDA's
double-precision exp/exp10/log/log10 and division on the device."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(x, ten, fn="pyro_exp_check"):
    from pyrometheus_gb300 import native
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for the gpu tests")
    xd = torch.as_tensor(x, dtype=torch.float64, device="cuda")
    mine = torch.empty_like(xd)
    ref = torch.empty_like(xd)
    st = getattr(native.mathcheck_lib(), fn)(
        xd.data_ptr(), mine.data_ptr(), ref.data_ptr(), int(ten), xd.numel(),
        torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    return mine.cpu().numpy(), ref.cpu().numpy()


def test_exp_against_cuda():
    rng = np.random.default_rng(0)
    x = np.concatenate([
        rng.uniform(-745.0, 709.7, 2_000_000),
        rng.uniform(-1.0, 1.0, 1_000_000),
        rng.uniform(-1e-6, 1e-6, 100_000),
        np.arange(-2048, 2048) * (np.log(2) / 2048),   # table knots
        [0.0, -0.0, 1e-300, -1e-300, 707.9999, 708.0, -708.0, 709.78, 710.0,
         -745.1, -746.0, -1e33, np.inf, -np.inf, np.nan]])
    mine, ref = _run(x, False)
    both_nan = np.isnan(mine) & np.isnan(ref)
    same = (mine == ref) | both_nan
    finite = np.isfinite(ref) & (ref > 1e-300)
    rel = np.abs(mine[finite] - ref[finite]) / ref[finite]
    # CUDA's exp is within 1 ulp of exp(x); the table method within about
    # 1.2 ulp plus |x| 8e-17 from its one-constant reduction, below the
    # |x| 1.1e-16 the rounding of x itself carries through exp
    bound = 1e-15 + 1.1e-16 * np.abs(x[finite])
    assert np.all(rel < bound), (rel / bound).max()
    small = finite & (np.abs(x) < 8.0)
    assert (np.abs(mine[small] - ref[small]) / ref[small]).max() < 1e-15
    edge = ~finite
    with np.errstate(invalid="ignore"):
        tol = (1e-15 + 1.1e-16 * np.abs(x[edge])) * np.abs(ref[edge])
        assert np.all(same[edge] | (np.abs(mine[edge] - ref[edge]) <= tol))


def test_exp10_against_cuda():
    rng = np.random.default_rng(1)
    x = rng.uniform(-20.0, 20.0, 500_000)
    mine, ref = _run(x, True)
    rel = np.abs(mine - ref) / ref
    # exp(x ln10) carries the rounding of x ln10: |x| ln10 ulp-relative
    assert rel.max() < 1e-14, rel.max()


def test_log_against_cuda():
    rng = np.random.default_rng(2)
    x = np.concatenate([
        10.0 ** rng.uniform(-307.0, 308.0, 2_000_000),
        rng.uniform(0.5, 2.0, 1_000_000),
        1.0 + rng.uniform(-1e-6, 1e-6, 100_000),
        1.0 + np.arange(-300, 300) / 2 ** 20,
        1.0 + np.arange(0, 129) / 128.0,                 # table knots
        [1.0, 2.0, 0.5, np.nextafter(1.0, 0.0), np.nextafter(1.0, 2.0),
         2.2250738585072014e-308, 1.7976931348623157e308, 5e-324, 0.0,
         -0.0, -1.0, np.inf, -np.inf, np.nan]])
    for ten in (False, True):
        mine, ref = _run(x, ten, "pyro_log_check")
        both_nan = np.isnan(mine) & np.isnan(ref)
        same = (mine == ref) | both_nan
        finite = np.isfinite(ref) & (ref != 0.0)
        rel = np.abs(mine[finite] - ref[finite]) / np.abs(ref[finite])
        # both within about 1 ulp of the logarithm: a few ulps apart
        assert rel.max() < 1e-15, (ten, rel.max())
        assert np.all(same[~finite])


@pytest.mark.parametrize("third", [0, 1], ids=["newton2", "cubic"])
def test_rcp_against_cuda_division(third):
    """Within an ulp of CUDA's correctly rounded 1.0 / x over the normal
    range whose reciprocals are normal, and equal to it on most
    arguments: two Newton-Raphson steps (pyro_rcp) and one third-order
    step (pyro_rcp3)."""
    rng = np.random.default_rng(3)
    mag = 10.0 ** rng.uniform(-300.0, 300.0, 2_000_000)
    x = np.concatenate([
        mag * rng.choice([-1.0, 1.0], mag.size),
        rng.uniform(0.5, 2.0, 1_000_000),
        1.0 + np.arange(-300, 300) / 2 ** 40,
        [1.0, -1.0, 2.0, 0.5, 3.0, 10.0, np.nextafter(1.0, 0.0),
         np.nextafter(1.0, 2.0)]])
    mine, ref = _run(x, third, "pyro_rcp_check")
    rel = np.abs(mine - ref) / np.abs(ref)
    assert rel.max() <= 2.3e-16, rel.max()
    assert np.mean(mine == ref) > 0.9
