import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def load_golden(name):
    """Golden vectors written by ``tests/golden/make_golden.py`` plus the
    mechanism they were computed for."""
    from pyrometheus_gb300.yaml_mech import load_mechanism
    g = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
    sol = load_mechanism(f"{name}.yaml", text=str(g.pop("mech_yaml")))
    return sol, g


# seeded synthetic mechanisms (the benchmark shapes and one with
# irreversible reactions, fractional orders and a zero default efficiency)
# and the reference's own test fixtures (test/mechs/*.yaml, the set
# test/CMakeLists.txt:9 runs every backend on), all with golden vectors
# from the reference's generated class
FIXTURE_SETS = ["ref_uiuc", "ref_sandiego", "ref_hong", "ref_uconn32",
                "ref_gri30"]
GOLDEN_SETS = ["synthetic9", "synthetic53", "quirks9"] + FIXTURE_SETS


def rel_err(x, ref, scale=None):
    """max |x - ref| / max(|ref|, scale), ignoring exact zeros of both."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    s = np.abs(ref) if scale is None else np.maximum(np.abs(ref), scale)
    d = np.abs(x - ref)
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(d == 0, 0.0, d / s)
    return float(np.nanmax(r)) if r.size else 0.0


@pytest.fixture(params=GOLDEN_SETS)
def golden(request):
    return load_golden(request.param)
