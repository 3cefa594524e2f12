"""Steady-flamelet residual and block Jacobian: the oracle against the
golden vectors (reference-generated chemistry, reference autodiff through
the enthalpy Newton), and the CUDA assembly against both (``-m gpu``)."""

import os

import numpy as np
import pytest

from conftest import GOLDEN

TAGS = ["s9", "s53"]


def _golden(tag):
    from pyrometheus_gb300.yaml_mech import load_mechanism
    g = np.load(os.path.join(GOLDEN, "flamelet.npz"))
    d = {k[len(tag) + 1:]: g[k] for k in g.files if k.startswith(tag + "_")}
    sol = load_mechanism(None, text=str(d["mech_yaml"]))
    return sol, d


def _resid_scale(d):
    """Element scale of the residual: the magnitudes of its three terms."""
    from oracle.flamelet_oracle import FlameletOracle
    phi = np.vstack([d["h"], d["Y"]])
    lap = FlameletOracle.laplacian(phi, float(d["dx"]))
    bc = np.zeros_like(phi)
    bc[0, 0], bc[0, -1] = d["h_ox"], d["h_fu"]
    bc[1:, 0], bc[1:, -1] = d["y_ox"], d["y_fu"]
    return np.abs(0.5 * d["chi"] * lap) + np.abs(d["src"]) + np.abs(bc)


def _source_part(d):
    """Golden source Jacobian: central blocks minus the Laplacian part."""
    from oracle.flamelet_oracle import FlameletOracle
    n_x, nv, _ = d["C"].shape
    _, lap_c, _ = FlameletOracle.blocks(np.zeros((n_x, nv, nv)), d["chi"],
                                        float(d["dx"]))
    return d["C"] - lap_c


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_residual_matches_golden(tag):
    from oracle.flamelet_oracle import FlameletOracle
    sol, d = _golden(tag)
    orc = FlameletOracle(sol)
    r = orc.residual(d["h"], d["Y"], d["chi"], d["visc"], d["T_guess"],
                     float(d["P"]), float(d["h_ox"]), float(d["h_fu"]),
                     d["y_ox"], d["y_fu"], float(d["dx"]))
    assert np.all(np.abs(r - d["resid"]) <= 1e-12 * _resid_scale(d))
    t = orc.temperature(d["h"], d["Y"], d["T_guess"])
    assert np.abs(t - d["T_solved"]).max() <= 1e-9


@pytest.mark.parametrize("tag", TAGS)
def test_laplacian_blocks_match_golden(tag):
    from oracle.flamelet_oracle import FlameletOracle
    sol, d = _golden(tag)
    n_x, nv, _ = d["C"].shape
    lo, c, up = FlameletOracle.blocks(np.zeros((n_x, nv, nv)), d["chi"],
                                      float(d["dx"]))
    assert np.array_equal(lo, d["L"]) and np.array_equal(up, d["U"])
    # boundary rows carry no source Jacobian
    assert np.array_equal(c[0], d["C"][0]) and np.array_equal(c[-1],
                                                              d["C"][-1])


def test_source_jacobian_order_of_convergence():
    """Central differences of the oracle source converge to the golden
    (autodiff) source Jacobian at second order, the reference's own check
    of its jacfwd Jacobian (test/test.py:360-374)."""
    from oracle.flamelet_oracle import FlameletOracle
    sol, d = _golden("s9")
    orc = FlameletOracle(sol)
    sj = _source_part(d)
    pts = [3, 5]
    ref = sj[pts]
    errs = []
    deltas = [1e-3, 1e-4, 1e-5]
    for rel in deltas:
        fd = orc.source_jacobian_fd(d["h"][pts], d["Y"][:, pts],
                                    d["visc"][pts], d["T_guess"][pts],
                                    float(d["P"]), rel=rel)
        errs.append(np.linalg.norm(fd - ref) / np.linalg.norm(ref))
    order = np.polyfit(np.log(deltas), np.log(errs), 1)[0]
    assert order > 1.95, (errs, order)
