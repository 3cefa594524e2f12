"""Compressible-EOS consistency pieces on the CPU: the flamelet oracle's
adjoint operator, ``R T`` and its gradient, the source's pressure gradient
and the adjoint enthalpy / EOS gradients against golden vectors restated
from the reference (``pyrometheus/flamelets/equations.py:451-535``,
``thermodynamic_consistency.py:105-307``) with its generated class, its
``block_thomas`` and autodiff stand-ins (``tests/golden/make_golden.py``)."""

import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_err
from oracle.flamelet_oracle import FlameletOracle
from pyrometheus_gb300.yaml_mech import load_mechanism

# stiff benchmark mechanisms, and the same with slow chemistry
TAGS = ["s9", "s53", "s9slow", "s53slow"]


def eos_golden(tag):
    d = np.load(os.path.join(GOLDEN, "eos_adjoint.npz"))
    g = {k[len(tag) + 1:]: d[k] for k in d.files if k.startswith(tag + "_")}
    sol = load_mechanism(f"{tag}.yaml", text=str(g.pop("mech_yaml")))
    return sol, g


@pytest.mark.parametrize("tag", TAGS)
def test_adjoint_operator_and_gradients_from_golden_pieces(tag):
    sol, g = eos_golden(tag)
    fo = FlameletOracle(sol)
    dx = float(g["dx"])
    lo, c, up = fo.adjoint_blocks(g["src_jac_all"], g["chi"], dx)
    assert np.array_equal(lo, g["adj_L"]) and np.array_equal(up, g["adj_U"])
    assert rel_err(c, g["adj_C"]) < 1e-15
    adj_h, hg = fo.enthalpy_gradient(g["src_jac_all"], g["chi"], dx,
                                     g["pdf"])
    assert rel_err(adj_h, g["adj_h"], np.abs(g["adj_h"]).max()) < 1e-12
    assert rel_err(hg, g["h_gradient"]) < 1e-11
    (dens, ener), (ad, ae) = fo.eos_gradient(
        g["src_jac_all"], g["rt"], g["rt_jac"], g["ds_dp"], g["chi"], dx,
        g["pdf"], float(g["P"]))
    assert rel_err(ad, g["adj_d"], np.abs(g["adj_d"]).max()) < 1e-12
    assert rel_err(ae, g["adj_e"], np.abs(g["adj_e"]).max()) < 1e-12
    assert rel_err(dens, g["density_gradient"]) < 1e-11
    assert rel_err(ener, g["energy_gradient"]) < 1e-11


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_derivative_pieces(tag):
    """R T exactly as the reference forms it; its gradient and the
    source's pressure gradient by finite differences against the golden
    forward-mode derivatives."""
    sol, g = eos_golden(tag)
    fo = FlameletOracle(sol)
    rt = fo.eos_rt(g["h"], g["Y"], g["T_guess"])
    assert rel_err(rt, g["rt"]) < 1e-13
    rtj = fo.eos_rt_jacobian_fd(g["h"], g["Y"], g["T_guess"])
    assert rel_err(rtj, g["rt_jac"], np.abs(g["rt_jac"]).max(axis=1,
                                                          keepdims=True)) \
        < 1e-6
    dsdp = fo.source_pressure_gradient_fd(g["h"], g["Y"], g["visc"],
                                          g["T_guess"], float(g["P"]))
    scale = np.abs(g["ds_dp"]).max(axis=1, keepdims=True)
    assert rel_err(dsdp, g["ds_dp"], scale) < 1e-8
