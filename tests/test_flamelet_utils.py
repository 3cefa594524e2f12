"""Flamelet set-up helpers (``pyrometheus_gb300.flamelet_utils``, after
``pyrometheus/flamelets/utils.py``): the stoichiometric mixture fraction of
the reference notebook's H2/N2 against air streams (it prints
``Z_st = 0.304``), the bell profile's shape, and both against the
reference's own functions run live when the checkout is present."""

import numpy as np
import pytest

from oracle import refgen
from pyrometheus_gb300 import synthetic
from pyrometheus_gb300.flamelet_utils import (bell_profile,
                                              stoichiometric_mixture_fraction)


def _streams(sol):
    w = sol.molecular_weights

    def y(x):
        v = np.array([x.get(n, 0.0) for n in sol.species_names]) * w
        return v / v.sum()
    return y({"O2": 0.21, "N2": 0.79}), y({"H2": 0.5, "N2": 0.5})


def test_notebook_stoichiometric_mixture_fraction():
    sol = synthetic.config1_mechanism()
    y_ox, y_fu = _streams(sol)
    assert round(stoichiometric_mixture_fraction(sol, y_ox, y_fu), 3) \
        == 0.304
    # pure streams: the fuel side has no oxygen, so b_fu > 0 > b_ox
    assert 0.0 < stoichiometric_mixture_fraction(sol, y_ox, y_fu) < 1.0


def test_bell_profile_shape():
    z = np.linspace(0.01, 0.99, 99)
    b = bell_profile(z)
    assert bell_profile(0.5) == 1.0
    np.testing.assert_allclose(b, b[::-1], rtol=1e-14)
    assert np.all(np.diff(b[:49]) > 0) and b.max() <= 1.0


@pytest.mark.skipif(not refgen.reference_available(),
                    reason="reference checkout not present")
def test_helpers_match_the_reference():
    from oracle import refdriver
    ref = refdriver.reference_flamelet_utils()
    for sol in (synthetic.config1_mechanism(),
                synthetic.config2_mechanism()):
        y_ox, y_fu = _streams(sol)
        assert stoichiometric_mixture_fraction(sol, y_ox, y_fu) == \
            ref.stoichiometric_mixture_fraction(sol, y_ox, y_fu)
    z = np.linspace(0.0, 1.0, 101)
    np.testing.assert_array_equal(bell_profile(z),
                                  np.asarray(ref.bell_profile(z)))


def test_burke_schumann_profile():
    """Complete one-step combustion along the mixing line: mass fractions
    sum to one, no fuel on the lean side, no O2 on the rich side, both
    gone at the stoichiometric mixture fraction, and the elements of the
    mixing line conserved."""
    from conftest import load_golden
    from pyrometheus_gb300.flamelet_utils import burke_schumann
    sol, _ = load_golden("ref_sandiego")
    S = sol.n_species
    W = np.asarray(sol.molecular_weights)
    idx = sol.species_index

    def from_x(d):
        x = np.zeros(S)
        for k, v in d.items():
            x[idx(k)] = v
        return x * W / np.dot(x, W)

    y_ox = from_x({"O2": 0.21, "N2": 0.79})
    y_fu = from_x({"H2": 0.5, "N2": 0.5})
    z_st = stoichiometric_mixture_fraction(sol, y_ox, y_fu)
    z = np.concatenate([np.linspace(0.0, 1.0, 41), [z_st]])
    y = burke_schumann(sol, z, y_ox, y_fu)
    assert np.allclose(y.sum(axis=0), 1.0, rtol=0, atol=1e-14)
    assert (y >= 0).all()
    lean, rich = z < z_st - 1e-9, z > z_st + 1e-9
    assert np.all(y[idx("H2"), lean] == 0) and np.all(y[idx("O2"), rich] == 0)
    assert y[idx("H2"), -1] < 1e-15 and y[idx("O2"), -1] < 1e-15
    mix = (1 - z)[None, :] * y_ox[:, None] + z[None, :] * y_fu[:, None]
    el = list(sol.element_names)
    for e in range(len(el)):
        n = np.array([sol.n_atoms(k, e) for k in range(S)]) / W
        assert np.allclose(n @ y, n @ mix, rtol=1e-12, atol=1e-15)
