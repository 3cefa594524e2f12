"""The reference's own C++ target (``pyrometheus/codegen/cpp.py``, rendered
through the stand-ins of ``oracle/refgen.py`` into ``oracle/_ref`` by
``oracle/ref_cpp.py``) against the golden vectors of its Python target:
the CPU baseline ``bench.py`` times is the reference's generated code and
computes the same numbers.  Skipped where the headers were never rendered
(they need the reference checkout once)."""

import numpy as np
import pytest

from conftest import GOLDEN_SETS, load_golden, rel_err
from oracle import ref_cpp


@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_reference_cpp_matches_reference_python(name):
    if not ref_cpp.available(name):
        pytest.skip("reference C++ header not rendered (needs "
                    "PYRO_REFERENCE_ROOT once)")
    sol, g = load_golden(name)
    lib = ref_cpp.load(name)
    assert int(lib.ref_num_species()) == sol.n_species
    assert int(lib.ref_num_reactions()) == sol.n_reactions
    w, tn = ref_cpp.fused_step(lib, g["P"], g["T"], g["Y"], g["e_mass"],
                               1500.0, nthreads=2)
    s = g["cdot"] + g["ddot"]
    assert rel_err(w, g["wdot"], s) < 1e-12
    # per-state Newton (ContainerT = double) against the Python target's
    # batch-wide one
    assert np.abs(tn - g["T_from_e"]).max() < 1e-10
