"""Mechanism-independent native libraries of the package.

``BUILDERS`` lists the functions ``__graft_entry__.build()`` runs; each
compiles one CUDA translation unit of ``csrc/`` into an in-tree shared
library (content-addressed under ``pyrometheus_gb300/_build``) and returns
its path.
"""

from __future__ import annotations

import ctypes
import os
from functools import lru_cache

from .codegen.cuda import CSRC, build_shared_library


def _build(fname: str, stem: str) -> str:
    with open(os.path.join(CSRC, fname)) as f:
        src = f.read()
    return build_shared_library(src, stem)


def build_peaks() -> str:
    return _build("peaks.cu", "peaks")


BUILDERS = [build_peaks]


@lru_cache(maxsize=None)
def peaks_lib() -> ctypes.CDLL:
    lib = ctypes.CDLL(build_peaks())
    lib.pyro_peaks_scratch_doubles.restype = ctypes.c_int64
    lib.pyro_peaks_scratch_doubles.argtypes = []
    lib.pyro_measure_fp64.restype = ctypes.c_int
    lib.pyro_measure_fp64.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int]
    return lib


def peaks_scratch_doubles() -> int:
    return int(peaks_lib().pyro_peaks_scratch_doubles())


def measure_fp64(scratch, repeats: int = 3):
    """(DFMA FLOP/s, exp(double)/s, log(double)/s) measured on the current
    device; *scratch* is a float64 CUDA tensor of
    :func:`peaks_scratch_doubles` elements."""
    res = (ctypes.c_double * 3)()
    st = peaks_lib().pyro_measure_fp64(ctypes.c_void_p(scratch.data_ptr()),
                                       res, int(repeats))
    if st != 0:
        raise RuntimeError(f"pyro_measure_fp64 failed (status {st})")
    return res[0], res[1], res[2]
