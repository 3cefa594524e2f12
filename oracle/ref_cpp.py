"""The reference's own C++ target as a CPU baseline and cross-check.

TEST INFRASTRUCTURE / CPU BASELINE ONLY -- the CUDA product never imports
it; ``bench.py``'s CPU legs and the tests do.

Recipe:

1. :func:`render` runs the reference's ``CppCodeGenerator``
   (``pyrometheus/codegen/cpp.py``) through the stand-ins of
   :mod:`oracle.refgen` (needs ``PYRO_REFERENCE_ROOT``) and writes the
   generated C++20 header to ``oracle/_ref/ref_<tag>.hpp``;
2. :func:`build` compiles ``oracle/ref_cpp_driver.cpp`` around that header
   with g++ (``-O3 -std=c++20 -fopenmp``, no target-specific flags, so the
   same recipe runs on x86 and Arm hosts) into
   ``oracle/_ref/libref_<tag>.so``;
3. :func:`load` opens it with ctypes.

``oracle/_ref/`` is git-ignored: neither the reference-generated header nor
the library enters the repository's history.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
DRIVER = os.path.join(HERE, "ref_cpp_driver.cpp")


def header_path(tag: str) -> str:
    return os.path.join(REF_DIR, f"ref_{tag}.hpp")


def lib_path(tag: str) -> str:
    return os.path.join(REF_DIR, f"libref_{tag}.so")


def render(sol, tag: str) -> str:
    """Write the reference-generated header for *sol*; returns its path."""
    from . import refgen
    src = refgen.reference_cpp_source(sol, "Thermochemistry")
    os.makedirs(REF_DIR, exist_ok=True)
    path = header_path(tag)
    with open(path, "w") as f:
        f.write(src)
    return path


def build(tag: str, force: bool = False) -> str:
    """Compile the driver around ``ref_<tag>.hpp``; returns the library
    path (raises if the header was never rendered)."""
    hdr = header_path(tag)
    if not os.path.exists(hdr):
        raise FileNotFoundError(hdr)
    lib = lib_path(tag)
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(hdr),
                                             os.path.getmtime(DRIVER))):
        return lib
    tmp = lib + f".{os.getpid()}.tmp"
    cmd = ["g++", "-O3", "-std=c++20", "-fopenmp", "-fPIC", "-shared",
           f'-DREF_HEADER="{hdr}"', "-o", tmp, DRIVER]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("g++ failed:\n" + " ".join(cmd) + "\n"
                           + proc.stderr[-4000:])
    os.replace(tmp, lib)
    return lib


def available(tag: str) -> bool:
    return os.path.exists(header_path(tag)) or os.path.exists(lib_path(tag))


def load(tag: str) -> ctypes.CDLL:
    lib = ctypes.CDLL(build(tag))
    P, I64, D, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, \
        ctypes.c_int
    lib.ref_fused_step.restype = I
    lib.ref_fused_step.argtypes = [I64, P, P, P, I64, P, D, P, I64, P, I]
    lib.ref_num_species.restype = I
    lib.ref_num_reactions.restype = I
    return lib


def fused_step(lib, p, t, y, e, t0, nthreads=1):
    """``(wdot [S, n], T [n])`` through the reference's generated C++ for
    numpy inputs ``p, t, e [n]``, ``y [S, n]``."""
    import numpy as np
    n = t.shape[0]
    S = int(lib.ref_num_species())
    p = np.ascontiguousarray(np.broadcast_to(p, (n,)), dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    w = np.empty((S, n))
    tout = np.empty(n)

    def ptr(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    st = lib.ref_fused_step(n, ptr(p), ptr(t), ptr(y), n, ptr(e),
                            float(t0), ptr(w), n, ptr(tout), int(nthreads))
    if st != 0:
        raise RuntimeError(f"ref_fused_step failed ({st})")
    return w, tout
