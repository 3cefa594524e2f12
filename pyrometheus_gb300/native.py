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


def build_mathcheck() -> str:
    return _build("mathcheck.cu", "mathcheck")


def build_runtime() -> str:
    return _build("runtime.cu", "runtime")


def build_block_thomas() -> str:
    return _build("block_thomas.cu", "block_thomas")


def build_batched_lu() -> str:
    return _build("batched_lu.cu", "batched_lu")


def build_reactor_step() -> str:
    return _build("reactor_step.cu", "reactor_step")


BUILDERS = [build_peaks, build_mathcheck, build_runtime, build_block_thomas,
            build_batched_lu, build_reactor_step]


@lru_cache(maxsize=None)
def peaks_lib() -> ctypes.CDLL:
    lib = ctypes.CDLL(build_peaks())
    lib.pyro_peaks_scratch_doubles.restype = ctypes.c_int64
    lib.pyro_peaks_scratch_doubles.argtypes = []
    lib.pyro_measure_fp64_rcp.restype = ctypes.c_int
    lib.pyro_measure_fp64_rcp.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int]
    lib.pyro_measure_fp64.restype = ctypes.c_int
    lib.pyro_measure_fp64.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int]
    lib.pyro_measure_dmma.restype = ctypes.c_int
    lib.pyro_measure_dmma.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
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


def measure_dmma(scratch, repeats: int = 3):
    """(FP64 FLOP/s of ``mma.sync`` m8n8k4, of m16n8k16) on the current
    device; *scratch* as for :func:`measure_fp64`."""
    res = (ctypes.c_double * 2)()
    st = peaks_lib().pyro_measure_dmma(ctypes.c_void_p(scratch.data_ptr()),
                                       res, int(repeats))
    if st != 0:
        raise RuntimeError(f"pyro_measure_dmma failed (status {st})")
    return res[0], res[1]


def measure_fp64_rcp(scratch, repeats: int = 3) -> float:
    """Double-precision reciprocals (``1.0 / x``) per second on the current
    device; *scratch* as for :func:`measure_fp64`."""
    res = ctypes.c_double()
    st = peaks_lib().pyro_measure_fp64_rcp(
        ctypes.c_void_p(scratch.data_ptr()), ctypes.byref(res), int(repeats))
    if st != 0:
        raise RuntimeError(f"pyro_measure_fp64_rcp failed (status {st})")
    return res.value


@lru_cache(maxsize=None)
def mathcheck_lib() -> ctypes.CDLL:
    lib = ctypes.CDLL(build_mathcheck())
    lib.pyro_exp_check.restype = ctypes.c_int
    lib.pyro_exp_check.argtypes = [ctypes.c_void_p] * 3 + [
        ctypes.c_int, ctypes.c_int64, ctypes.c_void_p]
    lib.pyro_log_check.restype = ctypes.c_int
    lib.pyro_log_check.argtypes = [ctypes.c_void_p] * 3 + [
        ctypes.c_int, ctypes.c_int64, ctypes.c_void_p]
    lib.pyro_rcp_check.restype = ctypes.c_int
    lib.pyro_rcp_check.argtypes = [ctypes.c_void_p] * 3 + [
        ctypes.c_int, ctypes.c_int64, ctypes.c_void_p]
    return lib


@lru_cache(maxsize=None)
def runtime_lib() -> ctypes.CDLL:
    lib = ctypes.CDLL(build_runtime())
    lib.pyro_memcpy2d_async.restype = ctypes.c_int
    lib.pyro_memcpy2d_async.argtypes = [
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
        ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]
    return lib


def copy_columns_async(dst, src, col0_dst: int, col0_src: int, ncols: int,
                       stream) -> None:
    """Copy columns [col0_src, col0_src + ncols) of the 2-D (or 1-D)
    float64 tensor *src* into columns starting at *col0_dst* of *dst* (host
    or device, row-major, unit column stride) with one pitched DMA."""
    if src.dim() == 1:
        src2, dst2 = src.view(1, -1), dst.view(1, -1)
    else:
        src2, dst2 = src, dst
    rows = src2.shape[0]
    es = src2.element_size()
    st = runtime_lib().pyro_memcpy2d_async(
        ctypes.c_void_p(dst2.data_ptr() + col0_dst * es),
        dst2.stride(0) * es,
        ctypes.c_void_p(src2.data_ptr() + col0_src * es),
        src2.stride(0) * es, ncols * es, rows,
        ctypes.c_void_p(stream.cuda_stream))
    if st != 0:
        raise RuntimeError(f"pyro_memcpy2d_async failed (status {st})")


@lru_cache(maxsize=None)
def block_thomas_lib() -> ctypes.CDLL:
    lib = ctypes.CDLL(build_block_thomas())
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.pyro_block_thomas.restype = I
    lib.pyro_block_thomas.argtypes = [P, P, P, P, P, P, P, I, I, P, P, P, I,
                                      I, P]
    lib.pyro_block_thomas_work_doubles.restype = I64
    lib.pyro_block_thomas_work_doubles.argtypes = [I, I64]
    lib.pyro_block_thomas_smem_bytes.restype = I64
    lib.pyro_block_thomas_smem_bytes.argtypes = [I]
    lib.pyro_block_thomas_small.restype = I
    lib.pyro_block_thomas_small.argtypes = [P, P, P, P, P, P, P, I, I, P, P,
                                            I, P]
    lib.pyro_block_thomas_seg.restype = I
    lib.pyro_block_thomas_seg.argtypes = [P, P, P, P, P, P, P, I, I, P, P, P,
                                          I, P]
    lib.pyro_block_thomas_resolve.restype = I
    lib.pyro_block_thomas_resolve.argtypes = [P, P, P, P, I, I64, P, P, I, I,
                                              P, P, P, P]
    lib.pyro_block_thomas_seg_resolve.restype = I
    lib.pyro_block_thomas_seg_resolve.argtypes = [P, P, P, P, I, I64, P, P,
                                                  I, I, P, P, P, P]
    return lib


@lru_cache(maxsize=None)
def batched_lu_lib() -> ctypes.CDLL:
    lib = ctypes.CDLL(build_batched_lu())
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.pyro_batched_lu_factor.restype = I
    lib.pyro_batched_lu_factor.argtypes = [P, P, P, I, I, P, P]
    lib.pyro_batched_lu_solve.restype = I
    lib.pyro_batched_lu_solve.argtypes = [P, P, P, P, I64, I64, P, I64, I64,
                                          I, I, P]
    return lib


@lru_cache(maxsize=None)
def reactor_step_lib() -> ctypes.CDLL:
    lib = ctypes.CDLL(build_reactor_step())
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.pyro_wrms_columns.restype = I
    lib.pyro_wrms_columns.argtypes = [P, I64, P, I64, I, I64, P, P]
    return lib
