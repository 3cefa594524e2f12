"""Batched block-Thomas solve on the GPU (flamelet Newton linear systems).

Mirrors ``pyrometheus/flamelets/linear_solver.py:6-103``
(``block_thomas(lower, central, upper, rhs)``) for one system, and adds
:class:`BlockThomasSolver` for thousands of systems of uneven lengths in one
persistent launch (``csrc/block_thomas.cu``), optionally captured in a CUDA
graph.  Systems are packed along the row axis: system ``s`` owns rows
``[offsets[s], offsets[s+1])`` of ``C[rows, nv, nv]``, ``L``, ``U`` (the
last row of each system's ``L``/``U`` is ignored) and ``b[rows, nv]``.
"""

from __future__ import annotations

import ctypes
import json
import os
from typing import Optional, Sequence

import numpy as np

from . import native

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _check(st, what):
    if st != 0:
        raise RuntimeError(f"{what} failed (status {st})")


class BlockThomasSolver:
    """Plan for solving ``len(lengths)`` block-tridiagonal systems with
    ``nv x nv`` blocks.

    ``threads``: CTA size (a multiple of 32; ``None`` picks from the
    autotuner cache or a size rule); ``ctas``: persistent grid (0: all
    resident CTAs); ``use_graph``: capture the counter reset and the launch
    in a CUDA graph on the first :meth:`solve` with given buffers and replay
    it afterwards.
    """

    def __init__(self, nv: int, lengths: Sequence[int], device=None,
                 threads: Optional[int] = None, ctas: int = 0,
                 use_graph: bool = False):
        if torch is None or not torch.cuda.is_available():
            raise RuntimeError("BlockThomasSolver needs a CUDA device")
        self.nv = int(nv)
        self.lengths = np.asarray(lengths, dtype=np.int64)
        if np.any(self.lengths < 1):
            raise ValueError("every system needs at least one row")
        self.device = torch.device(device if device is not None else "cuda")
        offs = np.concatenate([[0], np.cumsum(self.lengths)])
        self.rows = int(offs[-1])
        self.nsys = int(len(self.lengths))
        # longest systems first: the persistent grid takes them in order
        order = np.argsort(-self.lengths, kind="stable").astype(np.int32)
        self.offsets = torch.as_tensor(offs, dtype=torch.int64,
                                       device=self.device)
        self.order = torch.as_tensor(order, device=self.device)
        self.lib = native.block_thomas_lib()
        wd = int(self.lib.pyro_block_thomas_work_doubles(self.nv, self.rows))
        self.work = torch.empty(max(1, wd), dtype=torch.float64,
                                device=self.device)
        self.counter = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.threads = int(threads) if threads else default_threads(self.nv)
        self.ctas = int(ctas)
        self.use_graph = bool(use_graph)
        self._graph = None
        self._graph_key = None

    def _launch(self, L, C, U, b, x, stream):
        _check(self.lib.pyro_block_thomas(
            L.data_ptr(), C.data_ptr(), U.data_ptr(), b.data_ptr(),
            x.data_ptr(), self.offsets.data_ptr(), self.order.data_ptr(),
            self.nsys, self.nv, self.work.data_ptr(),
            self.counter.data_ptr(), self.status.data_ptr(), self.threads,
            self.ctas, ctypes.c_void_p(stream.cuda_stream)),
            "pyro_block_thomas")

    def _check_shapes(self, L, C, U, b):
        nv, rows = self.nv, self.rows
        for name, t, shape in (("L", L, (rows, nv, nv)),
                               ("C", C, (rows, nv, nv)),
                               ("U", U, (rows, nv, nv)),
                               ("b", b, (rows, nv))):
            if tuple(t.shape) != shape:
                raise ValueError(f"{name} must have shape {shape}")
            if not (t.is_cuda and t.dtype == torch.float64
                    and t.is_contiguous()):
                raise ValueError(f"{name} must be a contiguous CUDA float64 "
                                 "tensor")

    def solve(self, L, C, U, b, out=None):
        """x for the packed systems; raises on a zero pivot."""
        self._check_shapes(L, C, U, b)
        x = out if out is not None else torch.empty_like(b)
        stream = torch.cuda.current_stream(self.device)
        if self.use_graph:
            key = tuple(t.data_ptr() for t in (L, C, U, b, x))
            if self._graph is None or self._graph_key != key:
                # warm-up launch outside capture, then capture
                self._launch(L, C, U, b, x, stream)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._launch(L, C, U, b, x,
                                 torch.cuda.current_stream(self.device))
                self._graph, self._graph_key = g, key
            self._graph.replay()
        else:
            self._launch(L, C, U, b, x, stream)
        return x

    def check_status(self):
        if int(self.status.item()) != 0:
            self.status.zero_()
            raise RuntimeError("block-Thomas: singular diagonal block")


def default_threads(nv: int) -> int:
    """CTA size: from the autotuner cache when present, else one warp for
    small blocks and up to 128 threads for larger ones."""
    best = _tuned().get(str(nv))
    if best:
        return int(best)
    if nv <= 12:
        return 32
    if nv <= 24:
        return 64
    return 128


def _tune_path():
    from .codegen.cuda import default_build_dir
    return os.path.join(default_build_dir(), "block_thomas_tuning.json")


def _tuned():
    try:
        with open(_tune_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def autotune(nv: int, n_systems: int = 304, n_min: int = 64,
             n_max: int = 1024, candidates=(32, 64, 128, 256),
             seed: int = 0, device=None, repeats: int = 3):
    """Time the solve for each CTA size on a seeded sample of systems of
    the given shape; store the fastest in the build directory's tuning
    file and return ``{threads: ms}``."""
    rng = np.random.default_rng(seed)
    lengths = rng.integers(n_min, n_max + 1, size=n_systems)
    dev = torch.device(device if device is not None else "cuda")
    rows = int(lengths.sum())
    gen = torch.Generator(device=dev).manual_seed(seed)
    C = torch.randn((rows, nv, nv), dtype=torch.float64, device=dev,
                    generator=gen) + 10.0 * torch.eye(
        nv, dtype=torch.float64, device=dev)
    L = torch.randn((rows, nv, nv), dtype=torch.float64, device=dev,
                    generator=gen)
    U = torch.randn((rows, nv, nv), dtype=torch.float64, device=dev,
                    generator=gen)
    b = torch.randn((rows, nv), dtype=torch.float64, device=dev,
                    generator=gen)
    times = {}
    for th in candidates:
        if nv > th and th < 64:
            continue
        solver = BlockThomasSolver(nv, lengths, device=dev, threads=th)
        solver.solve(L, C, U, b)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
        e0.record()
        for _ in range(repeats):
            solver.solve(L, C, U, b)
        e1.record()
        torch.cuda.synchronize(dev)
        times[th] = e0.elapsed_time(e1) / repeats
    best = min(times, key=times.get)
    tuned = _tuned()
    tuned[str(nv)] = int(best)
    os.makedirs(os.path.dirname(_tune_path()), exist_ok=True)
    with open(_tune_path(), "w") as f:
        json.dump(tuned, f)
    return times


def block_thomas(lower, central, upper, rhs):
    """One block-tridiagonal system, the signature of
    ``pyrometheus.flamelets.linear_solver.block_thomas``: ``lower`` /
    ``upper`` (N-1, nv, nv), ``central`` (N, nv, nv), ``rhs`` (N, nv);
    returns x (N, nv) on the GPU."""
    dev = central.device if isinstance(central, torch.Tensor) else "cuda"
    f64 = dict(dtype=torch.float64, device=dev)
    C = torch.as_tensor(central, **f64).contiguous()
    n, nv = C.shape[0], C.shape[1]
    L = torch.zeros((n, nv, nv), **f64)
    U = torch.zeros((n, nv, nv), **f64)
    if n > 1:
        L[:n - 1] = torch.as_tensor(lower, **f64)
        U[:n - 1] = torch.as_tensor(upper, **f64)
    b = torch.as_tensor(rhs, **f64).contiguous()
    solver = BlockThomasSolver(nv, [n], device=dev)
    x = solver.solve(L, C, U, b)
    solver.check_status()
    return x
