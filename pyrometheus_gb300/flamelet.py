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

    ``kernel``: ``"cta"`` (one CTA per system, threads over matrix
    elements; any nv <= 64), ``"seg"`` (32 // nv systems per warp, one lane
    per block row, each system eliminated from both ends to its middle
    row; nv <= 16; re-solves through its own two-ended recurrence) or
    ``"small"`` (one thread per system, nv <= 16); ``threads``: CTA size
    (``"cta"``: a multiple of 32; ``"small"``: 32 or 64 systems per CTA;
    ``"seg"``: recorded as 32, the kernel's CTAs are four warps); both
    ``None`` pick from the autotuner cache or a size rule (``"seg"`` for
    nv <= 16).  ``ctas``: persistent grid (0: the kernel's default; for
    ``"seg"`` one or two warps per SM partition by the batch size);
    ``use_graph``: capture the launch in a CUDA graph on the first
    :meth:`solve` with given buffers and replay it afterwards.
    """

    def __init__(self, nv: int, lengths: Sequence[int], device=None,
                 threads: Optional[int] = None, ctas: int = 0,
                 use_graph: bool = False, kernel: Optional[str] = None):
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
        if kernel is None and threads is None:
            kernel, threads = default_plan(self.nv)
        self.kernel = kernel or "cta"
        if self.kernel not in ("cta", "small", "seg"):
            raise ValueError(f"unknown block-Thomas kernel {kernel!r}")
        if self.kernel in ("small", "seg") and self.nv > 16:
            raise ValueError(f"the {self.kernel!r} kernel takes nv <= 16")
        if self.kernel == "seg":
            self.threads = 32
        else:
            self.threads = int(threads) if threads else (
                _small_threads(self.nv) if self.kernel == "small"
                else default_threads(self.nv))
        self.ctas = int(ctas)
        self.use_graph = bool(use_graph)
        self._graph = None
        self._graph_key = None
        self._factored = False

    def _launch(self, L, C, U, b, x, stream):
        if self.kernel == "seg":
            _check(self.lib.pyro_block_thomas_seg(
                L.data_ptr(), C.data_ptr(), U.data_ptr(), b.data_ptr(),
                x.data_ptr(), self.offsets.data_ptr(), self.order.data_ptr(),
                self.nsys, self.nv, self.work.data_ptr(),
                self.counter.data_ptr(), self.status.data_ptr(), self.ctas,
                ctypes.c_void_p(stream.cuda_stream)),
                "pyro_block_thomas_seg")
            return
        if self.kernel == "small":
            _check(self.lib.pyro_block_thomas_small(
                L.data_ptr(), C.data_ptr(), U.data_ptr(), b.data_ptr(),
                x.data_ptr(), self.offsets.data_ptr(), self.order.data_ptr(),
                self.nsys, self.nv, self.work.data_ptr(),
                self.status.data_ptr(), self.threads,
                ctypes.c_void_p(stream.cuda_stream)),
                "pyro_block_thomas_small")
            return
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
        self._factored = True
        return x

    def resolve(self, L, U, B, out=None):
        """Solutions for further right-hand sides of the systems the last
        :meth:`solve` factorised (its LU factors stay in the workspace):
        ``B`` is ``[rows, nv]`` or ``[nrhs, rows, nv]``; ``L`` and ``U``
        must be that call's blocks.  Only the vector recurrences run
        (``4 nv^2`` FMAs per row and right-hand side)."""
        if not self._factored:
            raise RuntimeError("resolve() needs a solve() with the same "
                               "blocks first")
        nv, rows = self.nv, self.rows
        single = B.dim() == 2
        Bv = B[None] if single else B
        if tuple(Bv.shape[1:]) != (rows, nv) or not (
                Bv.is_cuda and Bv.dtype == torch.float64
                and Bv.is_contiguous()):
            raise ValueError(f"B must be a contiguous CUDA float64 tensor of "
                             f"shape {(rows, nv)} or (nrhs, {rows}, {nv})")
        for name, t in (("L", L), ("U", U)):
            if tuple(t.shape) != (rows, nv, nv) or not t.is_contiguous():
                raise ValueError(f"{name} must be the solved system's "
                                 "blocks")
        X = out if out is not None else torch.empty_like(B)
        Xv = X[None] if single else X
        if Xv.shape != Bv.shape or not Xv.is_contiguous():
            raise ValueError("out must be contiguous and shaped like B")
        stream = torch.cuda.current_stream(self.device)
        n = Bv.shape[0]
        fn = (self.lib.pyro_block_thomas_seg_resolve if self.kernel == "seg"
              else self.lib.pyro_block_thomas_resolve)
        for c0 in range(0, n, 4):
            k = min(4, n - c0)
            _check(fn(
                L.data_ptr(), U.data_ptr(), Bv[c0].data_ptr(),
                Xv[c0].data_ptr(), k, rows * nv, self.offsets.data_ptr(),
                self.order.data_ptr(), self.nsys, nv, self.work.data_ptr(),
                self.counter.data_ptr(), self.status.data_ptr(),
                ctypes.c_void_p(stream.cuda_stream)),
                "block-Thomas re-solve")
        return X

    def check_status(self):
        st = int(self.status.item())
        if st != 0:
            self.status.zero_()
            if st & 1:
                raise RuntimeError("block-Thomas: singular diagonal block")
            raise RuntimeError("block-Thomas: a system with no rows")


def default_threads(nv: int) -> int:
    """CTA size of the one-CTA-per-system kernel: from the autotuner cache
    when it holds one, else the sizes the autotuner picks on GB300."""
    best = _tuned().get(str(nv))
    if best and str(best).startswith("cta:"):
        return int(str(best).split(":")[-1])
    # the autotuner's choices on GB300 for 4,096 systems of 64..1024 rows:
    # 128 threads at nv = 10, 256 at nv = 54
    return 128 if nv <= 24 else 256


def _small_threads(nv: int) -> int:
    """Systems per CTA of the one-thread-per-system kernel: 64 while three
    blocks per thread fit the 227 KB of shared memory, else 32."""
    return 64 if 3 * nv * (nv + 1) * 8 * 64 <= 227 * 1024 else 32


def default_plan(nv: int):
    """(kernel, threads): the autotuner's choice when cached, else the
    several-systems-per-warp kernel for nv <= 16 (3.1x the CTA kernel at
    nv = 10 on 4,096 systems) and the one-CTA-per-system kernel above."""
    best = _tuned().get(str(nv))
    if best:
        kind, _, th = str(best).rpartition(":")
        return (kind or "cta"), int(th)
    if nv <= 16:
        return "seg", 32
    return "cta", default_threads(nv)


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
             n_max: int = 1024,
             candidates=(32, 64, 96, 128, 192, 256, 384, 512),
             seed: int = 0, device=None, repeats: int = 3, lengths=None):
    """Time the solve for each kernel and CTA size (the CTA kernel at each
    of *candidates*, and for nv <= 16 the several-systems-per-warp kernel
    and the one-thread-per-system kernel at 32 and 64 systems per CTA) on a
    seeded sample of systems of the given
    shape (or on systems of the given *lengths*); store the fastest in the
    build directory's tuning file and return ``{"kernel:threads": ms}``."""
    rng = np.random.default_rng(seed)
    if lengths is None:
        lengths = rng.integers(n_min, n_max + 1, size=n_systems)
    lengths = np.asarray(lengths, dtype=np.int64)
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
    # CTAs narrower than a block row, or wider than 256 threads for blocks
    # of at most 24 (too few matrix elements to share), are skipped
    plans = [("cta", th) for th in candidates
             if not (nv > th and th < 64) and not (nv <= 24 and th > 256)]
    if nv <= 16:
        plans += [("seg", 32)]
        plans += [("small", th) for th in (32, 64)
                  if 3 * nv * (nv + 1) * 8 * th <= 227 * 1024]
    times = {}
    for kind, th in plans:
        solver = BlockThomasSolver(nv, lengths, device=dev, threads=th,
                                   kernel=kind)
        solver.solve(L, C, U, b)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(True), torch.cuda.Event(True)
        e0.record()
        for _ in range(repeats):
            solver.solve(L, C, U, b)
        e1.record()
        torch.cuda.synchronize(dev)
        times[f"{kind}:{th}"] = e0.elapsed_time(e1) / repeats
    best = min(times, key=times.get)
    tuned = _tuned()
    tuned[str(nv)] = best
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


class FlameletEquations:
    """Steady-flamelet residual and block-tridiagonal Jacobian for many
    flamelets at once, on the GPU: the counterpart of
    ``pyrometheus.flamelets.equations.FlameletEquations`` (``rhs``
    ``equations.py:167-227``, ``jac`` :228-282, ``source_terms`` :313-359)
    with the Laplacian of ``onedim_laplacian.py:144-180``.

    Flamelets are packed along rows as for :class:`BlockThomasSolver`:
    flamelet ``s`` owns ``lengths[s]`` (>= 3) consecutive grid points on a
    uniform mixture-fraction grid of spacing ``dx[s]``.  The unknowns are
    ``h[rows]`` and ``Y[S, rows]``; ``jac`` returns the packed ``(L, C,
    U)`` blocks ``[rows, S+1, S+1]`` the solver takes (the last row of each
    flamelet's ``L``/``U`` is zero and unused).  ``y_ox``/``y_fu``: ``[S]``
    (shared) or ``[S, n_flamelets]``.
    """

    def __init__(self, thermo, lengths, dx, y_ox, y_fu, device=None):
        self.th = thermo
        self.S = thermo.num_species
        self.nv = self.S + 1
        self.device = torch.device(device if device is not None
                                   else thermo.device)
        lengths = np.asarray(lengths, dtype=np.int64)
        if np.any(lengths < 3):
            raise ValueError("every flamelet needs at least 3 grid points")
        self.lengths = lengths
        self.nsys = int(len(lengths))
        offs = np.concatenate([[0], np.cumsum(lengths)])
        self.rows = int(offs[-1])
        dev = self.device
        self.row_off = torch.as_tensor(offs, dtype=torch.int64, device=dev)
        self.sys_of_row = torch.as_tensor(
            np.repeat(np.arange(self.nsys, dtype=np.int32), lengths),
            device=dev)
        dx = np.broadcast_to(np.asarray(dx, dtype=np.float64), (self.nsys,))
        self.dx = np.array(dx)
        self.inv_dx2 = torch.as_tensor(1.0 / dx ** 2, device=dev)
        self.y_ox = self._bc_mat(y_ox)
        self.y_fu = self._bc_mat(y_fu)

    def subset(self, systems):
        """The equations of the flamelets *systems* (indices into this
        batch, in the order given), packed in that order."""
        idx = np.asarray(systems, dtype=np.int64)
        sel = torch.as_tensor(idx, device=self.device)
        return FlameletEquations(self.th, self.lengths[idx], self.dx[idx],
                                 self.y_ox[:, sel], self.y_fu[:, sel],
                                 device=self.device)

    def linear_solver(self):
        """A :class:`BlockThomasSolver` for these flamelets' blocks."""
        return BlockThomasSolver(self.nv, self.lengths, device=self.device)

    def _bc_mat(self, y):
        y = torch.as_tensor(np.asarray(y, dtype=np.float64)
                            if not torch.is_tensor(y) else y,
                            dtype=torch.float64, device=self.device)
        if y.dim() == 1:
            y = y[:, None].expand(self.S, self.nsys)
        return y.contiguous()

    def _rowvec(self, x):
        if torch.is_tensor(x):
            x = x.to(device=self.device, dtype=torch.float64)
        else:
            x = torch.as_tensor(np.asarray(x, dtype=np.float64),
                                device=self.device)
        if x.dim() == 0:
            x = x.expand(self.rows)
        return x.contiguous()

    def _sysvec(self, x):
        if torch.is_tensor(x):
            x = x.to(device=self.device, dtype=torch.float64)
        else:
            x = torch.as_tensor(np.asarray(x, dtype=np.float64),
                                device=self.device)
        if x.dim() == 0:
            x = x.expand(self.nsys)
        return x.contiguous()

    def _state(self, h, Y):
        h = self._rowvec(h)
        Y = Y.to(device=self.device, dtype=torch.float64) if torch.is_tensor(
            Y) else torch.as_tensor(np.asarray(Y, dtype=np.float64),
                                    device=self.device)
        if tuple(Y.shape) != (self.S, self.rows):
            raise ValueError(f"Y must have shape {(self.S, self.rows)}")
        return h, Y.contiguous()

    def _pressure(self, pressure):
        p = self._rowvec(pressure)
        return p, (0 if p.stride(0) == 0 else 1)

    @staticmethod
    def _stream():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def temperature(self, h, Y, temp_guess, check=True):
        """T with h_mix(T, Y) = h (``equation_of_state``,
        ``equations.py:284-311``).  ``check=False`` returns the last
        iterate of states whose iteration did not converge (nan for nan
        states) instead of raising."""
        if check:
            return self.th.get_temperature_from_enthalpy(
                h, Y, self._rowvec(temp_guess))
        return self.th._temperature(h, self._rowvec(temp_guess), Y, False,
                                    1.0e-10, 500, check=False)

    def equation_of_state(self, h, Y, temp_guess, pressure):
        """``(density [rows], temperature [rows])`` from the state:
        T(h, Y) by the enthalpy Newton, then the ideal-gas density
        (``equation_of_state``, ``equations.py:284-311``)."""
        h, Y = self._state(h, Y)
        T = self.temperature(h, Y, temp_guess)
        p, _ = self._pressure(pressure)
        return self.th.get_density(p, T, Y), T

    def source_terms(self, h, Y, viscous_diss, temp_guess, pressure,
                     temperature=None):
        """``(S_h [rows], S_Y [S, rows])``: the point-wise source
        ``(v / rho, W w / rho)`` (``source_terms``,
        ``equations.py:313-359``)."""
        h, Y = self._state(h, Y)
        T = temperature if temperature is not None else \
            self.temperature(h, Y, temp_guess)
        p, _ = self._pressure(pressure)
        F = self.th.get_reactor_source(p, T, Y)
        rho = self.th.get_density(p, T, Y)
        return self._rowvec(viscous_diss) / rho, F[1:]

    def boundary_conditions(self, h_ox, h_fu):
        """``(BC_h [rows], BC_Y [S, rows])``: ``h_ox``/``y_ox`` at each
        flamelet's first point, ``h_fu``/``y_fu`` at its last, zero inside
        (``boundary_conditions``, ``equations.py:391-409``)."""
        f64 = dict(dtype=torch.float64, device=self.device)
        bh = torch.zeros(self.rows, **f64)
        by = torch.zeros((self.S, self.rows), **f64)
        first, last = self.row_off[:-1], self.row_off[1:] - 1
        bh[first] = self._sysvec(h_ox)
        bh[last] = self._sysvec(h_fu)
        by[:, first] = self.y_ox
        by[:, last] = self.y_fu
        return bh, by

    def jacobian_action(self, v, h, Y, diss_rate, viscous_diss, temp_guess,
                        pressure, temperature=None):
        """``chi/2 Lap(v) + dS/dphi v`` per point, ``[S+1, rows]`` for a
        direction ``v`` ``[S+1, rows]`` (row 0 enthalpy): the matrix-free
        product of ``jacobian_action`` (``equations.py:411-450``), with
        every point's source Jacobian (the boundary points keep theirs,
        unlike :meth:`jac`'s blocks)."""
        h, Y = self._state(h, Y)
        T = temperature if temperature is not None else \
            self.temperature(h, Y, temp_guess)
        p, p_inc = self._pressure(pressure)
        v = v.to(device=self.device, dtype=torch.float64) if \
            torch.is_tensor(v) else torch.as_tensor(
                np.asarray(v, dtype=np.float64), device=self.device)
        if tuple(v.shape) != (self.nv, self.rows):
            raise ValueError(f"v must have shape {(self.nv, self.rows)}")
        v = v.contiguous()
        J = self.th.get_reactor_jacobian(p, T, Y)
        chi, visc = self._rowvec(diss_rate), self._rowvec(viscous_diss)
        A = torch.empty((self.nv, self.rows), dtype=torch.float64,
                        device=self.device)
        _check(self.th._lib.pyro_flamelet_jacobian_action(
            p.data_ptr(), p_inc, T.data_ptr(), Y.data_ptr(), Y.stride(0),
            J.data_ptr(), v.data_ptr(), v.stride(0), chi.data_ptr(),
            visc.data_ptr(), self.row_off.data_ptr(),
            self.sys_of_row.data_ptr(), self.inv_dx2.data_ptr(),
            A.data_ptr(), A.stride(0), self.rows, self._stream()),
            "flamelet Jacobian action")
        return A

    def rhs(self, h, Y, diss_rate, viscous_diss, temp_guess, pressure,
            h_ox, h_fu, temperature=None):
        """Residual ``[S+1, rows]`` (row 0 enthalpy, rows 1.. species)."""
        h, Y = self._state(h, Y)
        T = temperature if temperature is not None else \
            self.temperature(h, Y, temp_guess)
        p, p_inc = self._pressure(pressure)
        F = self.th.get_reactor_source(p, T, Y)
        chi, visc = self._rowvec(diss_rate), self._rowvec(viscous_diss)
        hox, hfu = self._sysvec(h_ox), self._sysvec(h_fu)
        R = torch.empty((self.nv, self.rows), dtype=torch.float64,
                        device=self.device)
        _check(self.th._lib.pyro_flamelet_residual(
            p.data_ptr(), p_inc, T.data_ptr(), h.data_ptr(), Y.data_ptr(),
            Y.stride(0), F.data_ptr(), F.stride(0), chi.data_ptr(),
            visc.data_ptr(), self.row_off.data_ptr(),
            self.sys_of_row.data_ptr(), self.inv_dx2.data_ptr(),
            hox.data_ptr(), hfu.data_ptr(), self.y_ox.data_ptr(),
            self.y_fu.data_ptr(), self.y_ox.stride(0), R.data_ptr(),
            R.stride(0), self.rows, self._stream()), "flamelet residual")
        return R

    def jac(self, h, Y, diss_rate, viscous_diss, temp_guess, pressure,
            temperature=None, out=None):
        """Packed ``(L, C, U)`` blocks ``[rows, S+1, S+1]``."""
        h, Y = self._state(h, Y)
        T = temperature if temperature is not None else \
            self.temperature(h, Y, temp_guess)
        p, p_inc = self._pressure(pressure)
        nv = self.nv
        if out is None:
            f64 = dict(dtype=torch.float64, device=self.device)
            out = tuple(torch.empty((self.rows, nv, nv), **f64)
                        for _ in range(3))
        L, C, U = out
        self.th.get_reactor_jacobian(p, T, Y, out=C)
        chi, visc = self._rowvec(diss_rate), self._rowvec(viscous_diss)
        _check(self.th._lib.pyro_flamelet_blocks(
            p.data_ptr(), p_inc, T.data_ptr(), Y.data_ptr(), Y.stride(0),
            chi.data_ptr(), visc.data_ptr(), self.row_off.data_ptr(),
            self.sys_of_row.data_ptr(), self.inv_dx2.data_ptr(),
            L.data_ptr(), C.data_ptr(), U.data_ptr(), self.rows,
            self._stream()), "flamelet blocks")
        return L, C, U

    # {{{ compressible-EOS consistency (thermodynamic_consistency.py)

    def adjoint_operator(self, h, Y, diss_rate, viscous_diss, temp_guess,
                         pressure, temperature=None, out=None):
        """Packed ``(L, C, U)`` of the adjoint operator of the
        EOS-consistency solves (``FlameletEquations.adjoint_operator``,
        ``equations.py:451-516``): ``Lap_c + (2/chi) dS/dphi^T`` inside,
        ``chi/2 Lap_c`` at the boundary points, the Laplacian's own
        couplings."""
        h, Y = self._state(h, Y)
        T = temperature if temperature is not None else \
            self.temperature(h, Y, temp_guess)
        p, p_inc = self._pressure(pressure)
        nv = self.nv
        if out is None:
            f64 = dict(dtype=torch.float64, device=self.device)
            out = tuple(torch.empty((self.rows, nv, nv), **f64)
                        for _ in range(3))
        L, C, U = out
        self.th.get_reactor_jacobian(p, T, Y, out=C)
        chi, visc = self._rowvec(diss_rate), self._rowvec(viscous_diss)
        _check(self.th._lib.pyro_flamelet_adjoint_blocks(
            p.data_ptr(), p_inc, T.data_ptr(), Y.data_ptr(), Y.stride(0),
            chi.data_ptr(), visc.data_ptr(), self.row_off.data_ptr(),
            self.sys_of_row.data_ptr(), self.inv_dx2.data_ptr(),
            L.data_ptr(), C.data_ptr(), U.data_ptr(), self.rows,
            self._stream()), "flamelet adjoint blocks")
        return L, C, U

    def eos_rt(self, h, Y, temp_guess=None, temperature=None,
               jacobian=True):
        """``(R T [rows], d(R T)/dphi [S+1, rows] or None)`` with
        ``R = R_u / W_mix`` at T(h, Y) (``compressible_eos_rt`` and
        ``compressible_eos_rt_jacobian``, ``equations.py:136-147,517-535``)."""
        h, Y = self._state(h, Y)
        T = temperature if temperature is not None else \
            self.temperature(h, Y, temp_guess)
        f64 = dict(dtype=torch.float64, device=self.device)
        rt = torch.empty(self.rows, **f64)
        J = torch.empty((self.nv, self.rows), **f64) if jacobian else None
        _check(self.th._lib.pyro_flamelet_eos_rt(
            T.data_ptr(), Y.data_ptr(), Y.stride(0), rt.data_ptr(),
            J.data_ptr() if J is not None else None,
            J.stride(0) if J is not None else self.rows, self.rows,
            self._stream()), "flamelet eos rt")
        return rt, J

    def source_gradient_wrt_pressure(self, h, Y, viscous_diss, temp_guess,
                                     pressure, temperature=None):
        """dS/dp per point, ``[rows, S+1]`` (``source_gradient_wrt_pressure``,
        ``equations.py:130-134``): ``-S_h / p`` for the enthalpy source
        ``v / rho`` and the reactor source's pressure derivative for the
        species rows (T(h, Y) does not depend on p)."""
        h, Y = self._state(h, Y)
        T = temperature if temperature is not None else \
            self.temperature(h, Y, temp_guess)
        p, _ = self._pressure(pressure)
        visc = self._rowvec(viscous_diss)
        dfdp = self.th.get_reactor_source_dp(p, T, Y)
        rho = self.th.get_density(p, T, Y)
        dfdp[0] = -(visc / rho) / p
        return dfdp.T

    def _sys_index(self):
        if getattr(self, "_sidx", None) is None:
            r0 = self.row_off[:-1]
            r1 = self.row_off[1:]
            self._sidx = (r0, r0 + 1, r0 + 2, r1 - 1, r1 - 2, r1 - 3)
            w = torch.ones(self.rows, dtype=torch.float64, device=self.device)
            w[r0] = 0.5
            w[r1 - 1] = 0.5
            self._trap_w = w
            # (flamelet, position) of every row: per-flamelet sums as a
            # dense [nsys, max length] reduction, in a fixed order
            pos = np.concatenate([np.arange(n) for n in self.lengths])
            self._pos = torch.as_tensor(pos, dtype=torch.int64,
                                        device=self.device)
        return self._sidx

    def _traces(self, a):
        """Per flamelet ``(1.5 a_0 + 2 a_1 - 0.5 a_2) / dx^2 + (1.5 a_{-1}
        + 2 a_{-2} - 0.5 a_{-3}) / dx^2`` of a per-row field
        (``thermodynamic_consistency.py:159-168``)."""
        i0, i1, i2, j0, j1, j2 = self._sys_index()
        ox = (1.5 * a[i0] + 2 * a[i1] - 0.5 * a[i2]) * self.inv_dx2
        fu = (1.5 * a[j0] + 2 * a[j1] - 0.5 * a[j2]) * self.inv_dx2
        return ox + fu

    def _trapezoid(self, f):
        """Per flamelet ``(f_0 + f_{N-1}) / 2 + sum of the interior``
        (``trapezoidal_rule``, ``thermodynamic_consistency.py:31-42``)."""
        self._sys_index()
        dense = torch.zeros((self.nsys, int(self.lengths.max())),
                            dtype=torch.float64, device=self.device)
        dense[self.sys_of_row.long(), self._pos] = f * self._trap_w
        return dense.sum(dim=1)

    def _eos_solver(self, solver):
        if solver is not None:
            return solver
        if getattr(self, "_bt", None) is None:
            self._bt = BlockThomasSolver(self.nv, self.lengths,
                                         device=self.device)
        return self._bt

    def enthalpy_gradient(self, h, Y, diss_rate, viscous_diss, temp_guess,
                          pressure, pdf, solver=None):
        """``(R T [rows], adjoint_h [S+1, rows], h_gradient [nsys])``: the
        adjoint solve with right-hand side ``-e_h pdf`` and its boundary
        traces, for every flamelet (``CompressibleEOS.enthalpy_gradient``,
        ``thermodynamic_consistency.py:105-171``)."""
        h, Y = self._state(h, Y)
        T = self.temperature(h, Y, temp_guess)
        rt, _ = self.eos_rt(h, Y, temperature=T, jacobian=False)
        L, C, U = self.adjoint_operator(h, Y, diss_rate, viscous_diss, None,
                                        pressure, temperature=T)
        b = torch.zeros((self.rows, self.nv), dtype=torch.float64,
                        device=self.device)
        b[:, 0] = -self._rowvec(pdf)
        bt = self._eos_solver(solver)
        adj = bt.solve(L, C, U, b).T
        bt.check_status()
        return rt, adj, self._traces(adj[0])

    def eos_gradient(self, h, Y, diss_rate, viscous_diss, temp_guess,
                     pressure, pdf, solver=None):
        """``((density_gradient [2, nsys], energy_gradient [2, nsys]),
        (adjoint_d, adjoint_e) [S+1, rows])`` for every flamelet
        (``CompressibleEOS.eos_gradient``,
        ``thermodynamic_consistency.py:173-307``): row 0 of a gradient is
        d/dp, row 1 d/dh at the boundaries.  The two adjoint solves share
        one factorisation (``BlockThomasSolver.resolve``); the pressure
        sensitivity of the source is formed once in forward mode
        (:meth:`source_gradient_wrt_pressure`) and contracted with both
        adjoint states."""
        h, Y = self._state(h, Y)
        T = self.temperature(h, Y, temp_guess)
        p, _ = self._pressure(pressure)
        chi, visc = self._rowvec(diss_rate), self._rowvec(viscous_diss)
        pdf = self._rowvec(pdf)
        rt, rtj = self.eos_rt(h, Y, temperature=T)
        L, C, U = self.adjoint_operator(h, Y, chi, visc, None, p,
                                        temperature=T)
        f64 = dict(dtype=torch.float64, device=self.device)
        B = torch.empty((2, self.rows, self.nv), **f64)
        B[0] = (rtj * ((p / rt ** 2) * pdf)).T
        B[1] = (rtj * pdf).T
        B[1][:, 0] -= pdf
        X = torch.empty_like(B)
        bt = self._eos_solver(solver)
        bt.solve(L, C, U, B[0], out=X[0])
        bt.resolve(L, U, B[1:], out=X[1:])
        bt.check_status()
        adj_d, adj_e = X[0].T, X[1].T
        # dS/dp once (forward mode), contracted with both adjoint states
        dsdp = self.source_gradient_wrt_pressure(h, Y, visc, None, p,
                                                 temperature=T).T
        half_chi = 0.5 * chi
        out = []
        for adj, base in ((adj_d, pdf / rt), (adj_e, None)):
            g = (adj * dsdp).sum(dim=0) / half_chi
            integrand = g if base is None else base + g
            out.append(torch.stack([self._trapezoid(integrand),
                                    self._traces(adj[0])]))
        return (out[0], out[1]), (adj_d, adj_e)

    # }}}

    def newton_step(self, h, Y, diss_rate, viscous_diss, temp_guess,
                    pressure, h_ox, h_fu, solver=None):
        """One Newton correction for every flamelet: ``(dphi [S+1, rows],
        R, T)`` with ``J dphi = -R``; *solver* is a
        :class:`BlockThomasSolver` for these lengths (built on first use
        when omitted)."""
        h, Y = self._state(h, Y)
        T = self.temperature(h, Y, temp_guess)
        R = self.rhs(h, Y, diss_rate, viscous_diss, None, pressure, h_ox,
                     h_fu, temperature=T)
        L, C, U = self.jac(h, Y, diss_rate, viscous_diss, None, pressure,
                           temperature=T)
        if solver is None:
            solver = BlockThomasSolver(self.nv, self.lengths,
                                       device=self.device)
        x = solver.solve(L, C, U, (-R).T.contiguous())
        return x.T, R, T
