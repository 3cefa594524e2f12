"""Continuous-batching server for implicit 0-D reactor integrations.

A request is a batch of cells -- adiabatic constant-pressure reactors
(``Thermochemistry.get_reactor_source``) with their own initial ``T``,
``Y``, pressure -- to integrate to ``t_end``.  The server keeps, per
mechanism, a fixed-capacity pool of cell slots resident in HBM (state,
history, step sizes, Jacobian and Newton workspaces); the capacity comes
from an HBM budget.  Between engine steps it admits queued requests into free
slots (first fit, arrival order), so requests that arrive while others are on
the GPU join the running batch; each engine step advances every occupied slot
by one implicit step, and finished requests are copied back and completed.

Integrator (per cell, independent of the batch): variable-step BDF2 started
with one backward-Euler step (the reference's implicit reactor stepping,
``examples/free_flame/time_integ.py:72-106``, uses Crank-Nicolson with a
Newton loop and ``jnp.linalg.solve``); Newton iterations use the analytic
Jacobian kernel and a batched LU solve (the block-Thomas kernel on
length-one systems); weighted RMS norms with ``rtol`` / ``atol``; local
error from the predictor-corrector difference; per-cell step acceptance and
step-size control.  Every quantity is computed per cell with the same
arithmetic whatever else is in the batch, so a request's result is the same
alone and in a mix.
"""

from __future__ import annotations

import ctypes
import heapq
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import native

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


@dataclass
class Request:
    rid: int
    mech: str
    T0: np.ndarray          # [n]
    Y0: np.ndarray          # [S, n]
    pressure: float
    t_end: float
    arrival: float = 0.0    # seconds on the server clock
    # filled by the server
    admitted: Optional[float] = None
    finished: Optional[float] = None
    T: Optional[np.ndarray] = None
    Y: Optional[np.ndarray] = None
    status: str = "queued"
    slots: Optional[np.ndarray] = None
    steps: Optional[np.ndarray] = None

    @property
    def n(self) -> int:
        return int(self.T0.shape[0])

    @property
    def latency(self) -> Optional[float]:
        if self.finished is None:
            return None
        return self.finished - self.arrival


class ReactorPool:
    """Device-resident slots of one mechanism and its integrator state."""

    BYTES_PER_CELL_DOUBLES = 4   # J, M, LU workspace + vectors (x nv^2)

    def __init__(self, thermo, capacity: int, rtol: float = 1e-8,
                 atol: float = 1e-14, max_newton: int = 6,
                 h0: float = 1e-10, stream=None):
        self.th = thermo
        self.S = thermo.num_species
        self.nv = self.S + 1
        self.cap = int(capacity)
        self.rtol, self.atol = float(rtol), float(atol)
        self.max_newton = int(max_newton)
        self.h0 = float(h0)
        self.h_min = 1e-14   # relative to t_end
        dev = thermo.device
        self.device = dev
        self.stream = stream if stream is not None else torch.cuda.Stream(
            dev)
        f64 = dict(dtype=torch.float64, device=dev)
        nv, cap = self.nv, self.cap
        with torch.cuda.stream(self.stream):
            self.y = torch.zeros((nv, cap), **f64)
            self.y_prev = torch.zeros((nv, cap), **f64)
            self.p = torch.ones(cap, **f64)
            self.t = torch.zeros(cap, **f64)
            self.t_end = torch.zeros(cap, **f64)
            self.h = torch.full((cap,), self.h0, **f64)
            self.h_prev = torch.ones(cap, **f64)
            self.f_prev = torch.zeros((nv, cap), **f64)
            self.nsteps = torch.zeros(cap, dtype=torch.int64, device=dev)
            self.active = torch.zeros(cap, dtype=torch.bool, device=dev)
            self.failed = torch.zeros(cap, dtype=torch.bool, device=dev)
            self.J = torch.empty((cap, nv, nv), **f64)
            self.rhs = torch.empty((cap, nv), **f64)
            self.dx = torch.empty((cap, nv), **f64)
            self.eye = torch.eye(nv, **f64)
            self.row_off = torch.arange(cap + 1, dtype=torch.int64,
                                        device=dev)
            self.order = torch.arange(cap, dtype=torch.int32, device=dev)
            lib = native.block_thomas_lib()
            wd = int(lib.pyro_block_thomas_work_doubles(nv, cap))
            self.work = torch.empty(wd, **f64)
            self.counter = torch.zeros(1, dtype=torch.int32, device=dev)
            self.lu_status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.lu = lib
        from .flamelet import default_threads
        self.lu_threads = default_threads(nv)
        self.free = list(range(cap))
        heapq.heapify(self.free)
        self.high_water = 0
        self.slot_req = np.full(cap, -1, dtype=np.int64)
        self.n_active = 0

    @classmethod
    def bytes_per_cell(cls, n_species: int) -> int:
        nv = n_species + 1
        return 8 * (3 * nv * nv + 8 * nv + 12)

    # -- slots -----------------------------------------------------------
    def can_admit(self, n: int) -> bool:
        return len(self.free) >= n

    def admit(self, req: Request) -> np.ndarray:
        slots = np.array([heapq.heappop(self.free) for _ in range(req.n)],
                         dtype=np.int64)
        self.high_water = max(self.high_water, int(slots.max()) + 1)
        self.slot_req[slots] = req.rid
        idx = torch.as_tensor(slots, device=self.device)
        with torch.cuda.stream(self.stream):
            y0 = torch.empty((self.nv, req.n), dtype=torch.float64)
            y0[0] = torch.from_numpy(np.asarray(req.T0, dtype=np.float64))
            y0[1:] = torch.from_numpy(np.asarray(req.Y0, dtype=np.float64))
            y0 = y0.to(self.device, non_blocking=False)
            self.y[:, idx] = y0
            self.y_prev[:, idx] = y0
            self.p[idx] = float(req.pressure)
            self.t[idx] = 0.0
            self.t_end[idx] = float(req.t_end)
            self.h[idx] = min(self.h0, float(req.t_end))
            self.h_prev[idx] = 1.0
            self.nsteps[idx] = 0
            self.f_prev[:, idx] = 0.0
            self.failed[idx] = False
            self.active[idx] = True
        self.n_active += req.n
        return slots

    def release(self, slots: np.ndarray):
        for s in slots.tolist():
            heapq.heappush(self.free, s)
        self.slot_req[slots] = -1
        self.n_active -= len(slots)
        occupied = np.nonzero(self.slot_req >= 0)[0]
        self.high_water = int(occupied.max()) + 1 if occupied.size else 0

    # -- numerics --------------------------------------------------------
    def _wrms(self, v, ref):
        w = self.rtol * ref.abs() + self.atol
        return torch.sqrt(((v / w) ** 2).mean(dim=0))

    def _lu_solve(self, n):
        """rhs[:n] <- M[:n]^-1 rhs[:n] (M in self.J, factorised in place
        in the workspace)."""
        st = self.lu.pyro_block_thomas(
            self.J.data_ptr(), self.J.data_ptr(), self.J.data_ptr(),
            self.rhs.data_ptr(), self.dx.data_ptr(),
            self.row_off.data_ptr(), self.order.data_ptr(), int(n), self.nv,
            self.work.data_ptr(), self.counter.data_ptr(),
            self.lu_status.data_ptr(), self.lu_threads, 0,
            ctypes.c_void_p(self.stream.cuda_stream))
        if st != 0:
            raise RuntimeError(f"batched LU failed (status {st})")

    def step(self):
        """One implicit step attempt for every occupied slot (asynchronous
        on the pool's stream)."""
        n = self.high_water
        if n == 0:
            return
        th = self.th
        with torch.cuda.stream(self.stream):
            act = self.active[:n]
            y, yp = self.y[:, :n], self.y_prev[:, :n]
            t, te = self.t[:n], self.t_end[:n]
            h = torch.minimum(self.h[:n], te - t)
            h = torch.where(act, h, torch.ones_like(h))
            first = self.nsteps[:n] == 0
            hp = self.h_prev[:n]
            om = torch.where(first, torch.zeros_like(h), h / hp)
            den = 1.0 + 2.0 * om
            ca = (1.0 + om) ** 2 / den
            cb = -(om * om) / den
            gh = (1.0 + om) / den * h
            base = ca * y + cb * yp
            # predictor: quadratic through y_{n-1}, y_n with slope f_n
            fp = self.f_prev[:, :n]
            cq = (yp - y + fp * hp) / (hp * hp)
            zp = torch.where(first, y, y + h * (fp + cq * h))
            z = zp.clone()
            p = self.p[:n]
            conv = ~act
            f = fp
            for _ in range(self.max_newton):
                f = th.get_reactor_source(p, z[0], z[1:])
                J = self.J[:n]
                th.get_reactor_jacobian(p, z[0], z[1:], out=J)
                # M = I - gamma h J ; G = z - base - gamma h f ; frozen
                # (converged / idle) cells solve I dx = 0
                live = ~conv
                J.mul_(-gh[:, None, None]).add_(self.eye)
                J[~live] = self.eye
                g = z - base - gh * f
                g = torch.where(live, g, torch.zeros_like(g))
                self.rhs[:n] = g.T
                self._lu_solve(n)
                dz = self.dx[:n].T
                z = z - dz
                conv = conv | (self._wrms(dz, z) < 1e-3)
            # BDF2 local error ~ 2 (z - z_pred) for the Hermite predictor
            # (constant-step error constants -2/9 and -1/3 of h^3 y^(3));
            # the first (backward-Euler) step is accepted on convergence
            err = 2.0 * self._wrms(z - zp, z)
            err = torch.where(first, torch.zeros_like(err), err)
            ok = act & conv & torch.isfinite(err) & (err <= 1.0)
            self.f_prev[:, :n] = torch.where(ok, f, fp)
            self.y_prev[:, :n] = torch.where(ok, y, yp)
            self.y[:, :n] = torch.where(ok, z, y)
            self.t[:n] = torch.where(ok, t + h, t)
            self.h_prev[:n] = torch.where(ok, h, self.h_prev[:n])
            self.nsteps[:n] += ok.to(torch.int64)
            fac = torch.clamp(0.9 * torch.pow(torch.clamp(err, min=1e-12),
                                              -1.0 / 3.0), 0.2, 4.0)
            fac = torch.where(conv, fac, torch.full_like(fac, 0.25))
            fac = torch.where(torch.isfinite(fac), fac,
                              torch.full_like(fac, 0.25))
            hn = torch.where(act, h * fac, self.h[:n])
            self.h[:n] = hn
            # a cell whose step collapses (or whose state is not finite)
            # fails instead of spinning: it leaves the batch with a flag
            bad = act & ((hn < self.h_min * te) |
                         ~torch.isfinite(self.y[:, :n]).all(dim=0))
            self.failed[:n] |= bad
            done = act & ((self.t[:n] >= te * (1.0 - 1e-12)) | bad)
            self.active[:n] = act & ~done
            self._done = done

    def finished_slots(self) -> np.ndarray:
        """Slots that completed in the last step (synchronises)."""
        if self.high_water == 0 or getattr(self, "_done", None) is None:
            return np.zeros(0, dtype=np.int64)
        self.stream.synchronize()
        fin = np.nonzero(self._done.cpu().numpy())[0]
        self._done = None
        return fin

    def results(self, slots: np.ndarray):
        """(T[n], Y[S, n], steps[n], failed[n]) of the given slots."""
        idx = torch.as_tensor(slots, device=self.device)
        with torch.cuda.stream(self.stream):
            yv = self.y[:, idx].cpu().numpy()
            ns = self.nsteps[idx].cpu().numpy()
            fl = self.failed[idx].cpu().numpy()
        return yv[0], yv[1:], ns, fl

    def deactivate(self, slots: np.ndarray):
        with torch.cuda.stream(self.stream):
            self.active[torch.as_tensor(slots, device=self.device)] = False
        self.stream.synchronize()

    def reset(self):
        """Drop every cell (after a failed engine step)."""
        with torch.cuda.stream(self.stream):
            self.active.zero_()
        self.stream.synchronize()
        self.free = list(range(self.cap))
        heapq.heapify(self.free)
        self.slot_req[:] = -1
        self.n_active = 0
        self.high_water = 0
        self._done = None


class ReactorServer:
    """Continuous batching over one pool per mechanism.

    *pools* maps mechanism names to pool objects (:class:`ReactorPool` or
    anything with its slot/step interface); :meth:`from_thermos` sizes one
    :class:`ReactorPool` per mechanism from an HBM budget.
    """

    def __init__(self, pools: Dict[str, object]):
        self.pools = dict(pools)
        self.queue: List[Request] = []
        self.running: Dict[int, Request] = {}
        self.done: List[Request] = []
        self.rejected: List[Request] = []
        self._remaining: Dict[int, int] = {}
        self.t0 = time.perf_counter()

    @classmethod
    def from_thermos(cls, thermos: Dict[str, object],
                     hbm_budget_bytes: float, rtol: float = 1e-8,
                     atol: float = 1e-14) -> "ReactorServer":
        """Equal cell counts per mechanism, as many as the budget holds
        (state, history, Jacobian/Newton matrices, LU workspace)."""
        total = sum(ReactorPool.bytes_per_cell(th.num_species)
                    for th in thermos.values())
        cap = int(hbm_budget_bytes / total)
        if cap < 1:
            raise ValueError("HBM budget too small for one cell")
        return cls({name: ReactorPool(th, cap, rtol=rtol, atol=atol)
                    for name, th in thermos.items()})

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, req: Request):
        pool = self.pools[req.mech]
        if req.n > pool.cap:
            req.status = "rejected: larger than the HBM budget"
            self.rejected.append(req)
            return
        self.queue.append(req)

    def cancel(self, rid: int) -> bool:
        for i, r in enumerate(self.queue):
            if r.rid == rid:
                r.status = "cancelled"
                self.done.append(self.queue.pop(i))
                return True
        r = self.running.get(rid)
        if r is not None:
            pool = self.pools[r.mech]
            pool.deactivate(r.slots)
            pool.release(r.slots)
            r.status = "cancelled"
            del self.running[rid]
            self.done.append(r)
            return True
        return False

    def _admit(self):
        now = self.now()
        keep = []
        for r in self.queue:
            pool = self.pools[r.mech]
            if r.arrival <= now and pool.can_admit(r.n):
                r.slots = pool.admit(r)
                r.admitted = now
                r.status = "running"
                self.running[r.rid] = r
                self._remaining[r.rid] = r.n
            else:
                keep.append(r)
        self.queue = keep

    def _harvest(self):
        for name, pool in self.pools.items():
            fin = pool.finished_slots()
            if fin.size == 0:
                continue
            rids = pool.slot_req[fin]
            for rid in np.unique(rids):
                self._remaining[int(rid)] -= int((rids == rid).sum())
                if self._remaining[int(rid)] == 0:
                    r = self.running.pop(int(rid))
                    r.T, r.Y, r.steps, failed = pool.results(r.slots)
                    r.finished = self.now()
                    r.status = "failed: integration did not converge" \
                        if failed.any() else "done"
                    pool.release(r.slots)
                    self.done.append(r)

    def _fail_pool(self, name: str, exc: BaseException):
        """An engine step raised: its running requests fail with the error,
        the pool is emptied, the other pools keep serving."""
        pool = self.pools[name]
        for rid in [rid for rid, r in self.running.items()
                    if r.mech == name]:
            r = self.running.pop(rid)
            r.status = f"failed: {type(exc).__name__}: {exc}"
            r.finished = self.now()
            self.done.append(r)
        pool.reset()

    def step(self):
        self._admit()
        for name, pool in self.pools.items():
            try:
                pool.step()
            except Exception as exc:  # noqa: BLE001 - isolate the pool
                self._fail_pool(name, exc)
        self._harvest()

    def idle(self) -> bool:
        return not self.queue and not self.running

    def run(self, requests: List[Request], time_limit: float = 60.0):
        """Serve *requests* (arrival times relative to now) until all are
        done or *time_limit* seconds pass; returns the completed ones."""
        self.t0 = time.perf_counter()
        pending = sorted(requests, key=lambda r: r.arrival)
        k = 0
        while True:
            now = self.now()
            while k < len(pending) and pending[k].arrival <= now:
                self.submit(pending[k])
                k += 1
            if self.idle():
                if k >= len(pending):
                    break
                time.sleep(max(0.0, min(1e-3, pending[k].arrival - now)))
                continue
            self.step()
            if now > time_limit:
                break
        return self.done


def latency_stats(done: List[Request]) -> Dict[str, float]:
    lat = np.array([r.latency for r in done if r.status == "done"])
    if lat.size == 0:
        return {"completed": 0}
    return {"completed": int(lat.size),
            "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}


def poisson_requests(rate: float, duration: float, mechs: Dict[str, object],
                     seed: int = 0, cells=(1, 65536), t_end: float = 1e-3,
                     pressure: float = 1e5, fuel_lean=(0.5, 1.0)):
    """Seeded Poisson arrivals: exponential gaps of mean 1/rate over
    *duration* s; cells log-uniform in *cells*; mechanism chosen uniformly;
    T0 ~ U[900, 1800] K; Y from an H2/O2/N2-type fuel-oxidiser-diluent
    mix between stoichiometric and lean (equivalence ratio in
    *fuel_lean*), read from the mechanism's species (``mechs`` maps names
    to Solution objects)."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    rid = 0
    names = list(mechs)
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        name = names[int(rng.integers(len(names)))]
        sol = mechs[name]
        n = int(np.exp(rng.uniform(np.log(cells[0]), np.log(cells[1] + 1))))
        n = max(cells[0], min(cells[1], n))
        T0 = rng.uniform(900.0, 1800.0, size=n)
        Y0 = np.zeros((sol.n_species, n))
        phi = rng.uniform(fuel_lean[0], fuel_lean[1], size=n)
        idx = sol.species_index
        # H2 + 0.5 O2 with air-like dilution by mass-ish fractions
        x_f, x_o = 2.0 * phi, np.ones(n)
        x_n = 3.76 * x_o
        w = sol.molecular_weights
        m_f = x_f * w[idx("H2")]
        m_o = x_o * w[idx("O2")]
        m_n = x_n * w[idx("N2")]
        tot = m_f + m_o + m_n
        Y0[idx("H2")] = m_f / tot
        Y0[idx("O2")] = m_o / tot
        Y0[idx("N2")] = m_n / tot
        out.append(Request(rid, name, T0, Y0, pressure, t_end, arrival=t))
        rid += 1
    return out
