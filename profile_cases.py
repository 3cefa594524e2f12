"""Small seeded cases of each kernel, for profiler captures.

    python profile_cases.py jacobian [states]
    python profile_cases.py vjp [states]
    python profile_cases.py block_thomas [nv] [systems] [n_min] [n_max]
    python profile_cases.py block_thomas_seg [nv] [systems] [n_min] [n_max] [ctas]
    python profile_cases.py block_thomas_resolve [nv] [systems] [n_min] [n_max]
    python profile_cases.py block_thomas_seg_resolve [nv] [systems] [n_min] [n_max]
    python profile_cases.py batched_lu [nv] [cells]
    python profile_cases.py transport [states]
    python profile_cases.py serving [cells] [launches]
    python profile_cases.py flamelet_solve [copies]
    python profile_cases.py flamelet_blocks [flamelets]
    python profile_cases.py source_dp [states]
    python profile_cases.py peaks [repeats]

Each case builds its inputs on the current CUDA device (inputs larger than
the 129 MB L2 at the default sizes, a few GB at most), runs the kernel three
times and exits 0; a profiler then captures one of those launches
(``-k <kernel> -s 1 -c 1``).  Uses the 53-species / 325-reaction benchmark
mechanism and the block-Thomas benchmark's random diagonally dominant
blocks.
"""

from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np


def _dev():
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("a CUDA device is required")
    return torch.device("cuda")


def jacobian(states: int = 1 << 15, vjp: bool = False):
    import torch

    from pyrometheus_gb300 import get_thermochem_class, synthetic
    dev = _dev()
    sol = synthetic.config2_mechanism()
    th = get_thermochem_class(sol)(device=dev)
    t, p, y = synthetic.sample_states(sol, states, seed=1)
    T = torch.as_tensor(t, device=dev)
    P = torch.as_tensor(p, device=dev)
    Y = torch.as_tensor(y, device=dev)
    if vjp:
        v = torch.randn((sol.n_species + 1, states), dtype=torch.float64,
                        device=dev,
                        generator=torch.Generator(device=dev).manual_seed(1))
        for _ in range(3):
            th.get_reactor_vjp(P, T, Y, v)
    else:
        nc = sol.n_species + 1
        J = torch.empty((states, nc, nc), dtype=torch.float64, device=dev)
        F = torch.empty((nc, states), dtype=torch.float64, device=dev)
        for _ in range(3):
            th.get_reactor_source_and_jacobian(P, T, Y, out=(F, J))
    torch.cuda.synchronize()


def block_thomas(nv: int = 10, systems: int = 304, n_min: int = 64,
                 n_max: int = 1024, ctas: int = 0, kernel=None,
                 resolve=False):
    import torch

    from pyrometheus_gb300.flamelet import BlockThomasSolver
    dev = _dev()
    lengths = np.random.default_rng(0).integers(n_min, n_max + 1,
                                                size=systems)
    rows = int(lengths.sum())
    g = torch.Generator(device=dev).manual_seed(nv)
    f64 = dict(dtype=torch.float64, device=dev)
    C = torch.randn((rows, nv, nv), generator=g, **f64) + \
        10.0 * torch.eye(nv, **f64)
    L = torch.randn((rows, nv, nv), generator=g, **f64)
    U = torch.randn((rows, nv, nv), generator=g, **f64)
    b = torch.randn((rows, nv), generator=g, **f64)
    solver = BlockThomasSolver(nv, lengths, device=dev, kernel=kernel,
                               ctas=ctas)
    for _ in range(3):
        solver.solve(L, C, U, b)
    if resolve:
        B = torch.randn((2, rows, nv), generator=g, **f64)
        for _ in range(3):
            solver.resolve(L, U, B)
    torch.cuda.synchronize()


def batched_lu(nv: int = 54, cells: int = 1 << 16):
    import ctypes

    import torch

    from pyrometheus_gb300 import native
    dev = _dev()
    lib = native.batched_lu_lib()
    g = torch.Generator(device=dev).manual_seed(nv)
    f64 = dict(dtype=torch.float64, device=dev)
    A = torch.randn((cells, nv, nv), generator=g, **f64) + \
        4.0 * torch.eye(nv, **f64)
    M = torch.empty_like(A)
    piv = torch.empty((cells, nv), dtype=torch.int32, device=dev)
    b = torch.randn((nv, cells), generator=g, **f64)
    x = torch.empty_like(b)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(3):
        M.copy_(A)
        if lib.pyro_batched_lu_factor(M.data_ptr(), piv.data_ptr(), None,
                                      cells, nv, st.data_ptr(), s) != 0:
            raise RuntimeError("batched LU factorisation failed")
        if lib.pyro_batched_lu_solve(M.data_ptr(), piv.data_ptr(), None,
                                     b.data_ptr(), 1, cells, x.data_ptr(), 1,
                                     cells, cells, nv, s) != 0:
            raise RuntimeError("batched LU solve failed")
    torch.cuda.synchronize()


def transport(states: int = 1 << 18):
    """Mixture viscosity, conductivity and species diffusivities
    (``k_transport_mixavg``); prints the mean of the timed launches."""
    import torch

    from pyrometheus_gb300 import get_thermochem_class, synthetic
    dev = _dev()
    sol = synthetic.config2_mechanism()
    th = get_thermochem_class(sol)(device=dev)
    t, p, y = synthetic.sample_states(sol, states, seed=1)
    T = torch.as_tensor(t, device=dev)
    P = torch.as_tensor(p, device=dev)
    Y = torch.as_tensor(y, device=dev)
    th.get_transport_mixavg(P, T, Y)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(2):
        th.get_transport_mixavg(P, T, Y)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 2
    print(f"transport: {states} states in {ms:.3f} ms "
          f"({states / ms * 1e3:.4g} states/s)")


def serving(cells: int = 1 << 16, launches: int = 3):
    """The fused reactor integrator (``k_reactor_bdf2``): one request of
    *cells* cells of the 9-species mechanism (T0 ~ U[900, 1800] K, H2/O2/N2
    stoichiometric to lean, 1 ms), *launches* engine steps of up to 64 step
    attempts per cell; prints the time per launch."""
    import torch

    from pyrometheus_gb300 import get_thermochem_class, synthetic
    from pyrometheus_gb300.serving import CudaReactorBackend, ReactorPool, poisson_requests
    dev = _dev()
    sol = synthetic.config1_mechanism()
    th = get_thermochem_class(sol)(device=dev)
    pool = ReactorPool(CudaReactorBackend(th), cells)
    req = poisson_requests(1e4, 1.0, {"s9": sol}, seed=3,
                           cells=(cells, cells))[0]
    pool.admit(req)
    torch.cuda.synchronize()
    import time
    t0 = time.perf_counter()
    for _ in range(launches):
        pool.step()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / launches
    print(f"serving: {cells} cells, {ms:.3f} ms per engine step")


def flamelet_solve(copies: int = 256):
    """The flamelet solver driver (``FlameletSolver.solve`` with the time
    march first, as the reference notebook runs it: 10 Crank-Nicolson steps
    of 1e-5 s, then Newton to |v| < 1e-8) on *copies* copies of three
    seeded flamelets (12, 12 and 9 points; peak dissipation 100, 10 and
    1000 1/s) of the 9-species mechanism with every rate coefficient times
    1e-12; prints the wall time and flamelets solved per second."""
    import time

    import torch

    from pyrometheus_gb300 import get_thermochem_class, synthetic
    from pyrometheus_gb300.flamelet_solver import FlameletSolver
    dev = _dev()
    sol = synthetic.scaled_rates(synthetic.config1_mechanism(), 1e-12)
    th = get_thermochem_class(sol)(device=dev)
    lengths, dxs, ys, ts, chis = [], [], [], [], []
    for n, chi_max, seed in ((12, 100.0, 1), (12, 10.0, 1),
                             (9, 1000.0, 5)):
        prof = synthetic.flamelet_profiles(sol, [n], seed=seed,
                                           chi_max=chi_max)
        chi = prof["chi"].copy()
        chi[0] = chi[-1] = 2.0 * prof["dx"][0] ** 2
        lengths.append(n)
        dxs.append(prof["dx"][0])
        ys.append(prof["Y"])
        ts.append(prof["T"])
        chis.append(chi)
    y_ox, y_fu = prof["y_ox"], prof["y_fu"]
    lengths, dxs = lengths * copies, dxs * copies
    Y = torch.as_tensor(np.hstack(ys * copies), device=dev)
    T = torch.as_tensor(np.concatenate(ts * copies), device=dev)
    chi = torch.as_tensor(np.concatenate(chis * copies), device=dev)
    h = th.get_mixture_enthalpy_mass(T, Y)
    offs = np.concatenate([[0], np.cumsum(lengths)])
    h_ox, h_fu = h[offs[:-1]], h[offs[1:] - 1]
    fs = FlameletSolver(th, lengths, dxs, (y_ox, y_fu))
    args = (False, 20, 1e-8, 20, 1e-9, 1e-5, 10, False, 2, chi,
            torch.zeros_like(chi), T, 101325.0, h_ox, h_fu, (h, Y))
    fs.solve(*args)                         # plans, kernels, first touch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fs.solve(*args)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    stages = np.bincount(fs.last_solve["stage"] + 1, minlength=4)
    print(f"flamelet_solve: {len(lengths)} flamelets ({offs[-1]} points) "
          f"in {wall:.3f} s = {len(lengths) / wall:.1f} flamelets/s; "
          f"flamelets per stage -1/0/1/2: "
          f"{'/'.join(str(int(c)) for c in stages[:4])}")


def flamelet_blocks(flamelets: int = 2048):
    """``FlameletEquations.jac`` (the per-point reactor Jacobians, then
    ``k_flamelet_blocks``) on *flamelets* seeded flamelets of 64..1024
    points of the 9-species mechanism, three times."""
    import torch

    from pyrometheus_gb300 import get_thermochem_class, synthetic
    from pyrometheus_gb300.flamelet import FlameletEquations
    dev = _dev()
    sol = synthetic.config1_mechanism()
    th = get_thermochem_class(sol)(device=dev)
    lengths = np.random.default_rng(11).integers(64, 1025, size=flamelets)
    prof = synthetic.flamelet_profiles(sol, lengths, seed=3)
    eq = FlameletEquations(th, lengths, prof["dx"], prof["y_ox"],
                           prof["y_fu"], device=dev)
    T = torch.as_tensor(prof["T"], device=dev)
    Y = torch.as_tensor(prof["Y"], device=dev)
    chi = torch.as_tensor(prof["chi"], device=dev)
    h = th.get_mixture_enthalpy_mass(T, Y)
    for _ in range(3):
        eq.jac(h, Y, chi, torch.zeros_like(chi), T, 101325.0, temperature=T)
    torch.cuda.synchronize()


def source_dp(states: int = 1 << 18):
    """``get_reactor_source_dp`` on seeded states of the 53-species
    mechanism, three times."""
    import torch

    from pyrometheus_gb300 import get_thermochem_class, synthetic
    dev = _dev()
    sol = synthetic.config2_mechanism()
    th = get_thermochem_class(sol)(device=dev)
    t, p, y = synthetic.sample_states(sol, states, seed=2)
    T = torch.as_tensor(t, device=dev)
    P = torch.as_tensor(p, device=dev)
    Y = torch.as_tensor(y, device=dev)
    for _ in range(3):
        th.get_reactor_source_dp(P, T, Y)
    torch.cuda.synchronize()


def peaks(repeats: int = 5):
    """The FP64 rates the rooflines use, measured live: DFMA FLOP/s, CUDA's
    double exp and log per second, and the FP64 tensor-core rate of
    mma.sync m8n8k4 and m16n8k16 (flops per second), printed as JSON."""
    import json

    import torch

    from pyrometheus_gb300 import native
    dev = _dev()
    scratch = torch.empty(int(native.peaks_scratch_doubles()),
                          dtype=torch.float64, device=dev)
    dfma, exp_rate, log_rate = native.measure_fp64(scratch, repeats)
    dmma_s, dmma_l = native.measure_dmma(scratch, repeats)
    rcp = native.measure_fp64_rcp(scratch, repeats)
    print(json.dumps({"dfma_flops": dfma, "exp_per_s": exp_rate,
                      "log_per_s": log_rate, "rcp_per_s": rcp,
                      "dmma_m8n8k4_flops": dmma_s,
                      "dmma_m16n8k16_flops": dmma_l,
                      "dmma_over_dfma": max(dmma_s, dmma_l) / dfma}))


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    if not argv:
        raise SystemExit(__doc__)
    case, rest = argv[0], [int(a) for a in argv[1:]]
    if case == "jacobian":
        jacobian(*rest)
    elif case == "vjp":
        jacobian(*rest, vjp=True)
    elif case == "block_thomas":
        block_thomas(*rest)
    elif case == "block_thomas_seg":
        block_thomas(*rest, kernel="seg")
    elif case == "block_thomas_resolve":
        block_thomas(*rest, kernel="cta", resolve=True)
    elif case == "block_thomas_seg_resolve":
        block_thomas(*rest, kernel="seg", resolve=True)
    elif case == "batched_lu":
        batched_lu(*rest)
    elif case == "transport":
        transport(*rest)
    elif case == "serving":
        serving(*rest)
    elif case == "flamelet_solve":
        flamelet_solve(*rest)
    elif case == "flamelet_blocks":
        flamelet_blocks(*rest)
    elif case == "source_dp":
        source_dp(*rest)
    elif case == "peaks":
        peaks(*rest)
    else:
        raise SystemExit(f"unknown case {case!r}")
    print("ok")


if __name__ == "__main__":
    main()
