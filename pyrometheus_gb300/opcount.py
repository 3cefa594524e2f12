"""Algorithmic FP64 work per state of the per-state kernels.

The rate kernels are bound by the FP64 pipe (GB300: ~1.2 TFLOP/s of DFMA
against ~7 TB/s of HBM), so their roofline is FP64 arithmetic.  This module
counts, for a mechanism, the FP64 operations the formulation of
``csrc/kinetics.cuh`` performs per state -- ``+ - *`` and comparisons-free
arithmetic as 1 flop, FMA as 2, division as 1 -- and, separately, the
transcendental calls (``exp``, ``log``, ``log10``, ``exp10``, ``pow``).

A transcendental is charged the FP64 flops of the implementation the
kernels use: the table-driven exponential and logarithm (12 and 22 flops
per call, see ``csrc/pyro_math.cuh``) and, for ``pow``, CUDA's libm log at
the FP64-pipe cost the benchmark measures (``DFMA FLOP/s / log/s``).  Then
``algorithmic flops / kernel time / DFMA peak`` is the fraction of the FP64
pipe's FMA throughput doing the algorithm's work (additions and
multiplications count one flop for a full pipe slot, so a perfectly busy
pipe reads below 1 unless the work is all FMAs).
"""

from __future__ import annotations

from collections import Counter
from typing import Dict

TRANSCENDENTALS = ("exp", "log", "log10", "exp10", "pow")


def _tables(sol):
    from .codegen.cuda import _Model
    return _Model(sol)


def _arrhenius(rate, c: Counter):
    if rate.Ta == 0.0 and rate.b == 0.0:
        return
    if rate.Ta == 0.0 and rate.b.is_integer() and abs(rate.b) <= 3:
        c["flops"] += int(abs(rate.b))
        return
    c["flops"] += 4          # two FMAs
    c["exp"] += 1


def _product(terms, c: Counter):
    for _, e in terms:
        if e == 1.0:
            c["flops"] += 1
        elif e == 2.0:
            c["flops"] += 2
        else:
            c["flops"] += 1
            c["pow"] += 1


def production_rates_counts(sol) -> Counter:
    """Per-state counts of the net production rates (given rho, T, Y)."""
    m = _tables(sol)
    S = m.S
    c = Counter()
    c["log"] += 1                 # ln T
    c["flops"] += 1 + 1           # 1/T, c0
    c["flops"] += 3 * S           # c_k = (1/W_k) rho Y_k, total
    c["flops"] += 17 * S          # g_k/RT (Horner with scaled coefficients)
    c["flops"] += 0               # accumulators start at zero
    for r in m.rx:
        if r.kind != "elementary":
            d = r.default_eff
            c["flops"] += 0 if d in (0.0, 1.0) else 1
            c["flops"] += 2 * sum(1 for e in r.eff.values() if e != d)
        if r.kind == "falloff":
            _arrhenius(r.high, c)
            _arrhenius(r.low, c)
            c["flops"] += 2       # Pr
            if r.ftype == "Troe":
                c["flops"] += 2 + 2 + 2   # T*a, products, sum
                c["exp"] += 2
                if len(r.fc) == 4:
                    c["flops"] += 2
                    c["exp"] += 1
                c["log10"] += 2
                c["flops"] += 3 + 4 + 1 + 2 + 1   # x, denominator, f, 1+f^2, /
                c["exp10"] += 1
            c["flops"] += 4       # kf = k_hi (F Pr / (1 + Pr))
        else:
            _arrhenius(r.rate, c)
            if r.kind == "three-body":
                c["flops"] += 1
        _product(r.fwd, c)
        if r.reversible:
            n_terms = len(r.nu_p) + len(r.nu_r)
            c["flops"] += n_terms + sum(1 for v in list(r.nu_p.values())
                                        + list(r.nu_r.values()) if v != 1.0)
            c["flops"] += 2 if r.dnu != 0 else 0
            c["flops"] += 1       # exponent sum or kf * exp(lk)
            c["exp"] += 1
            if r.kind == "three-body":
                c["flops"] += 1
            _product(r.rev, c)
        c["flops"] += 1           # q = rf - rr
        for nu in list(r.nu_r.values()) + list(r.nu_p.values()):
            c["flops"] += 1 if nu == 1.0 else 2
    return c


def temperature_counts(sol, iterations: float) -> Counter:
    """Per-state counts of the temperature Newton with *iterations* mean
    iterations (mass-weighted polynomials folded once per state)."""
    m = _tables(sol)
    S = m.S
    ng = len(m.tmid_groups)
    c = Counter()
    c["flops"] += S * (1 + 1 + 24)      # w_k, sum, 12 FMAs
    per_it = ng * (8 + 10 + 4 + 2) + 2 + 3   # cp, h, scaled q, sums; e-form; dT
    c["flops"] += int(round(per_it * iterations))
    return c


def fused_step_counts(sol, newton_iterations: float) -> Counter:
    """Density + net production rates + temperature Newton per state."""
    m = _tables(sol)
    c = Counter()
    c["flops"] += 2 * m.S + 4           # 1/W_mix and rho
    c.update(production_rates_counts(sol))
    c.update(temperature_counts(sol, newton_iterations))
    return c


def weighted_flops(counts: Dict[str, float], weights: Dict[str, float]
                   ) -> float:
    """``flops + sum_t weight_t * count_t``."""
    total = float(counts.get("flops", 0))
    for t in TRANSCENDENTALS:
        total += weights.get(t, 0.0) * float(counts.get(t, 0))
    return total


def libm_weights(dfma_flops: float, exp_rate: float, log_rate: float
                 ) -> Dict[str, float]:
    """FP64 flops charged per transcendental from measured throughputs."""
    w_exp = dfma_flops / exp_rate
    w_log = dfma_flops / log_rate
    return {"exp": w_exp, "exp10": w_exp, "log": w_log, "log10": w_log,
            "pow": w_exp + w_log}


#: FP64 flops of one call of the table-driven exponential
#: (csrc/pyro_math.cuh): 5 FMAs, one add, one multiply.
TANG_EXP_FLOPS = 12.0

#: FP64 flops of one call of the table-driven logarithm
#: (csrc/pyro_math.cuh): 8 FMAs, three multiplies, three adds (the two
#: int-to-double conversions are not counted).
TANG_LOG_FLOPS = 22.0


def kernel_weights(dfma_flops: float, log_rate: float) -> Dict[str, float]:
    """Flops charged per transcendental as the straight-line kernels
    evaluate them: ``exp``, ``10^x``, ``log`` and ``log10`` by the table
    methods (+1 flop for the ln 10 scalings), ``pow`` by CUDA's libm log
    at its measured FP64-pipe cost plus the table exponential."""
    w_log = dfma_flops / log_rate
    return {"exp": TANG_EXP_FLOPS, "exp10": TANG_EXP_FLOPS + 1.0,
            "log": TANG_LOG_FLOPS, "log10": TANG_LOG_FLOPS + 1.0,
            "pow": w_log + TANG_EXP_FLOPS}


def transport_counts(n_species: int, symmetric: bool = True) -> Counter:
    """Per-state FP64 work of ``k_transport_mixavg`` (``csrc/transport.cuh``)
    computing all three mixture quantities: ``flops`` (FMA = 2) and the
    divisions/reciprocals (``div``, square roots counted with them), plus
    one ``log``.  Pairs are formed once each with symmetric diffusivity
    fits, S^2 times otherwise."""
    S = n_species
    c = Counter()
    c["log"] += 1
    c["div"] += 1                       # sqrt(T)
    c["flops"] += 3                     # powers of ln T
    c["flops"] += 2 * S + 2 * S         # sum Y/W (FMA), x = Y/W * mmw
    c["div"] += 1                       # mmw
    # viscosity: fit, a_k and 1/a_k, x/a, x/a^2; Wilke's three FMAs per
    # pair; per species f_k and x mu / f
    c["flops"] += S * (8 + 1 + 2) + S * S * 6 + S * 10
    c["div"] += 2 * S
    # conductivity
    c["flops"] += S * 12 + 2
    c["div"] += S + 1
    # diffusivities: row j's j off-diagonal pairs in groups of four (one
    # reciprocal and nine products per group, csrc/transport.cuh rcp4)
    # and j mod 4 single reciprocals
    if symmetric:
        off = S * (S - 1) // 2
        groups = sum(j // 4 for j in range(S))
        singles = off - 4 * groups
        c["flops"] += off * (8 + 4) + groups * 9 + S * 10
        c["div"] += groups + singles + S
    else:
        c["flops"] += S * S * 10 + S * 8
        c["div"] += S * S + S
    c["flops"] += 1 + S * 7             # sqrt(T) T, denominators, D_k
    c["div"] += 1 + S
    return c


def transport_weighted_flops(counts: Dict[str, float], dfma_flops: float,
                             rcp_rate: float, log_rate: float) -> float:
    """Flops of :func:`transport_counts` with each division charged its
    measured FP64-pipe cost (``DFMA FLOP/s / reciprocals/s``) and the log
    CUDA's."""
    return (float(counts["flops"])
            + counts["div"] * dfma_flops / rcp_rate
            + counts["log"] * dfma_flops / log_rate)


def bytes_per_state(sol) -> int:
    """HBM bytes per state of the fused step: p, T, Y, e in; wdot, T out."""
    S = sol.n_species
    return 8 * (2 + S + 1) + 8 * (S + 1)


#: Constant per-call weights (flops) of the transcendentals for the
#: implementation-independent algorithmic count: every exp, log, log10 and
#: 10^x is charged 20 flops, pow 40 (a log and an exp), whatever the
#: kernels' own implementations cost, so a faster exp or log does not lower
#: the counted work.
FIXED_WEIGHTS = {"exp": 20.0, "exp10": 20.0, "log": 20.0, "log10": 20.0,
                 "pow": 40.0}


def _rate_derivative_counts(sol, c: Counter):
    """Per-reaction work shared by the Jacobian and the VJP: d ln kf/dT and
    d ln K/dT (2 flops per species slot + 4), dq/dT and dq/d[M] (10), the
    Troe blending's T and Pr derivatives (30 and one log10 per Troe
    reaction) and dq/dc per slot (the product of the other slots and a
    multiply); returns the slot counts per reaction."""
    m = _tables(sol)
    slots = []
    for r in m.rx:
        ns = len(r.nu_r) + len(r.nu_p)
        c["flops"] += 2 * ns + 4 + 10 + ns * (ns + 1)
        if r.kind == "falloff" and r.ftype == "Troe":
            c["flops"] += 30
            c["log10"] += 1
        slots.append((r, ns))
    return slots


def jacobian_counts(sol) -> Counter:
    """Per-state algorithmic work of the analytic reactor Jacobian
    ``d(dT/dt, dY/dt)/d(T, Y)`` as ``k_reactor_jacobian`` forms it: the
    rates of progress (:func:`production_rates_counts`) and their
    derivatives, species thermo with d(cp/R)/dT (40 flops per species), one
    FMA per (element, contribution) of the S x S block of dw/dc (the slot
    pairs of every reaction and its third-body entries), the chain rule
    through c(T, Y) and rho(T, Y) per element (3 flops), the per-species
    sums (10 flops per slot incidence) and the dT/dt row (12 flops per
    column) and column (5 per row)."""
    m = _tables(sol)
    S = m.S
    c = Counter(production_rates_counts(sol))
    entries = 0
    for r, ns in _rate_derivative_counts(sol, c):
        entries += ns * ns
        if r.kind != "elementary":
            entries += ns * sum(1 for e in r.eff.values()
                                if e != r.default_eff)
        c["flops"] += 10 * ns
    c["flops"] += 40 * S + 2 * entries + 3 * S * S + 12 * (S + 1) + 5 * S
    return c


def vjp_counts(sol) -> Counter:
    """Per-state algorithmic work of the reactor VJP ``v^T df/d(T, Y)``
    (``k_reactor_vjp``, reverse accumulation): the rates and their
    derivatives as for :func:`jacobian_counts` without the S x S block,
    plus per slot the adjoint weight and the scatter of ``mu dq/dc`` (8
    flops), per third-body entry one FMA, and per species the thermo and
    closing sums (70 flops)."""
    m = _tables(sol)
    c = Counter(production_rates_counts(sol))
    for r, ns in _rate_derivative_counts(sol, c):
        c["flops"] += 8 * ns
        if r.kind != "elementary":
            c["flops"] += 2 * sum(1 for e in r.eff.values()
                                  if e != r.default_eff) + 2
    c["flops"] += 70 * m.S
    return c
