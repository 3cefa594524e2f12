"""``-l cuda``: the GB300 (sm_103a) code-generation target.

``CudaCodeGenerator.generate(name, sol)`` emits one self-contained CUDA
translation unit for a mechanism.  It plays the role the Mako template of
``pyrometheus/codegen/python.py:106-642`` plays for numpy: the same
per-species/per-reaction formulas (``pyrometheus/chem_expr.py``), written as
FP64 device code with one thread per thermochemical state.

Design (GB300-first):

* the mechanism is baked into straight-line code: NASA-7 coefficients,
  Arrhenius parameters, efficiencies and stoichiometry are compile-time
  constants that the compiler places in the constant bank (operands of the
  FP64 instructions), so no table is fetched per state;
* states are independent: a grid-stride loop assigns one state per thread;
  inputs/outputs are species-major ``[S, N]`` arrays (unit stride along the
  state axis), so a warp's loads and stores are 256-byte coalesced rows;
* per-state working sets (concentrations, Gibbs energies) stay in registers
  for small mechanisms and move to a per-thread slice of shared memory for
  large ones; production-rate accumulators stay in registers;
* the work is FP64-pipe bound (GB300 FP64 is ~1.2 TFLOP/s against
  ~7 TB/s of HBM), so the generated code minimises FP64 instructions:
  ``k_r = exp(ln k_f + ln K)`` reuses the forward exponent, third-body sums
  use the total concentration plus per-species corrections, the temperature
  Newton folds the mass-weighted NASA polynomials into one mixture
  polynomial per range before iterating, and NASA ranges are chosen with
  selects instead of divergent branches.

The emitted C-ABI (``extern "C"``, plain pointers, sizes, strides and a
``cudaStream_t``) is declared in ``include/pyrometheus_gb300.h``.
"""

from __future__ import annotations

import hashlib
import math
import os
import subprocess
import sys
import threading
from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import CodeGenerationOptions, CodeGenerator

file_extension = "cu"

GAS_CONSTANT = 8314.46261815324
ONE_ATM = 101325.0
IRREVERSIBLE_LOG_KEQ_SLOPE = -0.17364695002734

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(
    __file__))), "csrc")


@dataclass(frozen=True)
class CudaGenerationOptions(CodeGenerationOptions):
    """Options of the ``cuda`` target.

    ``block_size``: threads per block of the per-state kernels (``None``:
    as many as let two blocks' per-thread shared-memory columns fit on an
    SM, at most 128);
    ``blocks_per_sm``: grid cap, in blocks per SM, of the grid-stride loops;
    ``unrolled``: emit the straight-line variant of the net-production-rate
    and fused-step kernels (the table-driven kernels serve every other
    method, and the rare states the fast path flags);
    ``accum_in_smem``: keep that variant's production-rate accumulators in
    a shared-memory column instead of registers;
    ``hot_block``: threads per block of the unrolled kernels (``None``: one
    block per SM, as many threads as fit their shared-memory columns beside
    the exp and log tables, at most 256; 224 at 53 species);
    ``fence_every``: in the unrolled kernels, a compiler memory fence (an
    empty ``asm volatile`` with a memory clobber; no instruction) after
    every that many reactions, which keeps the scheduler from hoisting the
    shared-memory loads of later reactions and so bounds register pressure
    (``None``: no fences).  At 53 species ``-Xptxas -v`` reports 2,504
    bytes of spill stores without fences and 148-188 with one every 2 to 16
    reactions; its effect on run time is not yet measured, so it is off.
    """

    block_size: Optional[int] = None
    blocks_per_sm: int = 8
    unrolled: bool = True
    accum_in_smem: bool = False
    hot_block: Optional[int] = None
    fence_every: Optional[int] = None


# {{{ mechanism model

def _hexd(x: float) -> str:
    """Exact C literal for a double."""
    x = float(x)
    if math.isinf(x):
        return "(1.0/0.0)" if x > 0 else "(-1.0/0.0)"
    if x == 0.0:
        return "0.0" if math.copysign(1.0, x) > 0 else "-0.0"
    return float.hex(x)


class _Rate:
    """Arrhenius parameters in the generated form (``chem_expr.py:310-324``)."""

    def __init__(self, rate):
        self.A = float(rate.pre_exponential_factor)
        self.b = float(rate.temperature_exponent)
        self.Ta = float(rate.activation_energy) / GAS_CONSTANT
        self.lnA = float(np.log(np.float64(self.A))) if self.A > 0 else None

    def exp_arg(self) -> Optional[str]:
        """C expression x with k = exp(x), or None if k has a direct form."""
        if self.Ta == 0.0:
            if self.b == 0.0 or (self.b.is_integer() and abs(self.b) <= 3):
                return None
            return f"({_hexd(self.lnA)} + {_hexd(self.b)}*lnT)"
        if self.lnA is None:
            return None
        if self.b == 0.0:
            return f"({_hexd(self.lnA)} - {_hexd(self.Ta)}*invT)"
        return (f"({_hexd(self.lnA)} + {_hexd(self.b)}*lnT"
                f" - {_hexd(self.Ta)}*invT)")

    def direct(self) -> str:
        """C expression of k for the forms without an exponential."""
        if self.Ta == 0.0 and self.b == 0.0:
            return _hexd(self.A)
        if self.Ta == 0.0 and self.b.is_integer() and abs(self.b) <= 3:
            base = "T" if self.b > 0 else "invT"
            return "*".join([_hexd(self.A)] + [base] * int(abs(self.b)))
        if self.lnA is None:
            return "0.0"
        raise AssertionError("rate has an exponential form")

    def expr(self) -> str:
        x = self.exp_arg()
        return f"exp{x}" if x is not None else self.direct()


class _Reaction:
    def __init__(self, j, r, sol, index):
        self.j = j
        self.equation = r.equation
        self.reversible = bool(r.reversible)
        rt = r.reaction_type
        if rt.startswith("falloff"):
            self.kind = "falloff"
            self.ftype = rt.split("-")[1]
            self.low = _Rate(r.rate.low_rate)
            self.high = _Rate(r.rate.high_rate)
            self.fc = [float(v) for v in r.rate.falloff_coeffs]
            if self.ftype not in ("Troe", "Lindemann"):
                raise NotImplementedError(f"falloff type {self.ftype}")
        elif rt == "three-body-Arrhenius":
            self.kind = "three-body"
            self.rate = _Rate(r.rate)
        elif rt in ("Arrhenius", "elementary", "reaction"):
            self.kind = "elementary"
            self.rate = _Rate(r.rate)
        else:
            raise NotImplementedError(f"reaction type '{rt}' ({r.equation})")
        # forward exponents pair reactants with the ``orders`` values
        # positionally, as chem_expr.py:436-446 zips them
        exps = list(r.orders.values()) if r.orders else \
            list(r.reactants.values())
        self.fwd = [(index(sp), float(nu)) for sp, nu in
                    zip(r.reactants, exps)]
        self.rev = [(index(sp), float(nu)) for sp, nu in r.products.items()]
        self.nu_r: Dict[int, float] = {}
        self.nu_p: Dict[int, float] = {}
        for sp in r.reactants:
            self.nu_r[index(sp)] = float(
                sol.reactant_stoich_coeff(index(sp), j))
        for sp in r.products:
            self.nu_p[index(sp)] = float(
                sol.product_stoich_coeff(index(sp), j))
        self.dnu = sum(self.nu_p.values()) - sum(self.nu_r.values())
        self.eff: Dict[int, float] = {}
        self.default_eff = 1.0
        if self.kind != "elementary":
            tb = r.third_body
            self.default_eff = float(tb.default_efficiency)
            for sp, e in tb.efficiencies.items():
                if sp in sol.species_names:
                    self.eff[index(sp)] = float(e)


class _Model:
    def __init__(self, sol):
        self.S = int(sol.n_species)
        self.R = int(sol.n_reactions)
        self.names = list(sol.species_names)
        self.W = [float(w) for w in sol.molecular_weights]
        self.invW = [float(v) for v in 1.0 / np.asarray(
            sol.molecular_weights, dtype=np.float64)]
        self.tmid, self.hi, self.lo = [], [], []
        for sp in sol.species():
            c = [float(v) for v in sp.thermo.coeffs]
            self.tmid.append(c[0])
            self.hi.append(c[1:8])
            self.lo.append(c[8:15])
        index = sol.species_index
        self.rx = [_Reaction(j, r, sol, index)
                   for j, r in enumerate(sol.reactions())]
        groups: Dict[float, List[int]] = {}
        for k, t in enumerate(self.tmid):
            groups.setdefault(t, []).append(k)
        self.tmid_groups = list(groups.items())
        self.n_falloff = sum(1 for r in self.rx if r.kind == "falloff")

# }}}


# {{{ emitter

def _cint(x) -> str:
    return str(int(x))


def _table(qual: str, ctype: str, name: str, dims: List[int],
           values: List[str]) -> str:
    shape = "".join(f"[{d}]" for d in dims)
    return f"{qual} {ctype} {name}{shape} = {{{', '.join(values)}}};"


def _transport_fits(sol) -> Optional[Tuple[np.ndarray, np.ndarray,
                                            np.ndarray]]:
    """``(viscosity (S,5), conductivity (S,5), diffusivity (S,S,5))`` fits
    read through the Cantera surface the reference's template uses
    (``python.py:564-593``), or None for a mechanism without them."""
    S = int(sol.n_species)
    try:
        visc = np.array([sol.get_viscosity_polynomial(k) for k in range(S)],
                        dtype=np.float64)
        cond = np.array([sol.get_thermal_conductivity_polynomial(k)
                         for k in range(S)], dtype=np.float64)
        diff = np.array([[sol.get_binary_diff_coeffs_polynomial(i, j)
                          for j in range(S)] for i in range(S)],
                        dtype=np.float64)
    except (AttributeError, ValueError, RuntimeError, NotImplementedError):
        return None
    if visc.shape != (S, 5) or cond.shape != (S, 5) or \
            diff.shape != (S, S, 5):
        return None
    return visc, cond, diff


def _rate_record(rate: _Rate) -> Tuple[int, List[float]]:
    """(form, [p0, p1, p2]) of an Arrhenius record (kinetics.cuh FORM_*)."""
    if rate.Ta == 0.0 and rate.b == 0.0:
        return 1, [rate.A, 0.0, 0.0]
    if rate.Ta == 0.0 and rate.b.is_integer() and abs(rate.b) <= 3:
        return 2, [rate.A, rate.b, 0.0]
    ln_a = float(np.log(np.float64(rate.A))) if rate.A > 0 else (
        -math.inf if rate.A == 0 else math.nan)
    return 0, [ln_a, rate.b, rate.Ta]


def _dlit(x: float) -> str:
    x = float(x)
    if math.isnan(x):
        return "(double)NAN"
    if math.isinf(x):
        return "(double)INFINITY" if x > 0 else "-(double)INFINITY"
    return _hexd(x)


class _Emitter:
    """Emits the mechanism tables; the kernels are the mechanism-independent
    ``csrc/kinetics.cuh``."""

    CONST_LIMIT = 60 * 1024

    def __init__(self, name: str, sol, opts: CudaGenerationOptions):
        self.name = name
        self.m = _Model(sol)
        self.transport = _transport_fits(sol)
        self.opts = opts
        self.block = int(opts.block_size) if opts.block_size else \
            _default_block(self.m.S)

    def _jacobian_tables(self, perm, flags, rates, dnu, defeff, tb_start,
                         tb_idx, tb_de, fo_slot, fo_form, fo_low,
                         fo_troe) -> List[str]:
        """Tables of the warp-per-state Jacobian kernel (jacobian.cuh).

        The lanes of a warp index these with different reactions or
        species, so they live in global memory (read through L1 with
        ``__ldg``) rather than in constant memory, whose cache serialises
        divergent indices.  Reactions are renumbered in ``perm`` order
        (grouped by kind); every reaction's species occupy consecutive
        "slots" (reactants, then products), and the S x S block of
        dw/dc is built from an update list: entry (output offset, source,
        coefficient) adds coefficient * D[source] into one element, where
        D holds per slot the partial derivative of the rate of progress
        with respect to that slot's concentration and, after the slots, the
        third-body derivative of each reaction.  Entries are sorted by
        output element and split into JGROUP contiguous, equally long runs,
        one per thread of the state's group (a warp, or two warps for large
        mechanisms), so each element is summed by one thread in a fixed order
        and stored once (no atomics, no divergent trip counts); elements
        without contributions are listed separately and zeroed with plain
        stores.  Species -> third-body entries give the column sums the
        assembly needs without reading the block back."""
        m = self.m
        S, R = m.S, m.R
        nc = S + 1
        qual = "__device__"
        slot0, sp, ex, nu, srx, sanu = [0], [], [], [], [], []
        q_nr = []
        for qq, j in enumerate(perm):
            r = m.rx[j]
            q_nr.append(len(r.fwd))
            for (k, e) in r.fwd:
                sp.append(k)
                ex.append(e)
                nu.append(-r.nu_r.get(k, 0.0))
            for (k, v) in r.rev:
                sp.append(k)
                ex.append(v)
                nu.append(v)
            for _ in range(len(r.fwd) + len(r.rev)):
                srx.append(qq)
                sanu.append(nu[len(srx) - 1] * defeff[j]
                            if r.kind != "elementary" else 0.0)
            slot0.append(len(sp))
        nslot = len(sp)
        zero_src = nslot + R
        entries = []
        for qq, j in enumerate(perm):
            r = m.rx[j]
            slots = range(slot0[qq], slot0[qq + 1])
            for b in slots:
                for a in slots:
                    entries.append(((sp[b] + 1) * nc + sp[a] + 1, a, nu[b]))
            if r.kind != "elementary":
                for t in range(tb_start[j], tb_start[j + 1]):
                    for b in slots:
                        entries.append(((sp[b] + 1) * nc + tb_idx[t] + 1,
                                        nslot + qq, nu[b] * tb_de[t]))
        have = {e[0] for e in entries}
        zero_offs = [(k + 1) * nc + mm + 1 for k in range(S)
                     for mm in range(S)
                     if (k + 1) * nc + mm + 1 not in have]
        entries.sort(key=lambda e: e[0])
        groups: List[List[Tuple[int, int, float]]] = []
        for e in entries:
            if groups and groups[-1][0][0] == e[0]:
                groups[-1].append(e)
            else:
                groups.append([e])
        # threads per state: 8 or 16 lanes for small mechanisms (its species
        # and reactions keep few lanes busy, so a warp serves 4 or 2
        # states), two warps where the per-state shared memory would hold
        # an SM to fewer than 24 warps (so twice the warps fit beside the
        # same shared memory), else one
        jw_doubles = 9 * S + 4 * R + nslot + R + 1
        if S <= 12 and R <= 64:
            jgroup = 8
        elif S <= 24 and R <= 128:
            jgroup = 16
        else:
            jgroup = 64 if 8 * jw_doubles > 8192 else 32
        # contiguous split of the groups into jgroup runs of nearly equal
        # length, one per thread of the state's group
        lanes: List[List[Tuple[int, int, float]]] = [[] for _ in
                                                     range(jgroup)]
        total, done, lane = len(entries), 0, 0
        for g in groups:
            if lane < jgroup - 1 and done >= (lane + 1) * total / jgroup:
                lane += 1
            lanes[lane].extend(g)
            done += len(g)
        iters = max(len(x) for x in lanes)
        u_off, u_src, u_coef = [], [], []
        for it in range(iters):
            for ln in range(jgroup):
                if it < len(lanes[ln]):
                    o, s, c = lanes[ln][it]
                else:
                    o, s, c = 0xFFFF, zero_src, 0.0
                u_off.append(o)
                u_src.append(s)
                u_coef.append(c)
        # elements of dw/dc without contributions: plain zero stores
        ziters = max(1, -(-len(zero_offs) // jgroup))
        z_off = [zero_offs[it * jgroup + ln]
                 if it * jgroup + ln < len(zero_offs) else 0xFFFF
                 for it in range(ziters) for ln in range(jgroup)]
        # reaction blocks: the 32 lanes of one warp in one round run
        # reactions of one kind (a falloff round, a three-body round, the
        # elementary rounds), never a mix whose branches the warp would run
        # one after another; blocks go to the warps of a state's group by
        # estimated cost (longest first to the least loaded warp), and
        # jq_lane_rx[round][lane] is the reaction of each lane (-1: none)
        # (with all reactions in one round anyway, a warp that mixes kinds
        # runs each branch once either way, and one round shares the rest)
        cat_cost = {"falloff": 3.0, "three-body": 1.25, "elementary": 1.0}
        blocks: List[List] = []
        for qq, j in enumerate(perm):
            kind = m.rx[j].kind
            if not blocks or blocks[-1][0] != kind or len(blocks[-1][1]) == 32:
                blocks.append([kind, []])
            blocks[-1][1].append(qq)
        nwarp = jgroup // 32
        warp_blocks: List[List[List[int]]] = [[] for _ in range(nwarp)]
        load = [0.0] * nwarp
        for kind, qs in (sorted(blocks, key=lambda b: -cat_cost[b[0]])
                         if nwarp else []):
            wi = min(range(nwarp), key=lambda i: (load[i], i))
            warp_blocks[wi].append(qs)
            load[wi] += cat_cost[kind]
        q_rounds = max(len(x) for x in warp_blocks) if nwarp else 0
        lane_rx = []
        if R <= jgroup or nwarp == 0:
            # one round, or sub-warp groups: consecutive reactions
            q_rounds = -(-R // jgroup)
            lane_rx = list(range(R)) + [-1] * (q_rounds * jgroup - R)
        for rd in range(q_rounds if (R > jgroup and nwarp) else 0):
            for wi in range(nwarp):
                qs = warp_blocks[wi][rd] if rd < len(warp_blocks[wi]) else []
                lane_rx.extend(qs[ln] if ln < len(qs) else -1
                               for ln in range(32))
        # species -> third-body entries (permuted reaction, e - default)
        stinc: List[List[Tuple[int, float]]] = [[] for _ in range(S)]
        for qq, j in enumerate(perm):
            for t in range(tb_start[j], tb_start[j + 1]):
                stinc[tb_idx[t]].append((qq, tb_de[t]))
        st0, st_q, st_de = [0], [], []
        for k in range(S):
            for qq, de in stinc[k]:
                st_q.append(qq)
                st_de.append(de)
            st0.append(len(st_q))
        # third-body efficiency entries, in permuted reaction order
        q_tb0, q_tbidx, q_tbde = [0], [], []
        for j in perm:
            for t in range(tb_start[j], tb_start[j + 1]):
                q_tbidx.append(tb_idx[t])
                q_tbde.append(tb_de[t])
            q_tb0.append(len(q_tbidx))
        # species -> slots
        inc: List[List[int]] = [[] for _ in range(S)]
        for s_, k in enumerate(sp):
            inc[k].append(s_)
        si0, si_slot = [0], []
        for k in range(S):
            si_slot.extend(inc[k])
            si0.append(len(si_slot))
        # per-species sums over a species' slots (five FMAs each) and its
        # third-body entries (one or two), split into parts of nearly equal
        # weight so the group's threads (one part each per round) run
        # balanced loops; a species' first part is its owner, which adds
        # the others' partial sums in order
        wt = [5 * (si0[k + 1] - si0[k]) + 2 * (st0[k + 1] - st0[k])
              for k in range(S)]
        target = max(1, -(-sum(wt) // jgroup))
        while True:
            parts = []
            for k in range(S):
                n_sl = si0[k + 1] - si0[k]
                n_p = max(1, -(-wt[k] // target))
                n_p = min(n_p, max(1, n_sl))
                for pp in range(n_p):
                    a0 = si0[k] + (n_sl * pp) // n_p
                    a1 = si0[k] + (n_sl * (pp + 1)) // n_p
                    last = pp == n_p - 1
                    parts.append((k, pp, a0, a1,
                                  st0[k] if last else 0,
                                  st0[k + 1] if last else 0))
            # one part per thread and round at most, and the others' partial
            # sums must fit the q vector they reuse (5 doubles a part)
            if (len(parts) <= jgroup and 5 * (len(parts) - S) <= R) or \
                    target >= max(wt):
                break
            target += 1
        p_rounds = -(-len(parts) // jgroup)
        # non-owner parts keep their partial sums in scratch slots; the
        # owner lists them
        extra_of: List[List[int]] = [[] for _ in range(S)]
        p_sp, p_s0, p_s1, p_t0, p_t1, p_slot = [], [], [], [], [], []
        nextra = 0
        for (k, pp, a0, a1, t0, t1) in parts:
            p_sp.append(k)
            p_s0.append(a0)
            p_s1.append(a1)
            p_t0.append(t0)
            p_t1.append(t1)
            if pp == 0:
                p_slot.append(-1)
            else:
                p_slot.append(nextra)
                extra_of[k].append(nextra)
                nextra += 1
        pad = p_rounds * jgroup - len(parts)
        p_sp += [-1] * pad
        p_s0 += [0] * pad
        p_s1 += [0] * pad
        p_t0 += [0] * pad
        p_t1 += [0] * pad
        p_slot += [-1] * pad
        px0, px_slot = [0], []
        for k in range(S):
            px_slot.extend(extra_of[k])
            px0.append(len(px_slot))
        if 5 * nextra > R:
            raise NotImplementedError("per-species parts exceed the "
                                      "scratch of the Jacobian kernel")
        nf = max(1, len(fo_low))
        nasa = [[m.tmid[k]] + list(m.hi[k]) + list(m.lo[k]) + [0.0]
                for k in range(S)]
        # states per CTA: as many as fit their shared memory beside the
        # exp table, at most 512 threads
        jgroups = max(1, min(512 // jgroup,
                             (227 * 1024 - 16384) // (8 * jw_doubles)))
        # sub-warp groups fill whole warps (their group sums shuffle across
        # the full warp)
        gpw = max(1, 32 // jgroup)
        if jgroups < gpw:
            raise NotImplementedError("mechanism too large for the "
                                      "Jacobian kernel's sub-warp groups")
        jgroups -= jgroups % gpw

        def arr(ctype, name, dims, vals):
            return _table(qual, ctype, name, dims, vals)

        L: List[str] = []
        w = L.append
        w("// Jacobian kernel tables (global memory; see jacobian.cuh)")
        w(f"#define NSLOT {nslot}")
        w(f"#define JU_ITERS {iters}")
        w(f"#define JZ_ITERS {ziters}")
        w(f"#define JD_ZERO {zero_src}")
        w(f"#define JW_DOUBLES {jw_doubles}")
        w(f"#define JGROUP {jgroup}")
        w(f"#define JGROUPS {jgroups}")
        w(f"#define JQ_ROUNDS {q_rounds}")
        w(f"#define JP_ROUNDS {p_rounds}")
        w(arr("short", "jq_lane_rx", [q_rounds * jgroup],
              [_cint(v) for v in lane_rx]))
        w(arr("short", "jp_sp", [p_rounds * jgroup],
              [_cint(v) for v in p_sp]))
        w(arr("int", "jp_s0", [p_rounds * jgroup], [_cint(v) for v in p_s0]))
        w(arr("int", "jp_s1", [p_rounds * jgroup], [_cint(v) for v in p_s1]))
        w(arr("int", "jp_t0", [p_rounds * jgroup], [_cint(v) for v in p_t0]))
        w(arr("int", "jp_t1", [p_rounds * jgroup], [_cint(v) for v in p_t1]))
        w(arr("short", "jp_slot", [p_rounds * jgroup],
              [_cint(v) for v in p_slot]))
        w(arr("int", "jp_x0", [S + 1], [_cint(v) for v in px0]))
        w(arr("short", "jp_xslot", [max(1, len(px_slot))],
              [_cint(v) for v in (px_slot or [0])]))
        w(arr("int", "jq_flags", [R], [_cint(flags[j]) for j in perm]))
        w(arr("int", "jq_slot0", [R + 1], [_cint(v) for v in slot0]))
        w(arr("int", "jq_nr", [R], [_cint(v) for v in q_nr]))
        w(arr("double", "jq_rate", [3, R],
              ["{" + ", ".join(_dlit(rates[j][p]) for j in perm) + "}"
               for p in range(3)]))
        w(arr("double", "jq_dnu", [R], [_hexd(dnu[j]) for j in perm]))
        w(arr("double", "jq_defeff", [R], [_hexd(defeff[j]) for j in perm]))
        w(arr("int", "jq_tb0", [R + 1], [_cint(v) for v in q_tb0]))
        w(arr("int", "jq_tbidx", [max(1, len(q_tbidx))],
              [_cint(v) for v in (q_tbidx or [0])]))
        w(arr("double", "jq_tbde", [max(1, len(q_tbde))],
              [_hexd(v) for v in (q_tbde or [0.0])]))
        w(arr("int", "jq_fo", [R], [_cint(fo_slot[j]) for j in perm]))
        w(arr("int", "jf_lowform", [nf], [_cint(v) for v in
                                          (fo_form or [0])]))
        w(arr("double", "jf_low", [3, nf],
              ["{" + ", ".join(_dlit(rec[p]) for rec in
                               (fo_low or [[0.0] * 3])) + "}"
               for p in range(3)]))
        w(arr("double", "jf_troe", [5, nf],
              ["{" + ", ".join(_dlit(rec[p]) for rec in
                               (fo_troe or [[0.0] * 5])) + "}"
               for p in range(5)]))
        w(arr("int", "jq_sp", [nslot], [_cint(v) for v in sp]))
        w(arr("double", "jq_e", [nslot], [_hexd(v) for v in ex]))
        w(arr("double", "jq_nu", [nslot], [_hexd(v) for v in nu]))
        w(arr("int", "jq_slot_rx", [nslot], [_cint(v) for v in srx]))
        w(arr("double", "jq_slot_anu", [nslot], [_hexd(v) for v in sanu]))
        w(arr("int", "jg_si0", [S + 1], [_cint(v) for v in si0]))
        w(arr("int", "jg_si_slot", [nslot], [_cint(v) for v in si_slot]))
        w(arr("double", "jg_nasa", [S, 16],
              ["{" + ", ".join(_hexd(v) for v in row) + "}"
               for row in nasa]))
        w(arr("double", "jg_mw", [S], [_hexd(v) for v in m.W]))
        w(arr("double", "jg_invmw", [S], [_hexd(v) for v in m.invW]))
        w(arr("int", "jg_st0", [S + 1], [_cint(v) for v in st0]))
        w(arr("int", "jg_st_q", [max(1, len(st_q))],
              [_cint(v) for v in (st_q or [0])]))
        w(arr("double", "jg_st_de", [max(1, len(st_de))],
              [_hexd(v) for v in (st_de or [0.0])]))
        w(arr("unsigned short", "jz_off", [jgroup * ziters],
              [_cint(v) for v in z_off]))
        w(arr("unsigned short", "ju_off", [jgroup * iters],
              [_cint(v) for v in u_off]))
        w(arr("unsigned short", "ju_src", [jgroup * iters],
              [_cint(v) for v in u_src]))
        w(arr("double", "ju_coef", [jgroup * iters],
              [_hexd(v) for v in u_coef]))
        if zero_src > 0xFFFE or (S + 1) * nc > 0xFFFE:
            raise NotImplementedError("mechanism too large for the "
                                      "Jacobian update list")
        return L

    def render(self) -> str:
        m = self.m
        S, R = m.S, m.R
        maxside = max([1] + [max(len(r.fwd), len(r.rev)) for r in m.rx])
        falloff = [r for r in m.rx if r.kind == "falloff"]
        nf = len(falloff)

        flags, rates, nr_l, np_l, sp_l, nu_l, ord_l = [], [], [], [], [], [], []
        dnu, defeff, tb_start, tb_idx, tb_de = [], [], [0], [], []
        fo_slot, fo_form, fo_low, fo_troe = [], [], [], []
        frac_row, frac = [], []
        for r in m.rx:
            f = 0
            if r.kind == "three-body":
                f |= 1
            elif r.kind == "falloff":
                f |= 2
            if r.reversible:
                f |= 4
            rate = r.high if r.kind == "falloff" else r.rate
            form, rec = _rate_record(rate)
            f |= form << 3
            rates.append(rec)
            if r.kind == "falloff":
                fo_slot.append(len(fo_low))
                lform, lrec = _rate_record(r.low)
                fo_form.append(lform)
                fo_low.append(lrec)
                if r.ftype == "Troe":
                    f |= 32
                    a, t3, t1 = r.fc[0], r.fc[1], r.fc[2]
                    t2 = r.fc[3] if len(r.fc) == 4 else 0.0
                    if len(r.fc) == 4:
                        f |= 64
                    fo_troe.append([1.0 - a, -1.0 / t3, a, -1.0 / t1, -t2])
                else:
                    fo_troe.append([0.0] * 5)
            else:
                fo_slot.append(-1)
            r_sp = [k for k, _ in r.fwd]
            r_ord = [e for _, e in r.fwd]
            r_nu = [r.nu_r.get(k, 0.0) for k in r_sp]
            p_sp = [k for k, _ in r.rev]
            p_nu = [nu for _, nu in r.rev]
            ints = all(float(v).is_integer() and abs(v) <= 127
                       for v in r_nu + p_nu + r_ord)
            if not ints:
                f |= 128
                frac_row.append(len(frac))
                row = ([float(v) for v in r_nu] + [0.0] * (maxside - len(r_nu))
                       + [float(v) for v in p_nu]
                       + [0.0] * (maxside - len(p_nu))
                       + [float(v) for v in r_ord]
                       + [0.0] * (maxside - len(r_ord)))
                frac.append(row)
            else:
                frac_row.append(0)
            flags.append(f)
            nr_l.append(len(r_sp))
            np_l.append(len(p_sp))
            sp_l.append(r_sp + [0] * (maxside - len(r_sp)) + p_sp
                        + [0] * (maxside - len(p_sp)))
            nu_l.append([int(v) if float(v).is_integer() and abs(v) <= 127
                         else 0 for v in r_nu]
                        + [0] * (maxside - len(r_nu))
                        + [int(v) if float(v).is_integer() and abs(v) <= 127
                           else 0 for v in p_nu]
                        + [0] * (maxside - len(p_nu)))
            ord_l.append([int(v) if float(v).is_integer() and abs(v) <= 127
                          else 0 for v in r_ord]
                         + [0] * (maxside - len(r_ord)))
            dnu.append(r.dnu)
            d = r.default_eff if r.kind != "elementary" else 1.0
            defeff.append(d)
            if r.kind != "elementary":
                for k, e in sorted(r.eff.items()):
                    if e != d:
                        tb_idx.append(k)
                        tb_de.append(e - d)
            tb_start.append(len(tb_idx))

        # species -> (reaction, slot) incidences and species -> third-body
        # entries, for the Jacobian / VJP kernels (csrc/jacobian.cuh)
        inc: List[List[Tuple[int, int]]] = [[] for _ in range(S)]
        for j, row in enumerate(sp_l):
            for a in range(nr_l[j]):
                inc[row[a]].append((j, a))
            for a in range(np_l[j]):
                inc[row[maxside + a]].append((j, maxside + a))
        si_start, si_rx, si_pos = [0], [], []
        for k in range(S):
            for j, a in inc[k]:
                si_rx.append(j)
                si_pos.append(a)
            si_start.append(len(si_rx))
        tbinc: List[List[Tuple[int, float]]] = [[] for _ in range(S)]
        for j in range(R):
            for t in range(tb_start[j], tb_start[j + 1]):
                tbinc[tb_idx[t]].append((j, tb_de[t]))
        st_start, st_rx, st_de = [0], [], []
        for k in range(S):
            for j, de in tbinc[k]:
                st_rx.append(j)
                st_de.append(de)
            st_start.append(len(st_rx))

        groups = m.tmid_groups
        grp_start, grp_sp, grp_tmid = [0], [], []
        for tmid, ks in groups:
            grp_sp.extend(ks)
            grp_start.append(len(grp_sp))
            grp_tmid.append(tmid)

        # table footprint decides constant vs global placement
        nbytes = (8 * S * 17 + 4 * (len(groups) + 1) + 2 * S
                  + 8 * len(groups) + R * (4 + 24 + 2 + 2 * 2 * maxside
                                           + 3 * maxside + 16 + 4 + 4 + 4)
                  + 4 * (R + 1) + max(1, len(tb_idx)) * 10
                  + max(1, nf) * (4 + 24 + 40)
                  + max(1, len(frac)) * 24 * maxside
                  + 8 * (S + 1) + 3 * len(si_rx) + 10 * len(st_rx) + 16)
        qual = "__constant__" if nbytes <= self.CONST_LIMIT else "__device__"

        L: List[str] = []
        w = L.append
        w(f"// Generated by pyrometheus_gb300 (-l cuda) for mechanism "
          f"'{self.name}':")
        w(f"// {S} species, {R} reactions ({nf} falloff); FP64, sm_103a.")
        w("// Tables only: the kernels are csrc/kinetics.cuh, the C ABI "
          "csrc/kinetics_abi.cuh.")
        w("#include <cmath>")
        w('#include "pyro_common.cuh"')
        w("")
        w(f"#define NS {S}")
        w(f"#define NR {R}")
        w(f"#define NF {max(1, nf)}")
        w(f"#define NF_REAL {nf}")
        w(f"#define NTB {max(1, len(tb_idx))}")
        w(f"#define NFRAC {max(1, len(frac))}")
        w(f"#define NG {len(groups)}")
        w(f"#define MAXSIDE {maxside}")
        w(f"#define BLOCK {self.block}")
        w(f"#define BLOCKS_PER_SM {int(self.opts.blocks_per_sm)}")
        w(f"#define TABLE_BYTES {nbytes}")
        w(f"#define LOG_P0_OVER_R {_hexd(math.log(ONE_ATM / GAS_CONSTANT))}")
        w("")
        w("// species: molecular weights, NASA-7 ranges [Tmid, hi(7), lo(7)]")
        w(_table(qual, "double", "k_mw", [S], [_hexd(v) for v in m.W]))
        w(_table(qual, "double", "k_inv_mw", [S], [_hexd(v) for v in m.invW]))
        w(_table(qual, "double", "k_tmid", [S], [_hexd(v) for v in m.tmid]))
        w(_table(qual, "double", "k_nasa_hi", [S, 7],
                 ["{" + ", ".join(_hexd(v) for v in row) + "}"
                  for row in m.hi]))
        w(_table(qual, "double", "k_nasa_lo", [S, 7],
                 ["{" + ", ".join(_hexd(v) for v in row) + "}"
                  for row in m.lo]))
        w(_table(qual, "int", "k_grp_start", [len(groups) + 1],
                 [_cint(v) for v in grp_start]))
        w(_table(qual, "short", "k_grp_sp", [S], [_cint(v) for v in grp_sp]))
        w(_table(qual, "double", "k_grp_tmid", [len(groups)],
                 [_hexd(v) for v in grp_tmid]))
        w("")
        w("// reactions (flags: kind | reversible | Arrhenius form | Troe...)")
        w(_table(qual, "int", "k_rx_flags", [R], [_cint(v) for v in flags]))
        w(_table(qual, "double", "k_rx_rate", [R, 3],
                 ["{" + ", ".join(_dlit(v) for v in rec) + "}"
                  for rec in rates]))
        w(_table(qual, "signed char", "k_rx_nr", [R], [_cint(v) for v in nr_l]))
        w(_table(qual, "signed char", "k_rx_np", [R], [_cint(v) for v in np_l]))
        w(_table(qual, "short", "k_rx_sp", [R, 2 * maxside],
                 ["{" + ", ".join(_cint(v) for v in row) + "}"
                  for row in sp_l]))
        w(_table(qual, "signed char", "k_rx_nu", [R, 2 * maxside],
                 ["{" + ", ".join(_cint(v) for v in row) + "}"
                  for row in nu_l]))
        w(_table(qual, "signed char", "k_rx_ord", [R, maxside],
                 ["{" + ", ".join(_cint(v) for v in row) + "}"
                  for row in ord_l]))
        w(_table(qual, "double", "k_rx_dnu", [R], [_hexd(v) for v in dnu]))
        w(_table(qual, "double", "k_rx_defeff", [R],
                 [_hexd(v) for v in defeff]))
        w(_table(qual, "int", "k_rx_tb", [R + 1],
                 [_cint(v) for v in tb_start]))
        w(_table(qual, "short", "k_tb_idx", [max(1, len(tb_idx))],
                 [_cint(v) for v in (tb_idx or [0])]))
        w(_table(qual, "double", "k_tb_de", [max(1, len(tb_de))],
                 [_hexd(v) for v in (tb_de or [0.0])]))
        w(_table(qual, "int", "k_rx_fo", [R], [_cint(v) for v in fo_slot]))
        w(_table(qual, "int", "k_fo_lowform", [max(1, nf)],
                 [_cint(v) for v in (fo_form or [0])]))
        w(_table(qual, "double", "k_fo_low", [max(1, nf), 3],
                 ["{" + ", ".join(_dlit(v) for v in rec) + "}"
                  for rec in (fo_low or [[0.0, 0.0, 0.0]])]))
        w(_table(qual, "double", "k_fo_troe", [max(1, nf), 5],
                 ["{" + ", ".join(_dlit(v) for v in rec) + "}"
                  for rec in (fo_troe or [[0.0] * 5])]))
        w(_table(qual, "int", "k_rx_frac", [R], [_cint(v) for v in frac_row]))
        w(_table(qual, "double", "k_frac", [max(1, len(frac)), 3 * maxside],
                 ["{" + ", ".join(_dlit(v) for v in row) + "}"
                  for row in (frac or [[0.0] * (3 * maxside)])]))
        w("// species -> reaction slots; species -> third-body entries")
        w(_table(qual, "int", "k_si_start", [S + 1],
                 [_cint(v) for v in si_start]))
        w(_table(qual, "short", "k_si_rx", [max(1, len(si_rx))],
                 [_cint(v) for v in (si_rx or [0])]))
        w(_table(qual, "signed char", "k_si_pos", [max(1, len(si_pos))],
                 [_cint(v) for v in (si_pos or [0])]))
        w(_table(qual, "int", "k_st_start", [S + 1],
                 [_cint(v) for v in st_start]))
        w(_table(qual, "short", "k_st_rx", [max(1, len(st_rx))],
                 [_cint(v) for v in (st_rx or [0])]))
        w(_table(qual, "double", "k_st_de", [max(1, len(st_de))],
                 [_hexd(v) for v in (st_de or [0.0])]))
        # reactions ordered for the Jacobian kernel's lane blocks: by kind,
        # then reversibility, side sizes and rate form, so the reactions a
        # warp runs side by side take the same branches and trip counts
        def kind_key(j):
            r = m.rx[j]
            rank = {"elementary": 0, "three-body": 1, "falloff": 2}[r.kind]
            troe = 1 if r.kind == "falloff" and r.ftype == "Troe" else 0
            return (rank, troe, int(r.reversible), len(r.fwd), len(r.rev),
                    flags[j] >> 3 & 3, j)
        perm = sorted(range(R), key=kind_key)
        w(_table(qual, "short", "k_rx_perm", [R], [_cint(v) for v in perm]))
        L.extend(self._jacobian_tables(perm, flags, rates, dnu, defeff,
                                       tb_start, tb_idx, tb_de, fo_slot,
                                       fo_form, fo_low, fo_troe))
        # VJP: five per-thread columns; as many threads per CTA as fit
        # beside the exp table (one CTA per SM at 53 species: 96 threads,
        # three warps, where 32-thread CTAs left two warps per SM)
        vblock = max(32, min(128, ((227 * 1024 - 17408) // (5 * S * 8))
                             // 32 * 32))
        w(f"#define VBLOCK {vblock}")
        # pressure derivative of the source: four per-thread columns
        dpblock = max(32, min(128, ((227 * 1024 - 17408) // (4 * S * 8))
                              // 32 * 32))
        w(f"#define DPBLOCK {dpblock}")
        w("")
        w('#include "kinetics.cuh"')
        w('#include "jacobian.cuh"')
        if self.opts.unrolled:
            L.extend(_UnrolledEmitter(m, self.opts.accum_in_smem,
                                      self.opts.hot_block,
                                      self.opts.fence_every).render())
        w('#include "kinetics_abi.cuh"')
        # fused per-cell reactor integrator: threads per CTA so that seven
        # per-thread columns (3 NS + 4 (NS + 1) doubles) fit beside the exp
        # and log tables (19,480 bytes) in 227 KB of shared memory
        per_thread = (3 * S + 4 * (S + 1)) * 8
        iblock = max(32, min(128, ((227 * 1024 - 19480) // per_thread)
                             // 32 * 32))
        w(f"#define IBLOCK {iblock}")
        if self.opts.unrolled and S <= 16:
            w("#define PYRO_BDF2_UNROLLED 1")
        w('#include "reactor_bdf2.cuh"')
        w('#include "flamelet.cuh"')
        L.extend(self._transport_tables())
        w('#include "transport.cuh"')
        return "\n".join(L) + "\n"

    def _transport_tables(self) -> List[str]:
        """Fits and mixture-rule constants of ``csrc/transport.cuh`` (none
        when the mechanism carries no transport fits).  Threads read them
        with uniform indices, through L1 (``__ldg``)."""
        if self.transport is None:
            return ["// no transport fits: the transport entry points "
                    "return PYRO_ERR_UNSUPPORTED"]
        visc, cond, diff = self.transport
        m = self.m
        S = m.S
        W = np.asarray(m.W, dtype=np.float64)
        sym = bool(np.array_equal(diff, diff.transpose(1, 0, 2)))
        if sym:
            pairs = [diff[i, j] for j in range(S) for i in range(j + 1)]
        else:
            pairs = [diff[i, j] for i in range(S) for j in range(S)]
        # Wilke: C_kj = 1 / sqrt(8 (1 + W_k/W_j)), a_k = |P_k| W_k^(-1/4)
        wilke = [1.0 / np.sqrt(8.0 * (1.0 + W[k] / W[j]))
                 for k in range(S) for j in range(S)]
        wq = [float(v) for v in W ** -0.25]
        # three per-thread columns of S doubles in the mixture kernel
        per_thread = 3 * S * 8
        tblock = max(32, min(256, (227 * 1024 - 1024) // per_thread
                             // 32 * 32))
        per_cta = per_thread * tblock + 1024
        tbps = max(1, min(8, (228 * 1024) // per_cta))

        def flat(a):
            return [_hexd(v) for r in a for v in r]
        out = [
            "// mixture-averaged transport fits (chem_expr.py:190-244), five"
            " coefficients per fit",
            "#define PYRO_HAS_TRANSPORT 1",
            f"#define PYRO_TR_SYM {1 if sym else 0}",
            f"#define TBLOCK {tblock}",
            f"#define TBLOCKS_PER_SM {tbps}",
            _table("__device__ const", "double", "k_tr_visc", [S * 5],
                   flat(visc)),
            _table("__device__ const", "double", "k_tr_cond", [S * 5],
                   flat(cond)),
            _table("__device__ const", "double", "k_tr_diff",
                   [len(pairs) * 5], flat(pairs)),
            _table("__device__ const", "double", "k_tr_wilke", [S * S],
                   [_hexd(v) for v in wilke]),
            _table("__device__ const", "double", "k_tr_wq", [S],
                   [_hexd(v) for v in wq]),
        ]
        return out


class _UnrolledEmitter:
    """Straight-line variant of the net-production-rate kernels.

    Every reaction becomes its own block of FP64 code with compile-time
    species offsets: the scheduler interleaves independent reactions (ILP
    across reactions), rate accumulators live in registers, and only the
    concentrations and Gibbs energies stay in shared memory (two columns
    instead of three, so more warps fit per SM).  Exponentials are
    branch-free (the table method on a sanitised argument); a state with an
    exponent outside |x| < 708 raises a flag and is recomputed exactly by
    the table-driven path on thread-private arrays.
    """

    def __init__(self, m: _Model, accum_in_smem: bool = False,
                 hot_block: Optional[int] = None,
                 fence_every: Optional[int] = None):
        self.m = m
        self.acc_smem = accum_in_smem
        if fence_every is not None and int(fence_every) < 1:
            raise ValueError("fence_every must be a positive reaction count")
        self.fence_every = int(fence_every) if fence_every else 0
        self.hot_block = int(hot_block) if hot_block else \
            _default_hot_block(m.S, 3 if accum_in_smem else 2)
        self.L: List[str] = []

    def W(self, k):
        return f"w[{k}]" if self.acc_smem else f"wd[{k}]"

    def w(self, s):
        self.L.append(s)

    @staticmethod
    def C(k):
        return f"c[{k}]"

    @staticmethod
    def G(k):
        return f"g[{k}]"

    def rate_expr(self, rate: _Rate, tag: str) -> Tuple[Optional[str], str]:
        """(exponent variable or None, statement defining e_<tag>)."""
        form, rec = _rate_record(rate)
        if form == 1:
            return None, f"const double e_{tag} = {_dlit(rec[0])};"
        if form == 2:
            b = int(rec[1])
            base = "T" if b > 0 else "invT"
            ex = "*".join([_dlit(rec[0])] + [base] * abs(b))
            return None, f"const double e_{tag} = {ex};"
        ln_a, b, ta = rec
        if b == 0.0:
            x = f"fma({_dlit(-ta)}, invT, {_dlit(ln_a)})"
        elif ta == 0.0:
            x = f"fma({_dlit(b)}, lnT, {_dlit(ln_a)})"
        else:
            x = (f"fma({_dlit(b)}, lnT, fma({_dlit(-ta)}, invT, "
                 f"{_dlit(ln_a)}))")
        return (f"x_{tag}", f"const double x_{tag} = {x}; "
                f"const double e_{tag} = fx(x_{tag}, bad);")

    def third_body(self, r: _Reaction) -> str:
        d = r.default_eff
        terms = []
        if d != 0.0:
            terms.append("ctot" if d == 1.0 else f"{_hexd(d)} * ctot")
        for k, e in sorted(r.eff.items()):
            if e != d:
                terms.append(f"{_hexd(e - d)} * {self.C(k)}")
        return " + ".join(terms) if terms else "0.0"

    def prod(self, terms) -> str:
        parts = []
        for k, nu in terms:
            c = self.C(k)
            if nu == 1.0:
                parts.append(c)
            elif nu == 2.0:
                parts.append(f"{c} * {c}")
            else:
                parts.append(f"pow({c}, {_hexd(nu)})")
        return " * ".join(parts) if parts else "1.0"

    def log_keq(self, r: _Reaction) -> str:
        def side(d):
            parts = [self.G(k) if nu == 1.0 else f"{_hexd(nu)} * {self.G(k)}"
                     for k, nu in d.items()]
            return "(" + " + ".join(parts) + ")" if parts else "0.0"
        e = f"{side(r.nu_p)} - {side(r.nu_r)}"
        if r.dnu != 0:
            e = f"fma({_hexd(-r.dnu)}, c0, {e})"
        return e

    def troe_term(self, coef: float, scale: str, fac: float) -> Optional[str]:
        """fac * exp(coef * scale) with the exponent's range known from
        T in [200, 5000] K: folded to 0 or fac when it under-/overflows
        the double range or rounds to exp(0)."""
        if fac == 0.0:
            return None
        if scale == "T":
            lo, hi = sorted((coef * 200.0, coef * 5000.0))
        else:  # invT
            lo, hi = sorted((coef / 200.0, coef / 5000.0))
        if hi < -745.2:
            return None
        if max(abs(lo), abs(hi)) < 1e-17:
            return _hexd(fac)
        return f"{_hexd(fac)} * fx({_hexd(coef)} * {scale}, bad)"

    def reaction(self, r: _Reaction):
        w = self.w
        w(f"  {{  // R{r.j}: {r.equation}")
        if r.kind != "elementary":
            w(f"    const double m = {self.third_body(r)};")
        xf = None
        if r.kind == "falloff":
            xh, sh = self.rate_expr(r.high, "hi")
            xl, sl = self.rate_expr(r.low, "lo")
            w(f"    {sh}")
            w(f"    {sl}")
            w("    const double pr = m * e_lo / e_hi;")
            if r.ftype == "Troe":
                a, t3, t1 = r.fc[0], r.fc[1], r.fc[2]
                terms = [self.troe_term(-1.0 / t3, "T", 1.0 - a),
                         self.troe_term(-1.0 / t1, "T", a)]
                if len(r.fc) == 4:
                    terms.append(self.troe_term(-r.fc[3], "invT", 1.0))
                terms = [t for t in terms if t is not None] or ["0.0"]
                w(f"    const double log_fc = pyro_log10({' + '.join(terms)});")
                w("    double fac = -1.0 / 0.14;")
                w("    if (pr > 0.0) {")
                w("      const double xx = pyro_log10(pr) + (-0.4 - 0.67 * "
                  "log_fc);")
                w("      fac = xx / ((0.75 - 1.27 * log_fc) - 0.14 * xx);")
                w("    }")
                w("    const double blend = fx(log_fc / (1.0 + fac * fac) * "
                  "2.302585092994045684, bad);")
            else:
                w("    const double blend = 1.0;")
            w("    const double kf = e_hi * (blend * pr / (1.0 + pr));")
        else:
            xf, sf = self.rate_expr(r.rate, "f")
            w(f"    {sf}")
            w("    const double kf = " + ("e_f * m" if r.kind == "three-body"
                                          else "e_f") + ";")
        if r.reversible:
            w(f"    const double lk = {self.log_keq(r)};")
            if xf is not None:
                w("    const double kr = fx(x_f + lk, bad)" +
                  (" * m" if r.kind == "three-body" else "") + ";")
            else:
                w("    const double kr = kf * fx(lk, bad);")
            w(f"    const double q = kf * {self.prod(r.fwd)} - kr * "
              f"{self.prod(r.rev)};")
        else:
            w(f"    const double q = kf * {self.prod(r.fwd)};")
        net: Dict[int, float] = {}
        for k, nu in r.nu_p.items():
            net[k] = net.get(k, 0.0) + nu
        for k, nu in r.nu_r.items():
            net[k] = net.get(k, 0.0) - nu
        for k, nu in sorted(net.items()):
            acc = self.W(k)
            if nu == 1.0:
                w(f"    {acc} += q;")
            elif nu == -1.0:
                w(f"    {acc} -= q;")
            elif nu != 0.0:
                w(f"    {acc} = fma({_hexd(nu)}, q, {acc});")
        w("  }")

    def render(self) -> List[str]:
        m = self.m
        w = self.w
        w("")
        w("// ---- unrolled hot path (generated) ----")
        w("#define PYRO_UNROLLED 1")
        w(f"#define PYRO_HOT_COLS {3 if self.acc_smem else 2}")
        w(f"#define HOT_BLOCK {self.hot_block}")
        w("namespace pyro_unrolled {")
        w("")
        w("// exp on a sanitised argument: out-of-range lanes set *bad* and")
        w("// are recomputed exactly afterwards")
        w("__device__ __forceinline__ double fx(double x, bool& bad) {")
        w("  const bool out = (__double2hiint(x) & 0x7fffffff) >= 0x40862000;")
        w("  bad |= out;")
        w("  return pyro_exp_core(out ? 0.0 : x);")
        w("}")
        w("")
        w("using HCols = pyro::ColsT<HOT_BLOCK>;")
        w("// mass fractions of state i in a species-major global array")
        w("struct GlobalY {")
        w("  const double* __restrict__ Y;")
        w("  int64_t ldy, i;")
        w("  __device__ __forceinline__ double operator()(int k) const {")
        w("    return __ldg(Y + (int64_t)k * ldy + i);")
        w("  }")
        w("};")
        w("// net production rates into wd (registers) or w (columns); Y is")
        w("// any accessor k -> Y_k, CT a per-thread column type")
        w("template <class YA, class CT>")
        w("__device__ __forceinline__ void net_rates_y(double T, double rho, "
          "const YA& Y, CT c, CT g, CT w, double (&wd)[NS]) {")
        w("  const double lnT = pyro_log(T);")
        w("  const double invT = 1.0 / T;")
        w("  const double c0 = LOG_P0_OVER_R - lnT;")
        w("  double ctot = 0.0;")
        for k in range(m.S):
            w(f"  {{ const double v = {_hexd(m.invW[k])} * rho * "
              f"Y({k}); c[{k}] = v; ctot += v; }}")
        w("  pyro::gibbs_all(T, lnT, invT, g);")
        for k in range(m.S):
            w(f"  {self.W(k)} = 0.0;")
        w("  bool bad = false;")
        for j, r in enumerate(m.rx):
            self.reaction(r)
            if self.fence_every and (j + 1) % self.fence_every == 0 \
                    and j + 1 < len(m.rx):
                w('  asm volatile("" ::: "memory");')
        w("  if (bad) {  // exact recompute through the table-driven path")
        w("    double lc[NS], lg[NS], lw[NS];")
        w("    const pyro::LocalCols C{lc}, G{lg}, W{lw};")
        w("    pyro::StateScalars s;")
        w("    s.T = T;")
        w("    s.lnT = log(T);")
        w("    s.invT = 1.0 / T;")
        w("    s.c0 = LOG_P0_OVER_R - s.lnT;")
        w("    double ct = 0.0;")
        w("    for (int k = 0; k < NS; ++k) {")
        w("      const double v = k_inv_mw[k] * rho * Y(k);")
        w("      lc[k] = v;")
        w("      ct += v;")
        w("    }")
        w("    s.ctot = ct;")
        w("    pyro::production_rates(s, C, G, W);")
        w("#pragma unroll")
        w("    for (int k = 0; k < NS; ++k) " +
          ("w[k] = lw[k];" if self.acc_smem else "wd[k] = lw[k];"))
        w("  }")
        if self.acc_smem:
            w("#pragma unroll")
            w("  for (int k = 0; k < NS; ++k) wd[k] = w[k];")
        w("}")
        w("")
        w("__device__ __forceinline__ void net_rates(double T, double rho, "
          "const double* __restrict__ Y, int64_t ldy, int64_t i, "
          "HCols c, HCols g, HCols w, double (&wd)[NS]) {")
        w("  net_rates_y(T, rho, GlobalY{Y, ldy, i}, c, g, w, wd);")
        w("}")
        w("")
        w("}  // namespace pyro_unrolled")
        return self.L


def _default_hot_block(n_species: int, cols: int) -> int:
    """Threads per block of the unrolled hot kernels: one block per SM, as
    many threads as let their shared-memory columns fit beside the exp and
    log tables (19,480 bytes) in 227 KB, 32..256.  Measured on GB300 at 53
    species: 224 threads 107.5 ms, 192 108.7, 160 114.5, 128 119.3 for
    4,194,304 states (more warps hide more FP64 latency than the L1 they
    take from the register spills costs)."""
    per_thread = cols * n_species * 8
    b = ((227 * 1024 - 19480) // max(per_thread, 1)) // 32 * 32
    return int(max(32, min(256, b)))


def _default_block(n_species: int) -> int:
    """Threads per block so that three per-thread columns of NS doubles fit
    in about 100 KB of shared memory (two resident blocks per SM)."""
    per_thread = 3 * n_species * 8
    b = (100 * 1024 // max(per_thread, 1)) // 32 * 32
    return int(max(32, min(128, b)))

# }}}


class CudaCodeGenerator(CodeGenerator):
    """The ``cuda`` target of the code-generator registry."""

    @staticmethod
    def get_name() -> str:
        return "cuda"

    @staticmethod
    def supports_overloading() -> bool:
        return True

    @staticmethod
    def generate(name: str, sol, opts: CodeGenerationOptions = None) -> str:
        if opts is None:
            opts = CudaGenerationOptions()
        if opts.directive_offload is not None:
            raise TypeError(
                "OpenMP/ACC directive based offloading is not supported for "
                "CUDA code generation")
        if opts.scalar_type not in (None, "double"):
            raise TypeError("the CUDA target computes in double precision "
                            f"only (got scalar_type={opts.scalar_type!r})")
        if not isinstance(opts, CudaGenerationOptions):
            opts = CudaGenerationOptions(scalar_type=opts.scalar_type)
        return _Emitter(name, sol, opts).render()

    @staticmethod
    def build_module(source: str, name: str = "mechanism",
                     build_dir: Optional[str] = None) -> str:
        """Compile generated source to a shared library (cached by content
        hash); returns its path."""
        return build_shared_library(source, name, build_dir)

    @staticmethod
    def compile_class(name: str, source: str, sol):
        """Compile generated CUDA *source* into the drop-in class named
        *name* (``python.py:689-697`` counterpart).  The reference's Python
        source carries the class attributes inline; here they come from the
        mechanism *sol* the source was generated from, and the compiled
        library's own species and reaction counts are checked against it.
        The source is kept as ``_MODULE_SOURCE_CODE``."""
        import ctypes

        from ..thermochemistry import load_library, make_thermochem_class
        lib_path = build_shared_library(source, name)
        ns, nr = ctypes.c_int(), ctypes.c_int()
        load_library(lib_path).pyro_mechanism_info(
            ctypes.byref(ns), ctypes.byref(nr), None, None, None)
        if (ns.value, nr.value) != (sol.n_species, sol.n_reactions):
            raise ValueError(
                f"source is for {ns.value} species / {nr.value} reactions, "
                f"the mechanism has {sol.n_species} / {sol.n_reactions}")
        cls = make_thermochem_class(sol, lib_path, name)
        cls._MODULE_SOURCE_CODE = source
        return cls

    @staticmethod
    def get_thermochem_class(sol, opts: Optional[CodeGenerationOptions] = None,
                             name: str = "Thermochemistry"):
        """For the mechanism *sol*, return the drop-in CUDA
        ``Thermochemistry`` class (``python.py:699-707`` counterpart)."""
        from ..thermochemistry import make_thermochem_class
        src = CudaCodeGenerator.generate(name, sol, opts)
        lib = build_shared_library(
            src, f"{sol.n_species}sp{sol.n_reactions}rx")
        return make_thermochem_class(sol, lib, name)


# {{{ build

NVCC_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def default_build_dir() -> str:
    return os.environ.get("PYRO_GB300_BUILD_DIR", os.path.join(
        os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
        "_build"))


def nvcc_path() -> str:
    cand = os.environ.get("NVCC")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    return "nvcc"


def build_shared_library(source: str, name: str = "mechanism",
                         build_dir: Optional[str] = None,
                         extra_flags: Tuple[str, ...] = ()) -> str:
    build_dir = build_dir or default_build_dir()
    os.makedirs(build_dir, exist_ok=True)
    flags = NVCC_ARCH + ["-O3", "-lineinfo", "-std=c++17", "-shared",
                         "-Xcompiler", "-fPIC", "-Xcompiler",
                         "-fvisibility=hidden", f"-I{CSRC}"] + list(
        extra_flags)
    deps = b""
    for fn in sorted(os.listdir(CSRC)):
        if fn.endswith((".cuh", ".h")):
            with open(os.path.join(CSRC, fn), "rb") as f:
                deps += f.read()
    h = hashlib.sha256(source.encode() + deps + " ".join(flags).encode()
                       ).hexdigest()[:16]
    stem = "".join(ch if ch.isalnum() else "_" for ch in str(name))[:40]
    lib = os.path.join(build_dir, f"libpyro_{stem}_{h}.so")
    if os.path.exists(lib):
        return lib
    # content-addressed output written under a unique name and renamed into
    # place, so concurrent builders (threads or processes) never collide
    tag = f"{os.getpid()}_{threading.get_ident()}"
    cu = lib[:-3] + f".{tag}.cu"
    with open(cu, "w") as f:
        f.write(source)
    tmp = lib + f".{tag}.tmp"
    cmd = [nvcc_path()] + flags + ["-o", tmp, cu]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n"
                           + proc.stdout + proc.stderr)
    os.replace(cu, lib[:-3] + ".cu")
    os.replace(tmp, lib)
    return lib

# }}}

# vim: foldmethod=marker
