"""Cantera-YAML mechanism reader (the subset pyrometheus' fixture mechanisms
use) and writer.

PyYAML is not a dependency, so this module carries a small YAML parser for
the constructs Cantera input files use (block mappings and sequences, flow
``{...}``/``[...]`` collections spanning lines, ``|``/``>`` block scalars,
comments) and a loader with Cantera's semantics for the fields the code
generators read:

* ``units`` with SI conversion of pre-exponential factors by reaction order
  and of activation energies to J/kmol;
* NASA-7 two-range thermo (``temperature-ranges: [Tlow, Tmid, Thigh]``, data
  rows low then high) packed as ``[Tmid, hi(7), lo(7)]``;
* elementary, ``three-body`` (``+ M``) and ``falloff`` (``(+ M)``) reactions
  with Troe or Lindemann blending, efficiencies, ``default-efficiency``,
  ``orders`` and irreversible ``=>``.

Semantic source: the reference loads mechanisms with
``ct.Solution(mech, phase)`` (``pyrometheus/cli.py:38``,
``test/backends.py:224``); the behaviours restated here are Cantera's.
"""

from __future__ import annotations

import re
from typing import Any, Dict, List, Optional, Tuple

import numpy as np

from .mechanism import (Arrhenius, LindemannRate, NasaPoly2, Reaction,
                        Solution, Species, ThirdBody, TroeRate, gas_constant)

# {{{ minimal YAML parser


class _L:
    __slots__ = ("indent", "text")

    def __init__(self, indent: int, text: str):
        self.indent = indent
        self.text = text


def _strip_comment(line: str) -> str:
    quote = None
    for i, ch in enumerate(line):
        if quote:
            if ch == quote:
                quote = None
        elif ch in ("'", '"'):
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i]
    return line


def _depth(s: str) -> int:
    d, quote = 0, None
    for ch in s:
        if quote:
            if ch == quote:
                quote = None
        elif ch in ("'", '"'):
            quote = ch
        elif ch in "[{":
            d += 1
        elif ch in "]}":
            d -= 1
    return d


_BLOCK_RE = re.compile(r"^(.*?:)\s*([|>])([-+]?)$")


def _logical_lines(text: str) -> Tuple[List[_L], Dict[str, str]]:
    raw = text.replace("\t", "    ").split("\n")
    out: List[_L] = []
    blocks: Dict[str, str] = {}
    i = 0
    while i < len(raw):
        line = _strip_comment(raw[i]).rstrip()
        if not line.strip() or line.strip() in ("---", "..."):
            i += 1
            continue
        indent = len(line) - len(line.lstrip(" "))
        content = line.strip()
        m = _BLOCK_RE.match(content)
        if m:
            body = []
            i += 1
            while i < len(raw):
                r = raw[i].rstrip()
                if r.strip() and (len(r) - len(r.lstrip(" "))) <= indent:
                    break
                body.append(r)
                i += 1
            nonblank = [b for b in body if b.strip()]
            strip = min((len(b) - len(b.lstrip(" ")) for b in nonblank),
                        default=0)
            lines = [b[strip:] for b in body]
            while lines and not lines[-1].strip():
                lines.pop()
            sep = "\n" if m.group(2) == "|" else " "
            value = sep.join(lines)
            if m.group(3) != "-":
                value += "\n"
            token = f"\x00B{len(blocks)}"
            blocks[token] = value
            out.append(_L(indent, f"{m.group(1)} {token}"))
            continue
        while _depth(content) > 0 and i + 1 < len(raw):
            i += 1
            content += " " + _strip_comment(raw[i]).strip()
        out.append(_L(indent, content))
        i += 1
    return out, blocks


_INT_RE = re.compile(r"^[-+]?\d+$")
_FLOAT_RE = re.compile(
    r"^[-+]?(\d+\.?\d*([eE][-+]?\d+)?|\.\d+([eE][-+]?\d+)?|\d+[eE][-+]?\d+)$")


def _scalar(s: str, blocks: Dict[str, str]) -> Any:
    s = s.strip()
    if s in blocks:
        return blocks[s]
    if len(s) >= 2 and s[0] == s[-1] and s[0] in ("'", '"'):
        return s[1:-1]
    if _INT_RE.match(s):
        return int(s)
    if _FLOAT_RE.match(s):
        return float(s)
    low = s.lower()
    # YAML 1.2 core schema (Cantera reads with yaml-cpp): only true/false are
    # booleans, so species such as ``NO`` stay strings.
    if low == "true":
        return True
    if low == "false":
        return False
    if low in ("null", "~", ""):
        return None
    if low in (".inf", "+.inf"):
        return float("inf")
    if low == "-.inf":
        return float("-inf")
    return s


def _split_top(s: str, sep: str) -> List[str]:
    parts, d, quote, cur = [], 0, None, []
    for ch in s:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in ("'", '"'):
            quote = ch
        elif ch in "[{":
            d += 1
        elif ch in "]}":
            d -= 1
        elif ch == sep and d == 0:
            parts.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    parts.append("".join(cur))
    return parts


def _find_colon(s: str) -> int:
    """Index of the mapping colon (``key: value`` / ``key:``), else -1."""
    d, quote = 0, None
    for i, ch in enumerate(s):
        if quote:
            if ch == quote:
                quote = None
            continue
        if ch in ("'", '"'):
            quote = ch
        elif ch in "[{":
            d += 1
        elif ch in "]}":
            d -= 1
        elif ch == ":" and d == 0 and (i + 1 == len(s) or s[i + 1] == " "):
            return i
    return -1


def _flow(s: str, blocks: Dict[str, str]) -> Any:
    s = s.strip()
    if s.startswith("[") and s.endswith("]"):
        inner = s[1:-1].strip()
        if not inner:
            return []
        return [_flow(p, blocks) for p in _split_top(inner, ",")
                if p.strip()]
    if s.startswith("{") and s.endswith("}"):
        inner = s[1:-1].strip()
        d: Dict[str, Any] = {}
        if not inner:
            return d
        for p in _split_top(inner, ","):
            if not p.strip():
                continue
            c = _find_colon(p)
            if c < 0:
                d[_scalar(p, blocks)] = None
            else:
                d[_scalar(p[:c], blocks)] = _flow(p[c + 1:], blocks)
        return d
    return _scalar(s, blocks)


def _parse_block(lines: List[_L], i: int, indent: int, blocks):
    if lines[i].text.startswith("- ") or lines[i].text == "-":
        return _parse_seq(lines, i, indent, blocks)
    return _parse_map(lines, i, indent, blocks)


def _parse_seq(lines: List[_L], i: int, indent: int, blocks):
    items = []
    n = len(lines)
    while (i < n and lines[i].indent == indent
           and (lines[i].text.startswith("- ") or lines[i].text == "-")):
        text = lines[i].text
        rest = text[1:].lstrip(" ")
        if not rest:
            if i + 1 < n and lines[i + 1].indent > indent:
                val, i = _parse_block(lines, i + 1, lines[i + 1].indent,
                                      blocks)
            else:
                val, i = None, i + 1
        elif (not rest.startswith(("[", "{", "'", '"'))
              and _find_colon(rest) >= 0):
            col = indent + (len(text) - len(rest))
            lines[i] = _L(col, rest)
            val, i = _parse_map(lines, i, col, blocks)
        else:
            val, i = _flow(rest, blocks), i + 1
        items.append(val)
    return items, i


def _parse_map(lines: List[_L], i: int, indent: int, blocks):
    d: Dict[str, Any] = {}
    n = len(lines)
    while (i < n and lines[i].indent == indent
           and not lines[i].text.startswith("- ")):
        text = lines[i].text
        c = _find_colon(text)
        if c < 0:
            raise ValueError(f"YAML: expected 'key: value', got '{text}'")
        key = _scalar(text[:c], blocks)
        rest = text[c + 1:].strip()
        if rest:
            d[key] = _flow(rest, blocks)
            i += 1
        elif i + 1 < n and (lines[i + 1].indent > indent
                            or (lines[i + 1].indent == indent
                                and lines[i + 1].text.startswith("-"))):
            d[key], i = _parse_block(lines, i + 1, lines[i + 1].indent,
                                     blocks)
        else:
            d[key] = None
            i += 1
    return d, i


def parse_yaml(text: str) -> Any:
    """Parse the YAML subset used by Cantera mechanism files."""
    lines, blocks = _logical_lines(text)
    if not lines:
        return None
    val, i = _parse_block(lines, 0, lines[0].indent, blocks)
    if i != len(lines):
        raise ValueError(f"YAML: could not parse line '{lines[i].text}'")
    return val

# }}}


# {{{ Cantera semantics

_QUANTITY = {"kmol": 1.0, "mol": 1e-3, "molec": 1.0 / 6.02214076e26}
_LENGTH = {"m": 1.0, "cm": 1e-2, "mm": 1e-3}
_ENERGY_PER_QTY = {
    "J/kmol": 1.0, "J/mol": 1e3, "kJ/mol": 1e6, "kJ/kmol": 1e3,
    "cal/mol": 4184.0, "kcal/mol": 4.184e6, "cal/kmol": 4.184,
    "kcal/kmol": 4184.0,
    "K": gas_constant, "eV": 96485332.12331001,
}


def _conc_factor(units: Dict[str, str]) -> float:
    """SI value of one (length^3 / quantity) of the file's units."""
    return (_LENGTH[units.get("length", "m")] ** 3
            / _QUANTITY[units.get("quantity", "kmol")])


def _arrhenius(spec: Dict[str, Any], order: float,
               units: Dict[str, str]) -> Arrhenius:
    if isinstance(spec, list):
        spec = {"A": spec[0], "b": spec[1], "Ea": spec[2]}
    a = float(spec["A"]) * _conc_factor(units) ** (order - 1.0)
    ea = float(spec.get("Ea", 0.0)) * _ENERGY_PER_QTY[
        units.get("activation-energy", "J/kmol")]
    return Arrhenius(a, float(spec.get("b", 0.0)), ea)


_COLLIDER_RE = re.compile(r"\(\s*\+\s*([^()\s]+(?:\([^()]*\))?)\s*\)")


def _parse_side(side: str) -> Tuple[Dict[str, float], bool]:
    terms: Dict[str, float] = {}
    has_m = False
    for tok in side.split(" + "):
        tok = tok.strip()
        if not tok:
            continue
        if tok == "M":
            has_m = True
            continue
        m = re.match(r"^(\d+\.?\d*|\.\d+)\s+(\S+)$", tok)
        if m:
            nu, name = float(m.group(1)), m.group(2)
        else:
            nu, name = 1.0, tok
        terms[name] = terms.get(name, 0.0) + nu
    return terms, has_m


def parse_equation(eq: str):
    """Split a Cantera equation string.

    :returns: ``(reactants, products, reversible, three_body, collider)``;
        *three_body* is True for ``+ M`` terms, *collider* is the falloff
        collider name (``"M"`` or a species) for ``(+ X)`` terms, else None.
    """
    collider = None
    cols = _COLLIDER_RE.findall(eq)
    if cols:
        if len(set(cols)) != 1:
            raise ValueError(f"inconsistent falloff colliders in '{eq}'")
        collider = cols[0]
        eq = _COLLIDER_RE.sub(" ", eq)
    if "<=>" in eq:
        lhs, rhs = eq.split("<=>")
        reversible = True
    elif "=>" in eq:
        lhs, rhs = eq.split("=>")
        reversible = False
    elif "=" in eq:
        lhs, rhs = eq.split("=")
        reversible = True
    else:
        raise ValueError(f"no reaction arrow in '{eq}'")
    norm = lambda s: " ".join(s.split())  # noqa: E731
    reac, m1 = _parse_side(norm(lhs))
    prod, m2 = _parse_side(norm(rhs))
    if m1 != m2:
        raise ValueError(f"unbalanced third body in '{eq}'")
    return reac, prod, reversible, m1, collider


def _reaction(entry: Dict[str, Any], units: Dict[str, str],
              species: List[str]) -> Reaction:
    eq = entry["equation"]
    reac, prod, reversible, three_body, collider = parse_equation(eq)
    rtype = entry.get("type")
    if rtype is None:
        rtype = ("falloff" if collider is not None
                 else "three-body" if three_body else "elementary")
    orders = {k: float(v) for k, v in (entry.get("orders") or {}).items()}
    order = sum(orders.get(k, v) for k, v in reac.items()) \
        + sum(v for k, v in orders.items() if k not in reac)
    eff = {k: float(v) for k, v in (entry.get("efficiencies") or {}).items()
           if k in species}
    default_eff = float(entry.get("default-efficiency", 1.0))
    dup = bool(entry.get("duplicate", False))
    if rtype in ("elementary", "reaction", "Arrhenius"):
        rate = _arrhenius(entry["rate-constant"], order, units)
        return Reaction(eq, reac, prod, rate, reversible, orders, None, dup)
    if rtype == "three-body":
        rate = _arrhenius(entry["rate-constant"], order + 1.0, units)
        tb = ThirdBody(eff, default_eff)
        return Reaction(eq, reac, prod, rate, reversible, orders, tb, dup)
    if rtype == "falloff":
        low = _arrhenius(entry["low-P-rate-constant"], order + 1.0, units)
        high = _arrhenius(entry["high-P-rate-constant"], order, units)
        if collider is not None and collider != "M":
            eff, default_eff = {collider: 1.0}, 0.0
        tb = ThirdBody(eff, default_eff)
        if "Troe" in entry:
            t = entry["Troe"]
            coeffs = [float(t["A"]), float(t["T3"]), float(t["T1"])]
            if "T2" in t:
                coeffs.append(float(t["T2"]))
            rate = TroeRate(low, high, coeffs)
        elif "SRI" in entry:
            raise NotImplementedError("SRI falloff is not supported")
        else:
            rate = LindemannRate(low, high)
        return Reaction(eq, reac, prod, rate, reversible, orders, tb, dup)
    raise NotImplementedError(f"reaction type '{rtype}' ({eq})")


def _species(entry: Dict[str, Any]) -> Species:
    th = entry["thermo"]
    if th.get("model") != "NASA7":
        raise NotImplementedError(f"thermo model '{th.get('model')}'")
    ranges = [float(v) for v in th["temperature-ranges"]]
    data = th["data"]
    if len(ranges) == 3 and len(data) == 2:
        poly = NasaPoly2(ranges[0], ranges[1], ranges[2], data[0], data[1])
    elif len(ranges) == 2 and len(data) == 1:
        poly = NasaPoly2(ranges[0], ranges[1], ranges[1], data[0], data[0])
    else:
        raise ValueError(f"species {entry['name']}: bad NASA7 ranges")
    return Species(str(entry["name"]), entry["composition"], poly)


def load_mechanism(source: str, phase: Optional[str] = None,
                   text: Optional[str] = None,
                   transport: Optional[str] = None) -> Solution:
    """Load a Cantera-YAML mechanism (``ct.Solution(source, phase)``).

    ``transport="kinetic-theory"`` attaches mixture-averaged transport fits
    made from the species' Lennard-Jones ``diameter`` and ``well-depth``
    by first-order Chapman-Enskog theory
    (:func:`pyrometheus_gb300.transport_fits.kinetic_theory_fits`).  These
    approximate Cantera's fits, which add polar and rotational corrections
    and tabulated collision integrals; with Cantera installed, pass its
    ``Solution`` to the code generator instead.  By default no fits are
    attached."""
    if text is None:
        with open(source) as f:
            text = f.read()
    doc = parse_yaml(text)
    units = dict(doc.get("units") or {})
    phases = doc.get("phases") or []
    ph = None
    if phase is not None:
        for p in phases:
            if p.get("name") == phase:
                ph = p
        if ph is None:
            raise ValueError(f"phase '{phase}' not found in {source}")
    elif phases:
        ph = phases[0]
    all_species = {str(s["name"]): s for s in doc["species"]}
    names = list(all_species) if ph is None or ph.get("species") in (
        None, "all") else [str(n) for n in ph["species"]]
    species = [_species(all_species[n]) for n in names]
    elements = list(ph.get("elements")) if ph and ph.get("elements") \
        else None
    rxn_entries = doc.get("reactions") or []
    reactions = []
    for e in rxn_entries:
        r = _reaction(e, units, names)
        if all(k in names for k in list(r.reactants) + list(r.products)):
            reactions.append(r)
    sol = Solution(species, reactions, elements, source=str(source),
                   name=(ph or {}).get("name", "gas"))
    if transport is not None:
        if transport != "kinetic-theory":
            raise ValueError(f"unknown transport fits '{transport}'")
        from .transport_fits import kinetic_theory_fits
        sigma, eps = [], []
        for n in names:
            tr = all_species[n].get("transport")
            if not tr or "diameter" not in tr or "well-depth" not in tr:
                raise ValueError(f"species '{n}' has no Lennard-Jones "
                                 "transport data")
            sigma.append(float(tr["diameter"]))
            eps.append(float(tr["well-depth"]))
        sol.transport = kinetic_theory_fits(sol, sigma=sigma,
                                            well_depth=eps)
    return sol


# }}}


# {{{ writer (SI units)

def _num(x: float) -> str:
    return repr(float(x))


def dump_mechanism(sol: Solution, description: str = "") -> str:
    """Cantera-YAML text for *sol* in SI units (m, kmol, J/kmol).

    Values are written with ``repr`` so a reload reproduces every double
    exactly.
    """
    out = []
    if description:
        out.append("description: |-")
        out.extend("  " + ln for ln in description.splitlines())
        out.append("")
    out.append("units: {length: m, quantity: kmol, "
               "activation-energy: J/kmol}")
    out.append("")
    out.append("phases:")
    out.append(f"- name: {sol.name}")
    out.append("  thermo: ideal-gas")
    out.append(f"  elements: [{', '.join(sol.element_names)}]")
    out.append(f"  species: [{', '.join(sol.species_names)}]")
    out.append("  kinetics: gas")
    out.append("  reactions: all")
    out.append("")
    out.append("species:")
    for sp in sol.species():
        comp = ", ".join(f"{k}: {int(v) if float(v).is_integer() else v}"
                         for k, v in sp.composition.items())
        th = sp.thermo
        out.append(f"- name: {sp.name}")
        out.append(f"  composition: {{{comp}}}")
        out.append("  thermo:")
        out.append("    model: NASA7")
        out.append(f"    temperature-ranges: [{_num(th.min_temp)}, "
                   f"{_num(th.t_mid)}, {_num(th.max_temp)}]")
        out.append("    data:")
        out.append("    - [" + ", ".join(_num(v) for v in th.low) + "]")
        out.append("    - [" + ", ".join(_num(v) for v in th.high) + "]")
    out.append("")
    out.append("reactions:")

    def arr(r):
        return (f"{{A: {_num(r.pre_exponential_factor)}, "
                f"b: {_num(r.temperature_exponent)}, "
                f"Ea: {_num(r.activation_energy)}}}")

    for r in sol.reactions():
        out.append(f"- equation: {r.equation}")
        if r.reaction_type == "three-body-Arrhenius":
            out.append("  type: three-body")
            out.append(f"  rate-constant: {arr(r.rate)}")
        elif r.reaction_type.startswith("falloff"):
            out.append("  type: falloff")
            out.append(f"  low-P-rate-constant: {arr(r.rate.low_rate)}")
            out.append(f"  high-P-rate-constant: {arr(r.rate.high_rate)}")
            if r.rate.type == "Troe":
                fc = r.rate.falloff_coeffs
                keys = ["A", "T3", "T1", "T2"][:len(fc)]
                out.append("  Troe: {" + ", ".join(
                    f"{k}: {_num(v)}" for k, v in zip(keys, fc)) + "}")
        else:
            out.append(f"  rate-constant: {arr(r.rate)}")
        if r.third_body is not None:
            if r.third_body.efficiencies:
                out.append("  efficiencies: {" + ", ".join(
                    f"{k}: {_num(v)}"
                    for k, v in r.third_body.efficiencies.items()) + "}")
            if r.third_body.default_efficiency != 1.0:
                out.append("  default-efficiency: "
                           f"{_num(r.third_body.default_efficiency)}")
        if r.orders:
            out.append("  orders: {" + ", ".join(
                f"{k}: {_num(v)}" for k, v in r.orders.items()) + "}")
        if r.duplicate:
            out.append("  duplicate: true")
    return "\n".join(out) + "\n"

# }}}

# vim: foldmethod=marker
