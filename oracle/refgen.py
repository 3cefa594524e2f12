"""Run the reference's own Python code generator in this container.

TEST INFRASTRUCTURE ONLY -- used by ``tests/golden/make_golden.py`` and by
CPU tests that are skipped when the reference checkout is absent.  Nothing in
the product imports this module.

The reference generator (``pyrometheus/codegen/python.py`` plus
``pyrometheus/chem_expr.py``) is pure Python, but its three dependencies are
not installed here (no network):

* ``cantera`` -- only its object model is needed at generation time
  (``Solution``, ``NasaPoly2``, ``TroeRate``, ``LindemannRate``,
  ``FalloffRate``, ``Arrhenius``, ``gas_constant``, ``one_atm``); it is
  provided by :mod:`pyrometheus_gb300.mechanism`, whose classes expose the
  same attribute surface;
* ``pymbolic`` -- the expression builder and ``StringifyMapper`` the
  generator subclasses (``python.py:56-86``); restated below with pymbolic's
  operator-simplification rules (adding 0, multiplying by 1 or 0, raising to
  0 or 1 are folded; sums and products flatten) so the emitted expressions
  have the same tree, hence the same floating-point evaluation order;
* ``mako`` -- the ``Template`` renderer for ``python.py:106-642``; restated
  below for the constructs that template uses (``%for/%if/%else/%end*``
  control lines, ``${...}`` substitutions, ``<% %>`` line joiners).

:func:`reference_class` then calls the reference's
``PythonCodeGenerator.generate`` / ``compile_class`` unchanged and returns
the reference's generated ``Thermochemistry`` class, which runs on numpy.
"""

from __future__ import annotations

import importlib
import numbers
import os
import re
import sys
import types

import numpy as np

# The reference checkout is found through PYRO_REFERENCE_ROOT alone; with
# it unset, everything that runs the reference is skipped.
REFERENCE_ROOT = os.environ.get("PYRO_REFERENCE_ROOT", "")


def reference_available() -> bool:
    return bool(REFERENCE_ROOT) and os.path.isfile(os.path.join(
        REFERENCE_ROOT, "pyrometheus", "codegen", "python.py"))


# {{{ pymbolic stand-in

PREC_NONE, PREC_IF, PREC_LOGICAL_OR, PREC_LOGICAL_AND = 0, 1, 2, 3
PREC_COMPARISON, PREC_SUM, PREC_PRODUCT, PREC_UNARY = 4, 5, 6, 7
PREC_POWER, PREC_CALL = 8, 9


def _is_num(x) -> bool:
    return isinstance(x, (numbers.Number, np.number)) and not isinstance(
        x, bool)


def _is_zero(x) -> bool:
    return _is_num(x) and x == 0


def _is_one(x) -> bool:
    return _is_num(x) and x == 1


def _valid(x) -> bool:
    return _is_num(x) or isinstance(x, Expression)


class Expression:
    # numpy must defer to our reflected operators (np.float64 + expr)
    __array_ufunc__ = None
    mapper_method = None

    def __add__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return self
        if isinstance(other, Sum):
            return Sum((self,) + other.children)
        return Sum((self, other))

    def __radd__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return self
        return Sum((other, self))

    def __sub__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return self
        return self + (-other)

    def __rsub__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return -self
        return Sum((other, -self))

    def __mul__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_one(other):
            return self
        if _is_zero(other):
            return 0
        if isinstance(other, Product):
            return Product((self,) + other.children)
        return Product((self, other))

    def __rmul__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_one(other):
            return self
        if _is_zero(other):
            return 0
        return Product((other, self))

    def __truediv__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_one(other):
            return self
        return Quotient(self, other)

    def __rtruediv__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return 0
        return Quotient(other, self)

    def __pow__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return 1
        if _is_one(other):
            return self
        return Power(self, other)

    def __rpow__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_one(other):
            return 1
        return Power(other, self)

    def __neg__(self):
        return -1 * self

    def __getitem__(self, index):
        return Subscript(self, index)

    def __call__(self, *params):
        return Call(self, tuple(params))

    def __repr__(self):
        return f"{type(self).__name__}({StringifyMapper()(self)})"


class Variable(Expression):
    mapper_method = "map_variable"

    def __init__(self, name):
        self.name = name


class Subscript(Expression):
    mapper_method = "map_subscript"

    def __init__(self, aggregate, index):
        self.aggregate = aggregate
        self.index = index


class Call(Expression):
    mapper_method = "map_call"

    def __init__(self, function, parameters):
        self.function = function
        self.parameters = parameters


class Sum(Expression):
    mapper_method = "map_sum"

    def __init__(self, children):
        self.children = tuple(children)

    def __add__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return self
        if isinstance(other, Sum):
            return Sum(self.children + other.children)
        return Sum(self.children + (other,))

    def __radd__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return self
        return Sum((other,) + self.children)

    def __sub__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_zero(other):
            return self
        return Sum(self.children + (-other,))


class Product(Expression):
    mapper_method = "map_product"

    def __init__(self, children):
        self.children = tuple(children)

    def __mul__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_one(other):
            return self
        if _is_zero(other):
            return 0
        if isinstance(other, Product):
            return Product(self.children + other.children)
        return Product(self.children + (other,))

    def __rmul__(self, other):
        if not _valid(other):
            return NotImplemented
        if _is_one(other):
            return self
        if _is_zero(other):
            return 0
        return Product((other,) + self.children)


class Quotient(Expression):
    mapper_method = "map_quotient"

    def __init__(self, numerator, denominator):
        self.numerator = numerator
        self.denominator = denominator


class Power(Expression):
    mapper_method = "map_power"

    def __init__(self, base, exponent):
        self.base = base
        self.exponent = exponent


class Comparison(Expression):
    mapper_method = "map_comparison"

    def __init__(self, left, operator, right):
        self.left = left
        self.operator = operator
        self.right = right


class If(Expression):
    mapper_method = "map_if"

    def __init__(self, condition, then, else_):
        self.condition = condition
        self.then = then
        self.else_ = else_


_ATOMIC = (Variable, Subscript, Call)


class StringifyMapper:
    """Renders expressions as Python source.  Compound operands are always
    parenthesised, which never changes the evaluation order of the tree."""

    def __call__(self, expr, prec=PREC_NONE, *args, **kwargs):
        return self.rec(expr, prec, *args, **kwargs)

    def rec(self, expr, prec, *args, **kwargs):
        if isinstance(expr, Expression):
            return getattr(self, expr.mapper_method)(expr, prec, *args,
                                                     **kwargs)
        if _is_num(expr):
            return self.map_constant(expr, prec, *args, **kwargs)
        raise TypeError(f"cannot stringify {type(expr)}")

    def format(self, fmt, *args):
        return fmt % args

    def join_rec(self, joiner, iterable, prec, *args, **kwargs):
        return joiner.join(self.rec(i, prec, *args, **kwargs)
                           for i in iterable)

    def _operand(self, expr, prec, *args, **kwargs):
        s = self.rec(expr, prec, *args, **kwargs)
        if isinstance(expr, _ATOMIC) or (_is_num(expr) and expr >= 0):
            return s
        return f"({s})"

    # defaults (the reference's mapper overrides constant/comparison/if/call)
    def map_constant(self, expr, enclosing_prec, *args, **kwargs):
        return repr(expr)

    def map_variable(self, expr, enclosing_prec, *args, **kwargs):
        return expr.name

    def map_subscript(self, expr, enclosing_prec, *args, **kwargs):
        idx = expr.index
        if isinstance(idx, tuple):
            inner = ", ".join(self.rec(i, PREC_NONE, *args, **kwargs)
                              for i in idx)
        else:
            inner = self.rec(idx, PREC_NONE, *args, **kwargs)
        return f"{self.rec(expr.aggregate, PREC_CALL, *args, **kwargs)}" \
               f"[{inner}]"

    def map_call(self, expr, enclosing_prec, *args, **kwargs):
        return "%s(%s)" % (self.rec(expr.function, PREC_CALL, *args,
                                    **kwargs),
                           self.join_rec(", ", expr.parameters, PREC_NONE,
                                         *args, **kwargs))

    def map_sum(self, expr, enclosing_prec, *args, **kwargs):
        return " + ".join(self._operand(c, PREC_SUM, *args, **kwargs)
                          for c in expr.children)

    def map_product(self, expr, enclosing_prec, *args, **kwargs):
        return "*".join(self._operand(c, PREC_PRODUCT, *args, **kwargs)
                        for c in expr.children)

    def map_quotient(self, expr, enclosing_prec, *args, **kwargs):
        return "%s / %s" % (
            self._operand(expr.numerator, PREC_PRODUCT, *args, **kwargs),
            self._operand(expr.denominator, PREC_PRODUCT, *args, **kwargs))

    def map_power(self, expr, enclosing_prec, *args, **kwargs):
        return "%s**%s" % (
            self._operand(expr.base, PREC_POWER, *args, **kwargs),
            self._operand(expr.exponent, PREC_POWER, *args, **kwargs))

    def map_comparison(self, expr, enclosing_prec, *args, **kwargs):
        return "%s %s %s" % (
            self._operand(expr.left, PREC_COMPARISON, *args, **kwargs),
            expr.operator,
            self._operand(expr.right, PREC_COMPARISON, *args, **kwargs))

    def map_if(self, expr, enclosing_prec, *args, **kwargs):
        return "(%s if %s else %s)" % (
            self.rec(expr.then, PREC_NONE, *args, **kwargs),
            self.rec(expr.condition, PREC_NONE, *args, **kwargs),
            self.rec(expr.else_, PREC_NONE, *args, **kwargs))

class CCodeMapper(StringifyMapper):
    """Renders expressions as C (``pymbolic.mapper.c_code.CCodeMapper``,
    which the reference's C++ target subclasses, ``cpp.py:48-52``):
    ``pow(a, b)`` for powers, ``(c ? a : b)`` for conditionals, ``&&`` /
    ``||`` / ``!`` for logic; everything else as the Python mapper, whose
    compound operands are always parenthesised (so the tree's evaluation
    order is kept)."""

    def map_power(self, expr, enclosing_prec, *args, **kwargs):
        return "pow(%s, %s)" % (self.rec(expr.base, PREC_NONE, *args,
                                         **kwargs),
                                self.rec(expr.exponent, PREC_NONE, *args,
                                         **kwargs))

    def map_if(self, expr, enclosing_prec, *args, **kwargs):
        return "(%s ? %s : %s)" % (
            self.rec(expr.condition, PREC_NONE, *args, **kwargs),
            self.rec(expr.then, PREC_NONE, *args, **kwargs),
            self.rec(expr.else_, PREC_NONE, *args, **kwargs))

# }}}


# {{{ mako stand-in

_CTRL_RE = re.compile(r"^[ \t]*%(?!%)(.*)$")


class Template:
    """Renders the Mako constructs the reference templates use."""

    def __init__(self, text, strict_undefined=False, **kwargs):
        self.text = text

    def _compile(self):
        text = re.sub(r"<%\s*%>", "", self.text)
        exprs = []
        out, i = [], 0
        while True:
            j = text.find("${", i)
            if j < 0:
                out.append(text[i:])
                break
            out.append(text[i:j])
            depth, k, quote = 1, j + 2, None
            while depth:
                ch = text[k]
                if quote:
                    if ch == quote:
                        quote = None
                elif ch in "'\"":
                    quote = ch
                elif ch in "{[(":
                    depth += 1
                elif ch in "}])":
                    depth -= 1
                k += 1
            exprs.append(text[j + 2:k - 1])
            out.append(f"\x01{len(exprs) - 1}\x01")
            i = k
        text = "".join(out)
        code, indent = ["def __render(__out, __ctx):",
                        "    globals().update(__ctx)"], 1
        for line in text.split("\n"):
            m = _CTRL_RE.match(line)
            if m:
                stmt = m.group(1).strip()
                word = stmt.split()[0] if stmt else ""
                if word.startswith("end"):
                    indent -= 1
                elif word in ("else:", "else") or word.startswith("elif"):
                    code.append("    " * (indent - 1) + stmt)
                else:
                    code.append("    " * indent + stmt)
                    indent += 1
                continue
            parts = re.split(r"\x01(\d+)\x01", line)
            pieces = []
            for n, part in enumerate(parts):
                if n % 2 == 0:
                    if part:
                        pieces.append(repr(part))
                else:
                    pieces.append("str((%s))" % exprs[int(part)]
                                  .replace("\n", " "))
            pieces.append(repr("\n"))
            code.append("    " * indent + "__out.append(%s)"
                        % " + ".join(pieces))
        return "\n".join(code)

    def render(self, **context):
        ns = {}
        exec(compile(self._compile(), "<template>", "exec"), ns)
        out = []
        ns["__render"](out, context)
        return "".join(out)

# }}}


# {{{ module registration

def _install_stubs():
    from pyrometheus_gb300 import mechanism as mech

    ct = types.ModuleType("cantera")
    for name in ("Solution", "NasaPoly2", "Arrhenius", "ArrheniusRate",
                 "FalloffRate", "TroeRate", "LindemannRate", "Reaction",
                 "Species", "ThirdBody", "gas_constant", "one_atm"):
        setattr(ct, name, getattr(mech, name))
    ct.FalloffReaction = mech.Reaction

    pymbolic = types.ModuleType("pymbolic")
    prim = types.ModuleType("pymbolic.primitives")
    for name in ("Expression", "Variable", "Subscript", "Call", "Sum",
                 "Product", "Quotient", "Power", "Comparison", "If"):
        setattr(prim, name, globals()[name])
    mapper = types.ModuleType("pymbolic.mapper")
    stringifier = types.ModuleType("pymbolic.mapper.stringifier")
    stringifier.StringifyMapper = StringifyMapper
    for name, val in globals().items():
        if name.startswith("PREC_"):
            setattr(stringifier, name, val)
    c_code = types.ModuleType("pymbolic.mapper.c_code")
    c_code.CCodeMapper = CCodeMapper
    pymbolic.primitives = prim
    pymbolic.mapper = mapper
    mapper.stringifier = stringifier
    mapper.c_code = c_code

    mako = types.ModuleType("mako")
    mako_template = types.ModuleType("mako.template")
    mako_template.Template = Template
    mako.template = mako_template

    # a package shell so importing submodules skips the reference's
    # __init__ (which imports the C++ and Fortran generators as well)
    pkg = types.ModuleType("pyrometheus")
    pkg.__path__ = [os.path.join(REFERENCE_ROOT, "pyrometheus")]

    mods = {"cantera": ct, "pymbolic": pymbolic,
            "pymbolic.primitives": prim, "pymbolic.mapper": mapper,
            "pymbolic.mapper.stringifier": stringifier,
            "pymbolic.mapper.c_code": c_code, "mako": mako,
            "mako.template": mako_template, "pyrometheus": pkg}
    return mods


_REF = None


def reference_generator():
    """The reference's ``PythonCodeGenerator`` class, imported from the
    reference checkout with the stand-ins above."""
    global _REF
    if _REF is not None:
        return _REF
    if not reference_available():
        raise RuntimeError("reference checkout not found (set "
                           "PYRO_REFERENCE_ROOT to its root)")
    mods = _install_stubs()
    saved = {k: sys.modules.get(k) for k in mods}
    saved.update({k: sys.modules.get(k) for k in
                  ("pyrometheus.codegen", "pyrometheus.codegen.python",
                   "pyrometheus.chem_expr")})
    try:
        sys.modules.update(mods)
        pycg = importlib.import_module("pyrometheus.codegen.python")
        _REF = pycg.PythonCodeGenerator
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return _REF


class _TransportPlaceholder:
    """The reference template also emits mixture-averaged transport methods
    (``python.py:564-641``), which read Cantera transport fits.  For a
    mechanism without fits, unit fits are supplied only to let the template
    render (its transport methods are then never called)."""

    def __init__(self, sol):
        self._sol = sol

    def __getattr__(self, name):
        return getattr(self._sol, name)

    @staticmethod
    def get_viscosity_polynomial(k):
        return np.array([1.0, 0.0, 0.0, 0.0, 0.0])

    get_thermal_conductivity_polynomial = get_viscosity_polynomial

    @staticmethod
    def get_binary_diff_coeffs_polynomial(i, j):
        return np.array([1.0, 0.0, 0.0, 0.0, 0.0])


_REF_CPP = None


def reference_cpp_generator():
    """The reference's ``CppCodeGenerator`` (``codegen/cpp.py``), imported
    the same way."""
    global _REF_CPP
    if _REF_CPP is not None:
        return _REF_CPP
    if not reference_available():
        raise RuntimeError("reference checkout not found (set "
                           "PYRO_REFERENCE_ROOT to its root)")
    mods = _install_stubs()
    saved = {k: sys.modules.get(k) for k in mods}
    saved.update({k: sys.modules.get(k) for k in
                  ("pyrometheus.codegen", "pyrometheus.codegen.cpp",
                   "pyrometheus.chem_expr")})
    try:
        sys.modules.update(mods)
        cppcg = importlib.import_module("pyrometheus.codegen.cpp")
        _REF_CPP = cppcg.CppCodeGenerator
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return _REF_CPP


def reference_cpp_source(sol, name: str = "Thermochemistry") -> str:
    """The C++20 header the reference's C++ target generates for *sol*."""
    if getattr(sol, "transport", None) is None:
        sol = _TransportPlaceholder(sol)
    return reference_cpp_generator().generate(name, sol)


def reference_source(sol, name: str = "Thermochemistry") -> str:
    if getattr(sol, "transport", None) is None:
        sol = _TransportPlaceholder(sol)
    return reference_generator().generate(name, sol)


def reference_class(sol, name: str = "Thermochemistry"):
    gen = reference_generator()
    return gen.compile_class(name, reference_source(sol, name))

# }}}

# vim: foldmethod=marker


# {{{ jax stand-in for the reference's block-Thomas

def _scan(f, init, xs):
    """``jax.lax.scan`` over the leading axis of a tuple of arrays."""
    leaves = xs if isinstance(xs, tuple) else (xs,)
    n = leaves[0].shape[0]
    if n == 0:
        # empty scan: outputs shaped like the carry (as in the reference's
        # two scans), with a zero-length leading axis
        if isinstance(init, tuple):
            return init, tuple(np.empty((0,) + np.shape(c)) for c in init)
        return init, np.empty((0,) + np.shape(init))
    carry = init
    outs = []
    for i in range(n):
        item = tuple(x[i] for x in leaves) if isinstance(xs, tuple) \
            else leaves[0][i]
        carry, y = f(carry, item)
        outs.append(y)
    if outs and isinstance(outs[0], tuple):
        stacked = tuple(np.stack([o[k] for o in outs])
                        for k in range(len(outs[0])))
    else:
        stacked = np.stack(outs) if outs else None
    return carry, stacked


def reference_block_thomas():
    """The reference's ``flamelets.linear_solver.block_thomas`` with
    ``jax``/``jax.numpy`` mapped to a numpy ``lax.scan`` and numpy."""
    if not reference_available():
        raise RuntimeError("reference checkout not found")
    jax = types.ModuleType("jax")
    lax = types.ModuleType("jax.lax")
    lax.scan = _scan
    jax.lax = lax
    jax.numpy = np
    path = os.path.join(REFERENCE_ROOT, "pyrometheus", "flamelets",
                        "linear_solver.py")
    saved = {k: sys.modules.get(k) for k in ("jax", "jax.numpy", "jax.lax")}
    try:
        sys.modules.update({"jax": jax, "jax.numpy": np, "jax.lax": lax})
        ns = {"__name__": "reference_linear_solver"}
        with open(path) as f:
            exec(compile(f.read(), path, "exec"), ns)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return ns["block_thomas"]

# }}}
