"""Run the reference's flamelet solver driver and compressible-EOS loop in
this container.

TEST INFRASTRUCTURE ONLY -- used by CPU tests that are skipped when the
reference checkout is absent.  Nothing in the product imports this module.

``pyrometheus/flamelets/solver.py`` and ``thermodynamic_consistency.py``
import JAX, which is not installed here.  Their control flow needs only a
small part of it, supplied by a stand-in while the reference files are
executed:

* ``jax.numpy`` is numpy (``array`` returns an array that also answers
  ``block_until_ready``); ``jax.jit`` returns the function unchanged;
  ``jax.lax.while_loop`` and ``jax.lax.scan`` are Python loops (the scan
  is :func:`oracle.refgen._scan`, which already runs the reference's
  ``linear_solver.block_thomas``); ``jax.tree_util`` registration and
  ``jax.config`` are no-ops;
* the reference's ``state.py`` and ``make_pyro.py`` run unchanged;
  ``_array_to_state`` is wrapped so the fields it builds answer
  ``block_until_ready`` as JAX arrays do;
* ``FlameletEquations`` (``equations.py``, ``jax.vmap``/``jax.jacfwd`` over
  the generated class) is replaced by :class:`OracleGovEquations`, the
  same methods over the :class:`~oracle.flamelet_oracle.FlameletOracle`
  pieces for one flamelet.

The reference's ``FlameletSolver`` and ``CompressibleEOS`` classes are then
used unchanged (instances are made without their constructors, which build
the JAX equations, and given the attributes the constructors would set).
Its ``utils.py`` set-up helpers, its ``Laplacian`` and its
``FlameletEquations`` (around the reference's generated class and its own
``make_pyro_object``; ``jax.vmap`` is a loop, ``jax.jacfwd`` is not
provided) run the same way.
"""

from __future__ import annotations

import os
import sys
import types

import numpy as np

from .flamelet_oracle import FlameletOracle
from .refgen import REFERENCE_ROOT, _scan, reference_available


class _AtIndex:
    def __init__(self, array, index):
        self.array, self.index = array, index

    def set(self, value):
        out = self.array.copy()
        out[self.index] = value
        return out


class _At:
    def __init__(self, array):
        self.array = array

    def __getitem__(self, index):
        return _AtIndex(self.array, index)


class _Ready(np.ndarray):
    """A numpy array that also answers JAX's ``block_until_ready`` and
    functional ``.at[index].set(value)`` (a copy with the update)."""

    def block_until_ready(self):
        return self

    @property
    def at(self):
        return _At(self)


def _ready(x):
    return np.asarray(x).view(_Ready)


def _while_loop(cond, body, carry):
    while cond(carry):
        carry = body(carry)
    return carry


def _vmap(fun, in_axes=0):
    """``jax.vmap`` as a loop over the mapped axis, outputs stacked."""
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (list, tuple)) \
            else (in_axes,) * len(args)
        n = next(np.shape(a)[ax] for a, ax in zip(args, axes)
                 if ax is not None)
        outs = [fun(*[a if ax is None else np.take(a, i, axis=ax)
                      for a, ax in zip(args, axes)]) for i in range(n)]
        return _ready(np.stack(outs))
    return mapped


def _jacfwd_fd(fun, argnums=0, rel=1e-6):
    """``jax.jacfwd`` with respect to a point's state vector (argument 0)
    by central differences, the oracle's step rule: ``rel * max(|h|, 1)``
    for the enthalpy, ``rel`` for the mass fractions."""
    if argnums != 0:
        return _no_jacfwd(fun, argnums)

    def jac(x, *args):
        x = np.asarray(x, dtype=np.float64)
        cols = []
        for q in range(x.shape[0]):
            step = rel * max(abs(x[q]), 1.0) if q == 0 else rel
            xp, xm = x.copy(), x.copy()
            xp[q] += step
            xm[q] -= step
            cols.append((np.asarray(fun(_ready(xp), *args))
                         - np.asarray(fun(_ready(xm), *args))) / (2 * step))
        return np.stack(cols, axis=1)
    return jac


def _no_jacfwd(fun, argnums=0):
    """Forward-mode autodiff is not part of the stand-in: the functions it
    builds may be made, not called."""
    def unavailable(*args, **kwargs):
        raise NotImplementedError("jax.jacfwd is not available here")
    return unavailable


def _jax_modules():
    jnp = types.ModuleType("jax.numpy")
    jnp.__dict__.update({k: getattr(np, k) for k in dir(np)
                         if not k.startswith("__")})
    jnp.array = lambda *a, **k: _ready(np.array(*a, **k))
    lax = types.ModuleType("jax.lax")
    lax.scan = _scan
    lax.while_loop = _while_loop
    tree_util = types.ModuleType("jax.tree_util")
    tree_util.register_pytree_node_class = lambda cls: cls
    jax = types.ModuleType("jax")
    jax.numpy, jax.lax, jax.tree_util = jnp, lax, tree_util
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)

    def jit(fun=None, **kwargs):
        return fun if fun is not None else (lambda f: f)
    jax.jit = jit
    jax.vmap = _vmap
    jax.jacfwd = _no_jacfwd
    return {"jax": jax, "jax.numpy": jnp, "jax.lax": lax,
            "jax.tree_util": tree_util}


def _exec(name, relpath):
    path = os.path.join(REFERENCE_ROOT, *relpath.split("/"))
    mod = types.ModuleType(name)
    mod.__file__ = path
    sys.modules[name] = mod
    with open(path) as f:
        exec(compile(f.read(), path, "exec"), mod.__dict__)
    return mod


_CACHE = {}


def reference_flamelet_modules():
    """``(state, solver, thermodynamic_consistency)`` modules of the
    reference, executed against the stand-in."""
    if "mods" in _CACHE:
        return _CACHE["mods"]
    if not reference_available():
        raise RuntimeError("reference checkout not found")
    names = ["jax", "jax.numpy", "jax.lax", "jax.tree_util", "pyrometheus",
             "pyrometheus.flamelets", "pyrometheus.flamelets.make_pyro",
             "pyrometheus.flamelets.state",
             "pyrometheus.flamelets.linear_solver",
             "pyrometheus.flamelets.equations",
             "pyrometheus.flamelets.onedim_laplacian",
             "pyrometheus.flamelets.solver",
             "pyrometheus.flamelets.thermodynamic_consistency"]
    saved = {k: sys.modules.get(k) for k in names}
    try:
        sys.modules.update(_jax_modules())
        for pkg in ("pyrometheus", "pyrometheus.flamelets"):
            m = types.ModuleType(pkg)
            m.__path__ = []
            sys.modules[pkg] = m
        eqs = types.ModuleType("pyrometheus.flamelets.equations")
        eqs.FlameletEquations = None
        lap = types.ModuleType("pyrometheus.flamelets.onedim_laplacian")
        lap.Laplacian = None
        sys.modules[eqs.__name__] = eqs
        sys.modules[lap.__name__] = lap
        fl = "pyrometheus/flamelets/"
        _exec("pyrometheus.flamelets.make_pyro", fl + "make_pyro.py")
        state = _exec("pyrometheus.flamelets.state", fl + "state.py")
        _exec("pyrometheus.flamelets.linear_solver", fl + "linear_solver.py")
        solver = _exec("pyrometheus.flamelets.solver", fl + "solver.py")
        tc = _exec("pyrometheus.flamelets.thermodynamic_consistency",
                   fl + "thermodynamic_consistency.py")
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    base = state._array_to_state

    def array_to_state(array):
        s = base(array)
        return type(s)(enthalpy=_ready(s.enthalpy),
                       mass_fractions=_ready(s.mass_fractions))
    solver._array_to_state = array_to_state
    tc._array_to_state = array_to_state
    _CACHE["mods"] = (state, solver, tc)
    return _CACHE["mods"]


class _Gas:
    def __init__(self, fo, n_species):
        self.fo = fo
        self.num_species = n_species

    def get_temperature_from_enthalpy(self, h, y, t_guess):
        return _ready(self.fo.temperature(h, y, t_guess))


class OracleGovEquations:
    """The reference ``FlameletEquations`` methods the driver and the EOS
    loop call, for one flamelet, on the oracle pieces (central-difference
    source Jacobian, ``R T`` Jacobian and pressure gradient)."""

    def __init__(self, state_module, sol, n_x, dx, y_ox, y_fu):
        self.fo = FlameletOracle(sol)
        self.pyro_gas = _Gas(self.fo, sol.n_species)
        self.dx = float(dx)
        self.laplacian = types.SimpleNamespace(
            domain=types.SimpleNamespace(dx=self.dx, num_x=int(n_x)))
        self.y_ox = np.asarray(y_ox, dtype=np.float64)
        self.y_fu = np.asarray(y_fu, dtype=np.float64)
        self.State = state_module.FlameletState

    def rhs(self, state, diss_rate, viscous_diss, temp_guess, pressure,
            h_ox, h_fu):
        r = self.fo.residual(np.asarray(state.enthalpy),
                             np.asarray(state.mass_fractions), diss_rate,
                             viscous_diss, temp_guess, pressure, h_ox, h_fu,
                             self.y_ox, self.y_fu, self.dx)
        return self.State(enthalpy=_ready(r[0]), mass_fractions=_ready(r[1:]))

    def _source_jac(self, state, viscous_diss, temp_guess, pressure):
        return self.fo.source_jacobian_fd(np.asarray(state.enthalpy),
                                          np.asarray(state.mass_fractions),
                                          viscous_diss, temp_guess, pressure)

    def jac(self, state, diss_rate, viscous_diss, temp_guess, pressure):
        sj = self._source_jac(state, viscous_diss, temp_guess, pressure)
        return self.fo.blocks(sj, diss_rate, self.dx)

    def adjoint_operator(self, state, diss_rate, viscous_diss, temp_guess,
                         pressure):
        sj = self._source_jac(state, viscous_diss, temp_guess, pressure)
        return self.fo.adjoint_blocks(sj, diss_rate, self.dx)

    def compressible_eos_rt(self, state_as_array, temp_guess, pressure):
        a = np.asarray(state_as_array)
        return self.fo.eos_rt(a[0], a[1:], temp_guess)

    def compressible_eos_rt_jacobian(self, state_as_array, temp_guess,
                                     pressure):
        a = np.asarray(state_as_array)
        return self.fo.eos_rt_jacobian_fd(a[0], a[1:], temp_guess)

    def source_gradient_wrt_pressure(self, state_as_array, viscous_diss,
                                     temp_guess, pressure):
        a = np.asarray(state_as_array)
        return self.fo.source_pressure_gradient_fd(a[0], a[1:], viscous_diss,
                                                   temp_guess, pressure)


def reference_solver(sol, n_x, dx, y_ox, y_fu):
    """The reference's ``FlameletSolver`` for one flamelet of *n_x* points
    of spacing *dx*, on the oracle pieces."""
    state, solver, _ = reference_flamelet_modules()
    fs = solver.FlameletSolver.__new__(solver.FlameletSolver)
    fs.domain = None
    fs.gov_eqns = OracleGovEquations(state, sol, n_x, dx, y_ox, y_fu)
    fs.num_v = sol.n_species + 1
    return fs


def reference_eos(config, forward_solver):
    """The reference's ``CompressibleEOS`` around a
    :func:`reference_solver`."""
    _, _, tc = reference_flamelet_modules()
    eos = tc.CompressibleEOS.__new__(tc.CompressibleEOS)
    eos.config = config
    eos.fwd_solver = forward_solver
    nv = forward_solver.num_v
    n_x = forward_solver.gov_eqns.laplacian.domain.num_x
    unit_h = np.zeros((nv, n_x))
    unit_h[0] = 1.0
    eos.unit_h = unit_h
    return eos


def state_of(phi):
    """A reference ``FlameletState`` of an ``[S+1, N]`` array."""
    state, _, _ = reference_flamelet_modules()
    return state.FlameletState(enthalpy=_ready(phi[0]),
                               mass_fractions=_ready(phi[1:]))


def reference_flamelet_utils():
    """The reference's ``flamelets/utils.py`` module (``bell_profile``,
    ``stoichiometric_mixture_fraction``), executed against the stand-in."""
    if "utils" in _CACHE:
        return _CACHE["utils"]
    if not reference_available():
        raise RuntimeError("reference checkout not found")
    names = ["jax", "jax.numpy", "jax.lax", "jax.tree_util",
             "pyrometheus.flamelets.utils"]
    saved = {k: sys.modules.get(k) for k in names}
    try:
        sys.modules.update(_jax_modules())
        mod = _exec("pyrometheus.flamelets.utils",
                    "pyrometheus/flamelets/utils.py")
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    _CACHE["utils"] = mod
    return mod


def reference_laplacian(num_x):
    """The reference's ``Laplacian`` (``onedim_laplacian.py``, with its
    ``stencils.py`` and ``domain.py``) on the uniform grid of *num_x* points
    over [0, 1], executed against the stand-in."""
    state, _, _ = reference_flamelet_modules()
    if "lap" not in _CACHE:
        names = ["jax", "jax.numpy", "jax.lax", "jax.tree_util", "pyrometheus",
                 "pyrometheus.flamelets", "pyrometheus.flamelets.state",
                 "pyrometheus.flamelets.stencils",
                 "pyrometheus.flamelets.domain",
                 "pyrometheus.flamelets.onedim_laplacian"]
        saved = {k: sys.modules.get(k) for k in names}
        try:
            sys.modules.update(_jax_modules())
            for pkg in ("pyrometheus", "pyrometheus.flamelets"):
                m = types.ModuleType(pkg)
                m.__path__ = []
                sys.modules[pkg] = m
            sys.modules["pyrometheus.flamelets.state"] = state
            fl = "pyrometheus/flamelets/"
            _exec("pyrometheus.flamelets.stencils", fl + "stencils.py")
            domain = _exec("pyrometheus.flamelets.domain", fl + "domain.py")
            lap = _exec("pyrometheus.flamelets.onedim_laplacian",
                        fl + "onedim_laplacian.py")
        finally:
            for k, v in saved.items():
                if v is None:
                    sys.modules.pop(k, None)
                else:
                    sys.modules[k] = v
        _CACHE["lap"] = (domain, lap)
    domain, lap = _CACHE["lap"]
    return lap.Laplacian(domain.Domain(domain.DomainConfig(
        num_x=int(num_x), x_l=0.0, x_r=1.0)))


def reference_flamelet_equations(sol, num_x, y_ox, y_fu,
                                 fd_jacobian=False):
    """The reference's ``FlameletEquations`` (``equations.py``) for one
    flamelet of *num_x* points over [0, 1], around the reference's generated
    class (``oracle.refgen``) wrapped by its own ``make_pyro_object`` on the
    stand-in ``jax.numpy``.  ``rhs``, ``source_terms`` and the vmapped
    ``compressible_eos_rt`` run; the ``jax.jacfwd`` Jacobians do not, unless
    *fd_jacobian* puts central differences in place of ``jax.jacfwd`` for
    the source Jacobian (``vmap_jacobian``, used by ``jac`` and
    ``jacobian_action``)."""
    from .refgen import reference_class
    state, _, _ = reference_flamelet_modules()
    lap = reference_laplacian(num_x)
    if "eqs" not in _CACHE:
        names = ["jax", "jax.numpy", "jax.lax", "jax.tree_util", "pyrometheus",
                 "pyrometheus.flamelets", "pyrometheus.flamelets.state",
                 "pyrometheus.flamelets.make_pyro",
                 "pyrometheus.flamelets.onedim_laplacian",
                 "pyrometheus.flamelets.equations"]
        saved = {k: sys.modules.get(k) for k in names}
        try:
            mods = _jax_modules()
            sys.modules.update(mods)
            for pkg in ("pyrometheus", "pyrometheus.flamelets"):
                m = types.ModuleType(pkg)
                m.__path__ = []
                sys.modules[pkg] = m
            sys.modules["pyrometheus.flamelets.state"] = state
            sys.modules["pyrometheus.flamelets.onedim_laplacian"] = \
                sys.modules.get("pyrometheus.flamelets.onedim_laplacian") \
                or types.ModuleType("pyrometheus.flamelets.onedim_laplacian")
            sys.modules["pyrometheus.flamelets.onedim_laplacian"].Laplacian \
                = type(lap)
            fl = "pyrometheus/flamelets/"
            make_pyro = _exec("pyrometheus.flamelets.make_pyro",
                              fl + "make_pyro.py")
            eqs = _exec("pyrometheus.flamelets.equations",
                        fl + "equations.py")
        finally:
            for k, v in saved.items():
                if v is None:
                    sys.modules.pop(k, None)
                else:
                    sys.modules[k] = v
        # JAX arrays defer arithmetic with unknown types to them; numpy
        # arrays do so for classes that opt out of ufuncs
        state.StateContainer.__array_ufunc__ = None
        _CACHE["eqs"] = (make_pyro, eqs, mods["jax.numpy"])
    make_pyro, eqs, jnp = _CACHE["eqs"]
    gas = make_pyro.make_pyro_object(reference_class(sol), jnp)
    if fd_jacobian:
        eqs.jax.jacfwd = _jacfwd_fd
    try:
        return eqs.FlameletEquations(gas, lap, _ready(y_ox), _ready(y_fu))
    finally:
        eqs.jax.jacfwd = _no_jacfwd
