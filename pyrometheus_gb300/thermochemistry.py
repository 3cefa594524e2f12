"""Drop-in ``Thermochemistry`` on torch CUDA tensors.

The class mirrors the generated numpy/JAX class of
``pyrometheus/codegen/python.py:106-642``: the same attribute names
(``python.py:180-199``), method names and argument order, and array shapes
(species-major: ``Y[S, N]``; outputs ``[S, N]`` / ``[R, N]``; per-state
scalars ``[N]``; Python scalars broadcast).  Every method runs a kernel of the
mechanism's generated CUDA library through its C ABI on the current torch
stream; there is no CPU path.  Inputs may be Python numbers, numpy arrays or
torch tensors; they are moved to the device as float64.  Outputs are fresh
CUDA float64 tensors, as the reference returns fresh arrays.

``get_temperature`` keeps the reference's contract: Newton on
``e(T) = e0`` (``do_energy=True``) or ``h(T) = h0`` with ``|dT| < 1e-6`` and
at most 500 iterations, raising ``RuntimeError("Temperature iteration failed
to converge")`` when any state does not converge (``python.py:375-396``).
"""

from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from .mechanism import gas_constant, one_atm

try:
    import torch
except ImportError:  # pragma: no cover - torch is a hard dependency
    torch = None

_STATUS = {
    0: "ok",
    1: "invalid argument",
    2: "CUDA launch failed",
    3: "Newton iteration did not converge",
    4: "unsupported option",
}

SPECIES_PROPS = {"cp_r": 0, "h_rt": 1, "s_r": 2, "g_rt": 3, "dcp_r": 4,
                 "dh_rt": 5, "ds_r": 6}
MIXTURE_PROPS = {"mmw": 0, "rspec": 1, "cp": 2, "cv": 3, "h": 4, "e": 5,
                 "density": 6, "pressure": 7}
REACTION_MODES = {"log_keq": 0, "k_fwd": 1, "net": 2, "fwd": 3, "rev": 4}

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_INT = ctypes.c_int
_D = ctypes.c_double

_SIGNATURES = {
    "pyro_hot_block_size": [],
    "pyro_mechanism_info": [_P, _P, _P, _P, _P],
    "pyro_species_property": [_INT, _P, _I64, _P, _I64, _I64, _P],
    "pyro_mixture_property": [_INT, _P, _I64, _P, _I64, _P, _I64, _P, _I64,
                              _P],
    "pyro_species_scale": [_INT, _P, _I64, _P, _I64, _P, _I64, _I64, _P],
    "pyro_reaction_quantity": [_INT, _P, _I64, _P, _I64, _P, _I64, _I64, _P],
    "pyro_net_production_rates": [_P, _I64, _P, _I64, _P, _I64, _P, _I64,
                                  _I64, _P],
    "pyro_creation_destruction_rates": [_P, _I64, _P, _I64, _P, _I64, _P, _P,
                                        _I64, _I64, _P],
    "pyro_temperature": [_P, _I64, _P, _I64, _P, _I64, _INT, _D, _INT, _P, _P,
                         _I64, _P],
    "pyro_fused_step": [_P, _I64, _P, _I64, _P, _I64, _P, _I64, _P, _I64,
                        _INT, _D, _INT, _P, _I64, _P, _P, _I64, _P],
    "pyro_reactor_source": [_P, _I64, _P, _I64, _P, _I64, _P, _I64, _I64,
                            _P],
    "pyro_reactor_jacobian": [_P, _I64, _P, _I64, _P, _I64, _P, _I64, _I64,
                              _P],
    "pyro_reactor_source_dp": [_P, _I64, _P, _I64, _P, _I64, _P, _I64, _I64,
                               _P],
    "pyro_reactor_source_jacobian": [_P, _I64, _P, _I64, _P, _I64, _P, _I64,
                                     _P, _I64, _I64, _P],
    "pyro_reactor_vjp": [_P, _I64, _P, _I64, _P, _I64, _P, _I64, _P, _P,
                         _I64, _P, _I64, _P],
    "pyro_reactor_bdf2": [_P, _P, _P, _I64] + [_P] * 18 + [_I64, _INT, _D,
                                                          _D, _I64, _P],
    "pyro_flamelet_blocks": [_P, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P,
                             _P, _P, _I64, _P],
    "pyro_transport_info": [_P, _P],
    "pyro_species_transport": [_INT, _P, _I64, _P, _I64, _I64, _P],
    "pyro_binary_diffusivities": [_P, _I64, _P, _I64, _I64, _P],
    "pyro_transport_mixavg": [_P, _I64, _P, _I64, _P, _I64, _P, _P, _P, _I64,
                              _I64, _P],
    "pyro_flamelet_adjoint_blocks": [_P, _I64, _P, _P, _I64, _P, _P, _P, _P,
                                     _P, _P, _P, _P, _I64, _P],
    "pyro_flamelet_eos_rt": [_P, _P, _I64, _P, _P, _I64, _I64, _P],
    "pyro_flamelet_jacobian_action": [_P, _I64, _P, _P, _I64, _P, _P, _I64,
                                      _P, _P, _P, _P, _P, _P, _I64, _I64,
                                      _P],
    "pyro_flamelet_residual": [_P, _I64, _P, _P, _P, _I64, _P, _I64, _P, _P,
                               _P, _P, _P, _P, _P, _P, _P, _I64, _P, _I64,
                               _I64, _P],
}


def _is_scalar(x) -> bool:
    return getattr(x, "ndim", 0) == 0


def load_library(path: str) -> ctypes.CDLL:
    """Open a generated mechanism library and declare its C ABI."""
    lib = ctypes.CDLL(path)
    for name, args in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    return lib


def _check(status: int, what: str):
    if status != 0:
        raise RuntimeError(f"{what}: {_STATUS.get(status, status)} "
                           f"(status {status})")


class _Vec:
    """A per-state scalar on the device: pointer + increment (0 broadcasts
    one value)."""

    __slots__ = ("t", "inc", "n", "scalar")

    def __init__(self, t, inc, n, scalar):
        self.t, self.inc, self.n, self.scalar = t, inc, n, scalar

    @property
    def ptr(self):
        return self.t.data_ptr()


class CudaThermochemistryBase:
    """Base class of the generated CUDA ``Thermochemistry`` classes."""

    _lib: ctypes.CDLL = None
    _lib_path: str = ""
    _sol = None

    def __init__(self, pyro_np=None, device=None):
        if torch is None or not torch.cuda.is_available():
            raise RuntimeError(
                "pyrometheus_gb300: the CUDA Thermochemistry needs a CUDA "
                "device (there is no CPU path)")
        self.pyro_np = pyro_np if pyro_np is not None else torch
        self.device = torch.device(device if device is not None else "cuda")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        sol = self._sol
        self.model_name = getattr(sol, "source", "")
        self.num_elements = int(sol.n_elements)
        self.num_species = int(sol.n_species)
        self.num_reactions = int(sol.n_reactions)
        self.num_falloff = sum(1 for r in sol.reactions()
                               if r.reaction_type.startswith("falloff"))
        self.one_atm = one_atm
        self.gas_constant = gas_constant
        self.big_number = 1.0e300
        self.species_names = list(sol.species_names)
        self.species_indices = {n: i for i, n in
                                enumerate(self.species_names)}
        self.molecular_weights = np.array(sol.molecular_weights,
                                          dtype=np.float64)
        self.inv_molecular_weights = 1 / self.molecular_weights
        ns, nr = ctypes.c_int(), ctypes.c_int()
        _check(self._lib.pyro_mechanism_info(ctypes.byref(ns),
                                             ctypes.byref(nr), None, None,
                                             None), "mechanism_info")
        if ns.value != self.num_species or nr.value != self.num_reactions:
            raise RuntimeError("generated library does not match mechanism")
        self._fail = torch.zeros(1, dtype=torch.int32, device=self.device)
        avail = ctypes.c_int()
        _check(self._lib.pyro_transport_info(ctypes.byref(avail), None),
               "transport_info")
        self.has_transport = bool(avail.value)

    # {{{ argument plumbing

    @property
    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(
            self.device).cuda_stream)

    def _dev(self, x):
        if isinstance(x, torch.Tensor):
            t = x.to(device=self.device, dtype=torch.float64)
        else:
            t = torch.as_tensor(np.asarray(x, dtype=np.float64),
                                device=self.device)
        return t

    def _scalar_vec(self, x, n: Optional[int] = None) -> _Vec:
        t = self._dev(x)
        if t.numel() == 1:
            return _Vec(t.reshape(1).contiguous(), 0, 1, t.dim() == 0)
        t = t.reshape(-1).contiguous()
        return _Vec(t, 1, t.numel(), False)

    def _species_mat(self, y, rows: int):
        """Species-major [rows, N] device matrix; returns (tensor, n,
        single) where *single* marks a 1-D (one state) input."""
        t = self._dev(y)
        single = t.dim() == 1
        if single:
            t = t.reshape(rows, 1)
        if t.dim() != 2 or t.shape[0] != rows:
            raise ValueError(f"expected a [{rows}, N] array, got "
                             f"{tuple(t.shape)}")
        if t.stride(1) != 1 or t.stride(0) < max(1, t.shape[1]):
            t = t.contiguous()
        return t, t.shape[1], single

    @staticmethod
    def _n(*vecs):
        n = 1
        for v in vecs:
            vn = v.n if isinstance(v, _Vec) else int(v)
            if vn != 1:
                if n != 1 and vn != n:
                    raise ValueError(f"incompatible batch sizes {n} and "
                                     f"{vn}")
                n = vn
        return n

    def _expand_mat(self, m, n):
        if m.shape[1] == n:
            return m
        if m.shape[1] == 1:
            return m.expand(m.shape[0], n).contiguous()
        raise ValueError("incompatible batch sizes")

    def _out(self, rows, n):
        return torch.empty((rows, n), dtype=torch.float64, device=self.device)

    @staticmethod
    def _shape_rows(out, single):
        return out[:, 0] if single else out

    @staticmethod
    def _shape_vec(out, single):
        return out[0] if single else out

    # }}}

    # {{{ mixture and species properties (python.py:242-358)

    def get_species_name(self, species_index):
        return self.species_names[species_index]

    def get_species_index(self, species_name):
        return self.species_indices[species_name]

    def _mixture(self, which, temperature, mass_fractions, aux=None):
        y, ny, single = self._species_mat(mass_fractions, self.num_species)
        tv = self._scalar_vec(temperature) if temperature is not None \
            else None
        av = self._scalar_vec(aux) if aux is not None else None
        n = self._n(ny, *(v for v in (tv, av) if v is not None))
        y = self._expand_mat(y, n)
        out = torch.empty(n, dtype=torch.float64, device=self.device)
        _check(self._lib.pyro_mixture_property(
            MIXTURE_PROPS[which], tv.ptr if tv else None,
            tv.inc if tv else 0, y.data_ptr(), y.stride(0),
            av.ptr if av else None, av.inc if av else 0, out.data_ptr(), n,
            self._stream), f"mixture property {which}")
        single = single and (tv is None or tv.n == 1)
        return self._shape_vec(out, single)

    def get_specific_gas_constant(self, mass_fractions):
        return self._mixture("rspec", None, mass_fractions)

    def get_mixture_molecular_weight(self, mass_fractions):
        return self._mixture("mmw", None, mass_fractions)

    def get_density(self, p, temperature, mass_fractions):
        return self._mixture("density", temperature, mass_fractions, p)

    def get_pressure(self, rho, temperature, mass_fractions):
        return self._mixture("pressure", temperature, mass_fractions, rho)

    def get_mixture_specific_heat_cp_mass(self, temperature, mass_fractions):
        return self._mixture("cp", temperature, mass_fractions)

    def get_mixture_specific_heat_cv_mass(self, temperature, mass_fractions):
        return self._mixture("cv", temperature, mass_fractions)

    def get_mixture_enthalpy_mass(self, temperature, mass_fractions):
        return self._mixture("h", temperature, mass_fractions)

    def get_mixture_internal_energy_mass(self, temperature, mass_fractions):
        return self._mixture("e", temperature, mass_fractions)

    def _scale(self, which, aux, mass_fractions):
        y, ny, single = self._species_mat(mass_fractions, self.num_species)
        av = self._scalar_vec(aux)
        n = self._n(ny, av)
        y = self._expand_mat(y, n)
        out = self._out(self.num_species, n)
        _check(self._lib.pyro_species_scale(
            which, av.ptr, av.inc, y.data_ptr(), y.stride(0), out.data_ptr(),
            out.stride(0), n, self._stream), "species scale")
        return self._shape_rows(out, single and av.n == 1)

    def get_concentrations(self, rho, mass_fractions):
        return self._scale(0, rho, mass_fractions)

    def get_mole_fractions(self, mix_mol_weight, mass_fractions):
        return self._scale(1, mix_mol_weight, mass_fractions)

    def get_mass_average_property(self, mass_fractions, spec_property):
        y, _, _ = self._species_mat(mass_fractions, self.num_species)
        p, _, _ = self._species_mat(spec_property, self.num_species)
        w = torch.as_tensor(self.inv_molecular_weights, device=self.device)
        return (y * p * w[:, None]).sum(dim=0)

    def _species(self, which, temperature):
        tv = self._scalar_vec(temperature)
        n = tv.n
        out = self._out(self.num_species, n)
        _check(self._lib.pyro_species_property(
            SPECIES_PROPS[which], tv.ptr, tv.inc, out.data_ptr(),
            out.stride(0), n, self._stream), f"species property {which}")
        return self._shape_rows(out, _is_scalar(temperature))

    def get_species_specific_heats_r(self, temperature):
        return self._species("cp_r", temperature)

    def get_species_enthalpies_rt(self, temperature):
        return self._species("h_rt", temperature)

    def get_species_entropies_r(self, temperature):
        return self._species("s_r", temperature)

    def get_species_gibbs_rt(self, temperature):
        return self._species("g_rt", temperature)

    def get_species_specific_heats_r_derivative(self, temperature):
        return self._species("dcp_r", temperature)

    def get_species_enthalpies_rt_derivative(self, temperature):
        return self._species("dh_rt", temperature)

    def get_species_entropies_rt_derivative(self, temperature):
        return self._species("ds_r", temperature)

    # }}}

    # {{{ kinetics (python.py:360-562)

    def _reaction(self, mode, temperature, concentrations=None):
        tv = self._scalar_vec(temperature)
        if concentrations is not None:
            c, nc, single = self._species_mat(concentrations,
                                              self.num_species)
            n = self._n(tv, nc)
            c = self._expand_mat(c, n)
        else:
            c, n, single = None, tv.n, True
        single = single and _is_scalar(temperature)
        out = self._out(self.num_reactions, n)
        _check(self._lib.pyro_reaction_quantity(
            REACTION_MODES[mode], tv.ptr, tv.inc,
            c.data_ptr() if c is not None else None,
            c.stride(0) if c is not None else n, out.data_ptr(),
            out.stride(0), n, self._stream), f"reaction quantity {mode}")
        return self._shape_rows(out, single)

    def get_equilibrium_constants(self, temperature):
        return self._reaction("log_keq", temperature)

    def get_fwd_rate_coefficients(self, temperature, concentrations):
        return self._reaction("k_fwd", temperature, concentrations)

    def get_falloff_rates(self, temperature, concentrations, k_fwd):
        """Overwrites the falloff slots of *k_fwd* in place and returns None,
        like ``python.py:399-450``."""
        k = self._reaction("k_fwd", temperature, concentrations)
        idx = [j for j, r in enumerate(self._sol.reactions())
               if r.reaction_type.startswith("falloff")]
        for j in idx:
            k_fwd[j] = k[j]

    def get_net_rates_of_progress(self, temperature, concentrations):
        return self._reaction("net", temperature, concentrations)

    def get_fwd_rates_of_progress(self, temperature, concentrations):
        return self._reaction("fwd", temperature, concentrations)

    def get_rev_rates_of_progress(self, temperature, concentrations):
        return self._reaction("rev", temperature, concentrations)

    def get_net_production_rates(self, rho, temperature, mass_fractions):
        """``python.py:486-495`` -- the hot path."""
        y, ny, single = self._species_mat(mass_fractions, self.num_species)
        rv = self._scalar_vec(rho)
        tv = self._scalar_vec(temperature)
        n = self._n(ny, rv, tv)
        y = self._expand_mat(y, n)
        out = self._out(self.num_species, n)
        _check(self._lib.pyro_net_production_rates(
            rv.ptr, rv.inc, tv.ptr, tv.inc, y.data_ptr(), y.stride(0),
            out.data_ptr(), out.stride(0), n, self._stream),
            "net production rates")
        return self._shape_rows(out, single and n == 1)

    def get_creation_destruction_rates(self, rho, temperature,
                                       mass_fractions):
        y, ny, single = self._species_mat(mass_fractions, self.num_species)
        rv = self._scalar_vec(rho)
        tv = self._scalar_vec(temperature)
        n = self._n(ny, rv, tv)
        y = self._expand_mat(y, n)
        cd = self._out(self.num_species, n)
        dd = self._out(self.num_species, n)
        _check(self._lib.pyro_creation_destruction_rates(
            rv.ptr, rv.inc, tv.ptr, tv.inc, y.data_ptr(), y.stride(0),
            cd.data_ptr(), dd.data_ptr(), cd.stride(0), n, self._stream),
            "creation/destruction rates")
        s = single and n == 1
        return self._shape_rows(cd, s), self._shape_rows(dd, s)

    def get_creation_rates(self, rho, temperature, mass_fractions):
        return self.get_creation_destruction_rates(rho, temperature,
                                                   mass_fractions)[0]

    def get_destruction_rates(self, rho, temperature, mass_fractions):
        return self.get_creation_destruction_rates(rho, temperature,
                                                   mass_fractions)[1]

    # }}}

    # {{{ temperature (python.py:375-396; flamelets/make_pyro.py:255-299)

    def _temperature(self, target, t_guess, y, do_energy, tol, max_iter,
                     check=True):
        ym, ny, single = self._species_mat(y, self.num_species)
        ev = self._scalar_vec(target)
        tv = self._scalar_vec(t_guess)
        n = self._n(ny, ev, tv)
        ym = self._expand_mat(ym, n)
        out = torch.empty(n, dtype=torch.float64, device=self.device)
        self._fail.zero_()
        _check(self._lib.pyro_temperature(
            ev.ptr, ev.inc, tv.ptr, tv.inc, ym.data_ptr(), ym.stride(0),
            1 if do_energy else 0, float(tol), int(max_iter),
            out.data_ptr(), self._fail.data_ptr(), n, self._stream),
            "temperature")
        if check and int(self._fail.item()) > 0:
            raise RuntimeError("Temperature iteration failed to converge")
        return self._shape_vec(out, single and ev.n == 1)

    def get_temperature(self, enthalpy_or_energy, t_guess, y,
                        do_energy=False):
        return self._temperature(enthalpy_or_energy, t_guess, y, do_energy,
                                 1.0e-6, 500)

    def get_temperature_from_enthalpy(self, enthalpy, mass_fractions,
                                      temp_init):
        """Enthalpy form used by the flamelet equations
        (``flamelets/make_pyro.py:255-299``), iterated per state to
        ``|dT| < 1e-10``."""
        return self._temperature(enthalpy, temp_init, mass_fractions, False,
                                 1.0e-10, 500)

    # }}}

    # {{{ fused state step

    def get_net_production_rates_and_temperature(
            self, pressure, temperature, mass_fractions, energy, t_guess,
            do_energy=True, check=True, out=None, chunk=None):
        """One pass per state of ``rho = get_density(p, T, Y)``,
        ``get_net_production_rates(rho, T, Y)`` and
        ``get_temperature(energy, t_guess, Y, do_energy)``.

        With host (CPU, preferably pinned) torch tensors for ``pressure``,
        ``temperature``, ``energy`` ([N]) and ``mass_fractions`` ([S, N]) and
        ``out = (wdot_host[S, N], T_host[N])``, the batch is streamed in
        chunks of *chunk* states (default: the whole waves of the hot kernel
        nearest 2^17 states): host-to-device copies, the kernel and
        device-to-host copies of successive chunks run on three streams
        with three device chunk buffers, so the transfers overlap the
        FP64 work.  Results land in *out*.

        :returns: ``(wdot[S, N], T_new[N])`` (the *out* tensors when given).
        """
        if out is not None:
            return self._fused_streamed(pressure, temperature, mass_fractions,
                                        energy, t_guess, do_energy, check,
                                        out, chunk)
        ym, ny, single = self._species_mat(mass_fractions, self.num_species)
        pv = self._scalar_vec(pressure)
        tv = self._scalar_vec(temperature)
        ev = self._scalar_vec(energy)
        gv = self._scalar_vec(t_guess)
        n = self._n(ny, pv, tv, ev, gv)
        ym = self._expand_mat(ym, n)
        wdot = self._out(self.num_species, n)
        tout = torch.empty(n, dtype=torch.float64, device=self.device)
        self._fail.zero_()
        _check(self._lib.pyro_fused_step(
            pv.ptr, pv.inc, tv.ptr, tv.inc, ym.data_ptr(), ym.stride(0),
            ev.ptr, ev.inc, gv.ptr, gv.inc, 1 if do_energy else 0, 1.0e-6,
            500, wdot.data_ptr(), wdot.stride(0), tout.data_ptr(),
            self._fail.data_ptr(), n, self._stream), "fused step")
        if check and int(self._fail.item()) > 0:
            raise RuntimeError("Temperature iteration failed to converge")
        return wdot, tout

    def _fused_streamed(self, p, t, y, e, t_guess, do_energy, check, out,
                        chunk):
        from . import native
        host = [x for x in (p, t, y, e)]
        if not all(isinstance(x, torch.Tensor) and x.device.type == "cpu"
                   and x.dtype == torch.float64 for x in host):
            raise ValueError("streamed fused step: p, T, Y, e must be CPU "
                             "float64 tensors")
        out_w, out_t = out
        S = self.num_species
        n = int(y.shape[1])
        if y.shape[0] != S or out_w.shape != (S, n) or out_t.shape != (n,):
            raise ValueError("streamed fused step: shape mismatch")
        for x in (p, t, e, out_t):
            if x.shape != (n,) or x.stride(0) != 1:
                raise ValueError("streamed fused step: [N] inputs must be "
                                 "contiguous")
        if y.stride(1) != 1 or out_w.stride(1) != 1:
            raise ValueError("streamed fused step: [S, N] arrays must have "
                             "unit column stride")
        if n == 0:
            return out_w, out_t
        tg = self._scalar_vec(t_guess)
        if tg.n != 1:
            raise ValueError("streamed fused step: t_guess must be a scalar")
        dev = self.device
        comp = torch.cuda.current_stream(dev)
        if getattr(self, "_copy_streams", None) is None:
            self._copy_streams = (torch.cuda.Stream(dev),
                                  torch.cuda.Stream(dev))
        h2d, d2h = self._copy_streams
        if chunk is None:
            wave = self._lib.pyro_hot_block_size() * torch.cuda.\
                get_device_properties(dev).multi_processor_count
            chunk = max(1, round((1 << 17) / wave)) * wave
        m0 = int(min(chunk, n))
        # three device chunks (the copies of one run ahead of the kernel on
        # another, so a slow transfer does not stall the pipeline), kept
        # allocated between calls (keyed by the chunk size): a fresh
        # allocation per call, held back by the copy streams until they
        # drain, sent some calls through device allocations that stalled
        # the pipeline; successive calls are ordered on the streams (each
        # starts after the last one's copies)
        bufs = self._stream_bufs.get(m0) if getattr(
            self, "_stream_bufs", None) is not None else None
        if bufs is None:
            f64 = dict(dtype=torch.float64, device=dev)
            bufs = []
            for _ in range(3):
                b = {"p": torch.empty(m0, **f64), "t": torch.empty(m0, **f64),
                     "e": torch.empty(m0, **f64),
                     "y": torch.empty((S, m0), **f64),
                     "w": torch.empty((S, m0), **f64),
                     "to": torch.empty(m0, **f64)}
                b["ready"] = torch.cuda.Event()
                b["done"] = torch.cuda.Event()
                b["free"] = torch.cuda.Event()
                bufs.append(b)
            self._stream_bufs = {m0: bufs}
        self._fail.zero_()
        h2d.wait_stream(comp)
        h2d.wait_stream(d2h)  # the previous call's reads of the chunks
        for c, s0 in enumerate(range(0, n, m0)):
            m = min(m0, n - s0)
            b = bufs[c % len(bufs)]
            if c >= len(bufs):
                h2d.wait_event(b["free"])
            for key, src in (("p", p), ("t", t), ("e", e), ("y", y)):
                native.copy_columns_async(b[key], src, 0, s0, m, h2d)
            b["ready"].record(h2d)
            comp.wait_event(b["ready"])
            _check(self._lib.pyro_fused_step(
                b["p"].data_ptr(), 1, b["t"].data_ptr(), 1,
                b["y"].data_ptr(), m0, b["e"].data_ptr(), 1, tg.ptr, tg.inc,
                1 if do_energy else 0, 1.0e-6, 500, b["w"].data_ptr(), m0,
                b["to"].data_ptr(), self._fail.data_ptr(), m,
                ctypes.c_void_p(comp.cuda_stream)), "fused step")
            b["done"].record(comp)
            d2h.wait_event(b["done"])
            native.copy_columns_async(out_w, b["w"], s0, 0, m, d2h)
            native.copy_columns_async(out_t, b["to"], s0, 0, m, d2h)
            b["free"].record(d2h)
        comp.wait_stream(d2h)
        if check and int(self._fail.item()) > 0:
            raise RuntimeError("Temperature iteration failed to converge")
        return out_w, out_t

    # }}}

    # {{{ mixture-averaged transport (python.py:564-641)

    def _need_transport(self):
        if not self.has_transport:
            raise ValueError(f"mechanism '{self.model_name}' has no transport"
                             " fits")

    def _species_transport(self, which, temperature):
        self._need_transport()
        tv = self._scalar_vec(temperature)
        out = self._out(self.num_species, tv.n)
        _check(self._lib.pyro_species_transport(
            which, tv.ptr, tv.inc, out.data_ptr(), out.stride(0), tv.n,
            self._stream), "species transport")
        return self._shape_rows(out, _is_scalar(temperature))

    def get_species_viscosities(self, temperature):
        """``sqrt(T) P_k(ln T)^2`` ([S, N]) -- python.py:564-571."""
        return self._species_transport(0, temperature)

    def get_species_thermal_conductivities(self, temperature):
        """``sqrt(T) Q_k(ln T)`` ([S, N]) -- python.py:573-580."""
        return self._species_transport(1, temperature)

    def get_species_binary_mass_diffusivities(self, temperature):
        """``sqrt(T) T R_ij(ln T)`` ([S, S, N]) -- python.py:582-593."""
        self._need_transport()
        tv = self._scalar_vec(temperature)
        S = self.num_species
        out = torch.empty((S, S, tv.n), dtype=torch.float64,
                          device=self.device)
        _check(self._lib.pyro_binary_diffusivities(
            tv.ptr, tv.inc, out.data_ptr(), tv.n, tv.n, self._stream),
            "binary diffusivities")
        return out[:, :, 0] if _is_scalar(temperature) else out

    def _mixavg(self, pressure, temperature, mass_fractions, want_mu,
                want_lam, want_d):
        self._need_transport()
        ym, ny, single = self._species_mat(mass_fractions, self.num_species)
        tv = self._scalar_vec(temperature)
        pv = self._scalar_vec(pressure) if want_d else None
        n = self._n(ny, tv, *((pv,) if pv is not None else ()))
        ym = self._expand_mat(ym, n)
        mu = torch.empty(n, dtype=torch.float64, device=self.device) \
            if want_mu else None
        lam = torch.empty(n, dtype=torch.float64, device=self.device) \
            if want_lam else None
        d = self._out(self.num_species, n) if want_d else None
        _check(self._lib.pyro_transport_mixavg(
            pv.ptr if pv else None, pv.inc if pv else 0, tv.ptr, tv.inc,
            ym.data_ptr(), ym.stride(0),
            mu.data_ptr() if mu is not None else None,
            lam.data_ptr() if lam is not None else None,
            d.data_ptr() if d is not None else None,
            d.stride(0) if d is not None else n, n, self._stream),
            "mixture-averaged transport")
        single = single and n == 1
        return (None if mu is None else self._shape_vec(mu, single),
                None if lam is None else self._shape_vec(lam, single),
                None if d is None else self._shape_rows(d, single))

    def get_mixture_viscosity_mixavg(self, temperature, mass_fractions):
        """Wilke's mixture rule ([N]) -- python.py:595-605."""
        return self._mixavg(None, temperature, mass_fractions, True, False,
                            False)[0]

    def get_mixture_thermal_conductivity_mixavg(self, temperature,
                                                mass_fractions):
        """``(sum x lam + 1 / sum x/lam) / 2`` ([N]) -- python.py:607-613."""
        return self._mixavg(None, temperature, mass_fractions, False, True,
                            False)[1]

    def get_species_mass_diffusivities_mixavg(self, pressure, temperature,
                                              mass_fractions):
        """Mixture-averaged diffusivities ([S, N]) -- python.py:615-641."""
        return self._mixavg(pressure, temperature, mass_fractions, False,
                            False, True)[2]

    def get_transport_mixavg(self, pressure, temperature, mass_fractions):
        """``(viscosity [N], conductivity [N], diffusivities [S, N])`` in
        one pass over the states (the three mixture methods above)."""
        return self._mixavg(pressure, temperature, mass_fractions, True,
                            True, True)

    # }}}

    # {{{ constant-pressure reactor source, Jacobian and VJP

    def _reactor_args(self, pressure, temperature, mass_fractions):
        ym, ny, single = self._species_mat(mass_fractions, self.num_species)
        pv = self._scalar_vec(pressure)
        tv = self._scalar_vec(temperature)
        n = self._n(ny, pv, tv)
        return pv, tv, self._expand_mat(ym, n), n, single

    def get_reactor_source(self, pressure, temperature, mass_fractions):
        """``[dT/dt, dY_1/dt, ...]`` ([S+1, N]) of an adiabatic
        constant-pressure reactor: ``dY_k/dt = W_k w_k / rho``,
        ``dT/dt = -sum_k H_k w_k / (rho cp)`` -- the right-hand side the
        reference's reactors differentiate
        (``examples/free_flame/reactors.py:115-125``)."""
        pv, tv, ym, n, single = self._reactor_args(pressure, temperature,
                                                   mass_fractions)
        out = self._out(self.num_species + 1, n)
        _check(self._lib.pyro_reactor_source(
            pv.ptr, pv.inc, tv.ptr, tv.inc, ym.data_ptr(), ym.stride(0),
            out.data_ptr(), out.stride(0), n, self._stream), "reactor source")
        return self._shape_rows(out, single and n == 1)

    def get_reactor_source_dp(self, pressure, temperature, mass_fractions):
        """``d[dT/dt, dY/dt]/dp`` ([S+1, N]) at fixed temperature and mass
        fractions, in forward mode from the homogeneity of the mass-action
        rates in the concentrations and [M] (the pressure derivative the
        reference takes with ``jacfwd``,
        ``flamelets/equations.py:130-134``)."""
        pv, tv, ym, n, single = self._reactor_args(pressure, temperature,
                                                   mass_fractions)
        out = self._out(self.num_species + 1, n)
        _check(self._lib.pyro_reactor_source_dp(
            pv.ptr, pv.inc, tv.ptr, tv.inc, ym.data_ptr(), ym.stride(0),
            out.data_ptr(), out.stride(0), n, self._stream),
            "reactor source pressure derivative")
        return self._shape_rows(out, single and n == 1)

    def get_reactor_jacobian(self, pressure, temperature, mass_fractions,
                             out=None):
        """Jacobian ``d[dT/dt, dY/dt] / d[T, Y]`` per state, ``[N, S+1,
        S+1]`` (row-major per state), by the analytic warp-per-state
        kernel."""
        pv, tv, ym, n, single = self._reactor_args(pressure, temperature,
                                                   mass_fractions)
        nc = self.num_species + 1
        if out is None:
            out = torch.empty((n, nc, nc), dtype=torch.float64,
                              device=self.device)
        if (tuple(out.shape) != (n, nc, nc) or out.stride(2) != 1
                or out.stride(1) != nc):
            raise ValueError("out must be a [N, S+1, S+1] row-major tensor")
        _check(self._lib.pyro_reactor_jacobian(
            pv.ptr, pv.inc, tv.ptr, tv.inc, ym.data_ptr(), ym.stride(0),
            out.data_ptr(), out.stride(0) if n > 1 else nc * nc, n,
            self._stream), "reactor Jacobian")
        return out[0] if single and n == 1 else out

    def get_reactor_source_and_jacobian(self, pressure, temperature,
                                        mass_fractions, out=None):
        """``(f, J)``: the reactor source ``[S+1, N]`` (as
        :meth:`get_reactor_source`) and its Jacobian ``[N, S+1, S+1]`` (as
        :meth:`get_reactor_jacobian`) from one pass of the Jacobian kernel
        -- the primal and tangents ``jax.jacfwd`` yields together
        (``flamelets/equations.py:124-129``).  *out*: optional ``(f, J)``
        tensors to fill (``f`` with unit stride along N)."""
        pv, tv, ym, n, single = self._reactor_args(pressure, temperature,
                                                   mass_fractions)
        nc = self.num_species + 1
        if out is None:
            f = self._out(nc, n)
            jac = torch.empty((n, nc, nc), dtype=torch.float64,
                              device=self.device)
        else:
            f, jac = out
        if (tuple(jac.shape) != (n, nc, nc) or jac.stride(2) != 1
                or jac.stride(1) != nc):
            raise ValueError("J must be a [N, S+1, S+1] row-major tensor")
        if tuple(f.shape) != (nc, n) or f.stride(1) != 1:
            raise ValueError("f must be a [S+1, N] tensor with unit stride "
                             "along N")
        _check(self._lib.pyro_reactor_source_jacobian(
            pv.ptr, pv.inc, tv.ptr, tv.inc, ym.data_ptr(), ym.stride(0),
            f.data_ptr(), max(f.stride(0), n), jac.data_ptr(),
            jac.stride(0) if n > 1 else nc * nc, n, self._stream),
            "reactor source and Jacobian")
        if single and n == 1:
            return self._shape_rows(f, True), jac[0]
        return f, jac

    def get_reactor_vjp(self, pressure, temperature, mass_fractions,
                        cotangent):
        """``v^T df/dx`` for cotangents ``v`` ([S+1, N]) without forming
        the Jacobian; returns ``(g_T[N], g_Y[S, N], g_p[N])``."""
        pv, tv, ym, n, single = self._reactor_args(pressure, temperature,
                                                   mass_fractions)
        v, nv, _ = self._species_mat(cotangent, self.num_species + 1)
        v = self._expand_mat(v, n)
        gT = torch.empty(n, dtype=torch.float64, device=self.device)
        gY = self._out(self.num_species, n)
        gp = torch.empty(n, dtype=torch.float64, device=self.device)
        _check(self._lib.pyro_reactor_vjp(
            pv.ptr, pv.inc, tv.ptr, tv.inc, ym.data_ptr(), ym.stride(0),
            v.data_ptr(), v.stride(0), gT.data_ptr(), gY.data_ptr(),
            gY.stride(0), gp.data_ptr(), n, self._stream), "reactor VJP")
        return gT, gY, gp

    def reactor_source(self, pressure, temperature, mass_fractions):
        """Differentiable reactor source: a ``torch.autograd.Function``
        whose backward is the VJP kernel (gradients for p, T and Y)."""
        return ReactorSource.apply(self, self._dev(pressure),
                                   self._dev(temperature),
                                   self._dev(mass_fractions))

    # }}}


if torch is not None:
    class ReactorSource(torch.autograd.Function):
        """f = (dT/dt, dY/dt) of the constant-pressure reactor with a
        hand-written VJP backward (``k_reactor_vjp``)."""

        @staticmethod
        def forward(ctx, thermo, p, t, y):
            ctx.thermo = thermo
            ctx.save_for_backward(p, t, y)
            return thermo.get_reactor_source(p, t, y)

        @staticmethod
        def backward(ctx, grad):
            p, t, y = ctx.saved_tensors
            th = ctx.thermo
            g = grad.reshape(th.num_species + 1, -1)
            gT, gY, gp = th.get_reactor_vjp(p, t, y, g)
            gp_out = gp.reshape(p.shape) if p.numel() > 1 else gp.sum(
            ).reshape(p.shape)
            gT_out = gT.reshape(t.shape) if t.numel() > 1 else gT.sum(
            ).reshape(t.shape)
            return None, gp_out, gT_out, gY.reshape(y.shape)


def make_thermochem_class(sol, lib_path: str, name: str = "Thermochemistry"):
    """A ``Thermochemistry`` class bound to the compiled library."""
    lib = load_library(lib_path)
    return type(name, (CudaThermochemistryBase,),
                {"_lib": lib, "_lib_path": lib_path, "_sol": sol,
                 "__doc__": f"CUDA thermochemistry for {sol.n_species} "
                            f"species / {sol.n_reactions} reactions."})

# vim: foldmethod=marker
