"""CPU backend for the reactor integrator, built on the numpy oracle.

TEST INFRASTRUCTURE ONLY.  Used by ``tests/`` (to check the integrator's
step control, Newton and bookkeeping on the CPU against SciPy) and by
``bench.py``'s CPU baseline leg (the same integrator on the oracle, timed on
the host cores).  The CUDA product never imports it.

It supplies the interface ``ReactorPool`` expects -- ``source``,
``jacobian``, ``lu_factor``, ``lu_solve`` and ``wrms`` on float64 CPU
tensors -- from ``Thermochemistry.reactor_source`` (the constant-pressure
reactor right-hand side of ``examples/free_flame/reactors.py:115-123``),
its central-difference Jacobian, and LAPACK's getrf/getrs through SciPy
(the factorisation behind the reference's ``jnp.linalg.solve``,
``examples/free_flame/time_integ.py:94``).
"""

from __future__ import annotations

import numpy as np
import scipy.linalg
import torch

from .thermo_oracle import Thermochemistry


class OracleReactorBackend:
    def __init__(self, sol, fd_rel: float = 1e-7):
        self.orc = Thermochemistry(sol)
        self.num_species = sol.n_species
        self.device = "cpu"
        self.fd_rel = float(fd_rel)

    @staticmethod
    def _np(x):
        return x.detach().cpu().numpy() if torch.is_tensor(x) else \
            np.asarray(x)

    def source(self, p, T, Y):
        f = self.orc.reactor_source(self._np(p), self._np(T), self._np(Y))
        return torch.from_numpy(np.ascontiguousarray(f))

    def jacobian(self, p, T, Y, out):
        j = self.orc.reactor_jacobian_fd(self._np(p), self._np(T),
                                         self._np(Y), rel=self.fd_rel)
        out.copy_(torch.from_numpy(j))

    def lu_factor(self, M, piv, mask, status):
        m = self._np(mask).astype(bool)
        for s in np.nonzero(m)[0]:
            lu, pv = scipy.linalg.lu_factor(M[s].numpy(), check_finite=False)
            if not np.all(np.isfinite(lu)) or np.any(np.diag(lu) == 0):
                status |= 1
            M[s] = torch.from_numpy(lu)
            piv[s] = torch.from_numpy(pv.astype(np.int32))

    def lu_solve(self, M, piv, mask, rhs, out):
        m = self._np(mask).astype(bool)
        for s in np.nonzero(m)[0]:
            x = scipy.linalg.lu_solve((M[s].numpy(), piv[s].numpy()),
                                      rhs[:, s].numpy(), check_finite=False)
            out[:, s] = torch.from_numpy(x)

    def wrms(self, v, w, out):
        q = (v / w).numpy()
        out.copy_(torch.from_numpy(np.sqrt((q * q).sum(axis=0)
                                           / q.shape[0])))
        return out
