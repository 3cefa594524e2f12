"""Shared inputs of the flamelet-solver tests: seeded flamelets of the
9-species benchmark mechanism with slow chemistry (every rate coefficient
times 1e-12), chosen so that one batch exercises each branch of the
reference driver (``pyrometheus/flamelets/solver.py:476-600``): the first
steady Newton converges; it diverges and a time march rescues it; or no
round converges.  The boundary dissipation rate is ``2 dx^2`` (Dirichlet
rows, ``equations.py:150-165``), the viscous dissipation zero.

Also an adapter giving the oracle the interface of
``pyrometheus_gb300.flamelet.FlameletEquations`` (CPU torch tensors, one
flamelet at a time), so the batched driver can run on the oracle pieces."""

import numpy as np
import torch

from oracle.block_thomas_oracle import solve_packed
from oracle.flamelet_oracle import FlameletOracle
from oracle.thermo_oracle import Thermochemistry
from pyrometheus_gb300 import synthetic

# (grid points, peak dissipation rate, profile seed, linear enthalpy guess)
FLAMELETS = [(12, 100.0, 1, False), (12, 10.0, 1, False),
             (12, 10.0, 1, True), (9, 1000.0, 5, False)]
PRESSURE = 101325.0
SOLVE = dict(newton_maxiter=10, newton_tol=1e-8, bdf_newton_maxiter=20,
             bdf_newton_tol=1e-9, bdf_time_step=1e-5, bdf_maxsteps=10,
             try_newton=True, max_attempts=3)


def mechanism():
    return synthetic.scaled_rates(synthetic.config1_mechanism(), 1e-12)


def flamelet_batch(sol, flamelets=FLAMELETS):
    """Packed inputs: lengths, dx, y_ox, y_fu, phi [S+1, rows], chi, visc,
    T guess (all numpy), h_ox, h_fu per flamelet."""
    th = Thermochemistry(sol)
    out = dict(lengths=[], dx=[], phi=[], chi=[], T=[], h_ox=[], h_fu=[])
    for n, chi_max, seed, linear in flamelets:
        prof = synthetic.flamelet_profiles(sol, [n], seed=seed,
                                           chi_max=chi_max)
        dx = float(prof["dx"][0])
        chi = prof["chi"].copy()
        chi[0] = chi[-1] = 2.0 * dx ** 2
        T, Y = prof["T"], prof["Y"]
        h = th.get_mixture_enthalpy_mass(T, Y)
        if linear:
            z = np.linspace(0.0, 1.0, n)
            h = (1.0 - z) * h[0] + z * h[-1]
        out["lengths"].append(n)
        out["dx"].append(dx)
        out["phi"].append(np.vstack([h, Y]))
        out["chi"].append(chi)
        out["T"].append(T)
        out["h_ox"].append(h[0])
        out["h_fu"].append(h[-1])
        y_ox, y_fu = prof["y_ox"], prof["y_fu"]
    res = {k: (np.hstack(v) if k == "phi" else np.concatenate(v)
               if k in ("chi", "T") else np.asarray(v))
           for k, v in out.items()}
    res["visc"] = np.zeros_like(res["chi"])
    res["y_ox"], res["y_fu"] = y_ox, y_fu
    return res


def split(x, lengths):
    offs = np.concatenate([[0], np.cumsum(lengths)])
    return [x[..., offs[s]:offs[s + 1]] for s in range(len(lengths))]


class OracleSolver:
    def __init__(self, lengths):
        self.lengths = lengths

    def solve(self, L, C, U, b, out=None):
        x = solve_packed(self.lengths, L.numpy(), C.numpy(), U.numpy(),
                         b.numpy())
        return torch.as_tensor(x)


class OracleEquations:
    """``FlameletEquations``' interface on the CPU oracle, flamelet by
    flamelet (the oracle's temperature iteration is batch-wide, so each
    flamelet is evaluated on its own, as the single-flamelet oracle driver
    does)."""

    def __init__(self, sol, lengths, dx, y_ox, y_fu):
        self.sol = sol
        self.fo = FlameletOracle(sol)
        self.S = sol.n_species
        self.nv = self.S + 1
        self.lengths = np.asarray(lengths, dtype=np.int64)
        self.nsys = len(self.lengths)
        self.rows = int(self.lengths.sum())
        self.device = torch.device("cpu")
        self.dx = np.broadcast_to(np.asarray(dx, dtype=np.float64),
                                  (self.nsys,)).copy()
        y_ox, y_fu = np.asarray(y_ox), np.asarray(y_fu)
        self.y_ox = y_ox if y_ox.ndim == 2 else np.repeat(
            y_ox[:, None], self.nsys, axis=1)
        self.y_fu = y_fu if y_fu.ndim == 2 else np.repeat(
            y_fu[:, None], self.nsys, axis=1)

    def subset(self, systems):
        return OracleEquations(self.sol, self.lengths[systems],
                               self.dx[systems], self.y_ox[:, systems],
                               self.y_fu[:, systems])

    def linear_solver(self):
        return OracleSolver(self.lengths)

    def _rows(self, x):
        x = np.asarray(x.numpy() if torch.is_tensor(x) else x,
                       dtype=np.float64)
        if x.ndim == 0:
            return [float(x)] * self.nsys
        return split(x, self.lengths)

    def temperature(self, h, Y, temp_guess, check=True):
        t = [self.fo.temperature(hs, ys, tg) for hs, ys, tg in zip(
            self._rows(h), split(Y.numpy(), self.lengths),
            self._rows(temp_guess))]
        return torch.as_tensor(np.concatenate(t))

    def rhs(self, h, Y, diss_rate, viscous_diss, temp_guess, pressure,
            h_ox, h_fu, temperature=None):
        parts = zip(self._rows(h), split(Y.numpy(), self.lengths),
                    self._rows(diss_rate), self._rows(viscous_diss),
                    self._rows(temp_guess), self._rows(pressure))
        hox = np.broadcast_to(np.asarray(h_ox), (self.nsys,))
        hfu = np.broadcast_to(np.asarray(h_fu), (self.nsys,))
        r = [self.fo.residual(hs, ys, chi, visc, tg, p, hox[s], hfu[s],
                              self.y_ox[:, s], self.y_fu[:, s], self.dx[s])
             for s, (hs, ys, chi, visc, tg, p) in enumerate(parts)]
        return torch.as_tensor(np.hstack(r))

    def jac(self, h, Y, diss_rate, viscous_diss, temp_guess, pressure,
            temperature=None, out=None):
        nv = self.nv
        L = np.zeros((self.rows, nv, nv))
        C = np.zeros((self.rows, nv, nv))
        U = np.zeros((self.rows, nv, nv))
        r0 = 0
        for s, (hs, ys, chi, visc, tg, p) in enumerate(zip(
                self._rows(h), split(Y.numpy(), self.lengths),
                self._rows(diss_rate), self._rows(viscous_diss),
                self._rows(temp_guess), self._rows(pressure))):
            n = len(hs)
            sj = self.fo.source_jacobian_fd(hs, ys, visc, tg, p)
            lo, c, up = self.fo.blocks(sj, chi, self.dx[s])
            L[r0:r0 + n - 1], C[r0:r0 + n], U[r0:r0 + n - 1] = lo, c, up
            r0 += n
        return torch.as_tensor(L), torch.as_tensor(C), torch.as_tensor(U)

    # the compressible-EOS pieces, flamelet by flamelet

    def _parts(self, h, Y, *rowvecs):
        return zip(range(self.nsys), self._rows(h),
                   split(Y.numpy(), self.lengths),
                   *(self._rows(x) for x in rowvecs))

    def eos_rt(self, h, Y, temp_guess=None, temperature=None,
               jacobian=True):
        assert not jacobian
        rt = [self.fo.eos_rt(hs, ys, tg)
              for _, hs, ys, tg in self._parts(h, Y, temp_guess)]
        return torch.as_tensor(np.concatenate(rt)), None

    def enthalpy_gradient(self, h, Y, diss_rate, viscous_diss, temp_guess,
                          pressure, pdf):
        rts, adjs, gs = [], [], []
        for s, hs, ys, chi, visc, tg, p, w in self._parts(
                h, Y, diss_rate, viscous_diss, temp_guess, pressure, pdf):
            p = float(np.asarray(p).ravel()[0])
            rts.append(self.fo.eos_rt(hs, ys, tg))
            sj = self.fo.source_jacobian_fd(hs, ys, visc, tg, p)
            adj, g = self.fo.enthalpy_gradient(sj, chi, self.dx[s], w)
            adjs.append(adj)
            gs.append(g)
        return (torch.as_tensor(np.concatenate(rts)),
                torch.as_tensor(np.hstack(adjs)), torch.as_tensor(gs))

    def eos_gradient(self, h, Y, diss_rate, viscous_diss, temp_guess,
                     pressure, pdf):
        fo = self.fo
        dgs, egs, ads, aes = [], [], [], []
        for s, hs, ys, chi, visc, tg, p, w in self._parts(
                h, Y, diss_rate, viscous_diss, temp_guess, pressure, pdf):
            p = float(np.asarray(p).ravel()[0])
            rt = fo.eos_rt(hs, ys, tg)
            rtj = fo.eos_rt_jacobian_fd(hs, ys, tg)
            dsdp = fo.source_pressure_gradient_fd(hs, ys, visc, tg, p)
            sj = fo.source_jacobian_fd(hs, ys, visc, tg, p)
            (dg, eg), (ad, ae) = fo.eos_gradient(sj, rt, rtj, dsdp, chi,
                                                 self.dx[s], w, p)
            dgs.append(dg)
            egs.append(eg)
            ads.append(ad)
            aes.append(ae)
        t = torch.as_tensor
        return ((t(np.stack(dgs, axis=1)), t(np.stack(egs, axis=1))),
                (t(np.hstack(ads)), t(np.hstack(aes))))


# compressible-EOS consistency: two flamelets whose steady Newton converges,
# targets from their solutions at (PRESSURE, h_ox, h_fu), iterations
# started 10 % off in pressure
EOS_FLAMELETS = [FLAMELETS[0], FLAMELETS[3]]


def eos_config(method, maxiter=3, tol=1e-12):
    return dict(verbosity=False,
                newton=dict(maxiter=SOLVE["newton_maxiter"],
                            tol=SOLVE["newton_tol"]),
                bdf=dict(newton=dict(maxiter=SOLVE["bdf_newton_maxiter"],
                                     tol=SOLVE["bdf_newton_tol"]),
                         time_step=SOLVE["bdf_time_step"],
                         maxsteps=SOLVE["bdf_maxsteps"]),
                max_attempts=SOLVE["max_attempts"],
                eos=dict(update_size=1.0, update_method=method,
                         maxiter=maxiter, tol=tol))


def eos_case(sol, b):
    """Per-flamelet PDF weights [rows], true params [3, n], start params
    [3, n] and the targets (density, energy) [n] of the true params (from
    the oracle)."""
    from oracle.eos_consistency_oracle import CompressibleEOSOracle
    n = b["lengths"]
    pdfs, rho, e = [], [], []
    true = np.stack([np.full(len(n), PRESSURE), b["h_ox"], b["h_fu"]])
    for s, (phi0, chi, visc, tg) in enumerate(zip(
            split(b["phi"], n), split(b["chi"], n), split(b["visc"], n),
            split(b["T"], n))):
        z = np.linspace(0.0, 1.0, n[s])
        pdf = 1e-3 + z ** 1.5 * (1.0 - z) ** 2.5
        pdfs.append(pdf / pdf.sum())
        orc = CompressibleEOSOracle(sol, b["dx"][s], b["y_ox"], b["y_fu"],
                                    eos_config("gauss_newton"))
        out = orc.evaluate_flamelet(true[:, s], pdfs[-1], chi, visc, tg,
                                    phi0)
        rho.append(out[2])
        e.append(out[3])
    start = true.copy()
    start[0] *= 1.1
    return np.concatenate(pdfs), true, start, np.array(rho), np.array(e)
