// Fused per-cell implicit integrator of the adiabatic constant-pressure 0-D
// reactor (FP64, sm_103a): one thread integrates one cell for up to
// `attempts` step attempts per launch, entirely on the device.
//
// The reference steps one reactor at a time from Python (Crank-Nicolson,
// a Newton loop that re-forms the JAX Jacobian and calls jnp.linalg.solve
// each iteration: examples/free_flame/time_integ.py:70-106).  The serving
// pool (pyrometheus_gb300/serving.py) runs the same variable-step BDF2 /
// chord-Newton algorithm either as batched tensor operations, one step
// attempt per engine step, or through this kernel, which keeps every
// per-cell decision (Jacobian refresh, refactorisation, Newton
// convergence, error test, step size) inside the thread that owns the
// cell, so hundreds of attempts cost one launch.
//
// Per cell (same arithmetic as the batched path apart from the Jacobian):
//   predictor  z_p = y + h (f_n + c h),  c = (y_{n-1} - y + f_n h_{n-1}) /
//              h_{n-1}^2  (explicit Euler on the first, backward-Euler step)
//   corrector  z - (a y + b y_{n-1}) - gamma f(z) = 0 by chord Newton with
//              M = I - gamma J factorised (partial pivoting) when J is
//              refreshed or gamma moved by more than 30 %
//   Jacobian   forward differences at z_p (one source evaluation per
//              column, step sqrt(eps) max(|z_j|, 1e-8)), refreshed on
//              admission, after a Newton failure and every 20 accepted steps
//   error      (1 + w) / (3 w + 2) wrms(z - z_p)  (1/2 on the first step)
// with weights rtol |y| + atol and a fixed summation order, so a cell's
// result depends on its own data only.
//
// Layout: vectors species-major [NS+1][ld] (y, y_prev, f_n), scalars [ld],
// the Jacobian and the factored Newton matrix element-major
// [(NS+1)^2][ld] and the pivots [NS+1][ld], so the threads of a warp (32
// consecutive cells) touch 32 consecutive doubles of each element.  Each
// thread's working vectors (state, source, correction and the source's
// concentrations / Gibbs energies / rates) are shared-memory columns
// interleaved by thread.  No thread waits on another.
#pragma once

#ifndef IBLOCK
#define IBLOCK 64
#endif
#define INV (NS + 1)

namespace pyro {

using ICols = ColsT<IBLOCK>;

__device__ __forceinline__ ICols icol(double* smem, int off) {
  return ICols{smem + (size_t)off * IBLOCK + threadIdx.x};
}

// f = reactor source at x = (T, Y) (k_reactor_source's arithmetic).
__device__ __forceinline__ void cell_rhs(double P, ICols X, ICols F, ICols c,
                                         ICols g, ICols w) {
  const double T = X[0];
  double sigma = 0.0, cpp = 0.0;
  for (int k = 0; k < NS; ++k) {
    const double wk = X[k + 1] * k_inv_mw[k];
    sigma += wk;
    const Nasa a(k, T > k_tmid[k]);
    cpp = fma(wk,
              fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]),
              cpp);
  }
  const double rho = P / (GAS_CONSTANT * T * sigma);
  const double invT = 1.0 / T;
#if defined(PYRO_UNROLLED) && defined(PYRO_BDF2_UNROLLED)
  // straight-line rates (small mechanisms): accumulators in registers
  struct ColY {
    ICols X;
    __device__ __forceinline__ double operator()(int k) const {
      return X[k + 1];
    }
  };
  double wd[NS];
  pyro_unrolled::net_rates_y(T, rho, ColY{X}, c, g, w, wd);
#pragma unroll
  for (int k = 0; k < NS; ++k) w[k] = wd[k];
#else
  StateScalars s;
  s.T = T;
  s.lnT = log(T);
  s.invT = invT;
  s.c0 = LOG_P0_OVER_R - s.lnT;
  double ctot = 0.0;
  for (int k = 0; k < NS; ++k) {
    const double v = k_inv_mw[k] * rho * X[k + 1];
    c[k] = v;
    ctot += v;
  }
  s.ctot = ctot;
  production_rates(s, c, g, w);
#endif
  double q = 0.0;
  for (int k = 0; k < NS; ++k) {
    const Nasa a(k, T > k_tmid[k]);
    const double hrt =
        fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                          a[2] * (1.0 / 3.0)),
                  a[1] * 0.5),
            a[0]) +
        a[5] * invT;
    q = fma(GAS_CONSTANT * T * hrt, w[k], q);
    F[k + 1] = k_mw[k] * w[k] / rho;
  }
  F[0] = -q / (rho * GAS_CONSTANT * cpp);
}

}  // namespace pyro

// Device-side BDF2 integration of cells [0, n), or of the n cells listed in
// Slots (the pool's active cells, so every thread has a cell; inactive
// cells are skipped either way).
// done[i] is set when cell i finished (reached t_end or failed) in this
// launch; failed[i] marks a failure.
__global__ void __launch_bounds__(IBLOCK)
    k_reactor_bdf2(double* __restrict__ Yv, double* __restrict__ Ypv,
                   double* __restrict__ Fnv, int64_t ld,
                   const double* __restrict__ Pp, double* __restrict__ Tt,
                   const double* __restrict__ Te, double* __restrict__ Hh,
                   double* __restrict__ Hp, double* __restrict__ Glu,
                   double* __restrict__ Crate, int64_t* __restrict__ Nsteps,
                   int64_t* __restrict__ Natt, int64_t* __restrict__ Jage,
                   unsigned char* __restrict__ Active,
                   unsigned char* __restrict__ Failed,
                   unsigned char* __restrict__ Jstale,
                   unsigned char* __restrict__ Done, double* __restrict__ Jm,
                   double* __restrict__ Mm, int* __restrict__ Piv,
                   const int64_t* __restrict__ Slots, int64_t n,
                   int attempts, double rtol, double atol,
                   int64_t max_attempts) {
  extern __shared__ double smem[];
  PEXP_PRELOAD();
#if defined(PYRO_UNROLLED) && defined(PYRO_BDF2_UNROLLED)
  PYRO_LOG_PRELOAD();
#endif
  using pyro::ICols;
  const ICols c = pyro::icol(smem, 0), g = pyro::icol(smem, NS),
              w = pyro::icol(smem, 2 * NS);
  const ICols Z = pyro::icol(smem, 3 * NS), F = pyro::icol(smem, 3 * NS + INV),
              DZ = pyro::icol(smem, 3 * NS + 2 * INV),
              X1 = pyro::icol(smem, 3 * NS + 3 * INV);
#define VY(j) Yv[(int64_t)(j) * ld + i]
#define VYP(j) Ypv[(int64_t)(j) * ld + i]
#define VFN(j) Fnv[(int64_t)(j) * ld + i]
#define EJ(r, q) Jm[((int64_t)(r) * INV + (q)) * ld + i]
#define EM(r, q) Mm[((int64_t)(r) * INV + (q)) * ld + i]
#define EP(r) Piv[(int64_t)(r) * ld + i]
  for (int64_t q = (int64_t)blockIdx.x * IBLOCK + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * IBLOCK) {
    const int64_t i = Slots ? Slots[q] : q;
    if (!Active[i]) continue;
    const double P = Pp[i], te = Te[i];
    double t = Tt[i], h = Hh[i], hp = Hp[i], glu = Glu[i], crate = Crate[i];
    int64_t nsteps = Nsteps[i], natt = Natt[i], jage = Jage[i];
    bool jstale = Jstale[i] != 0, failed = false, finished = false;
    for (int att = 0; att < attempts; ++att) {
      const double hu = fmin(h, te - t);
      const bool first = nsteps == 0;
      const double om = first ? 0.0 : hu / hp;
      const double den = 1.0 + 2.0 * om;
      const double gam = (1.0 + om) / den * hu;
      const double ca = (1.0 + om) * (1.0 + om) / den;
      const double cb = om * om / den;
      // predictor into Z
      for (int j = 0; j < INV; ++j) {
        const double y = VY(j), fn = VFN(j);
        const double cq = first ? 0.0 : (VYP(j) - y + fn * hp) / (hp * hp);
        Z[j] = y + hu * (fn + cq * hu);
      }
      // Jacobian by forward differences at the predictor
      bool jnew = false, have_f = false;
      if (jstale) {
        pyro::cell_rhs(P, Z, F, c, g, w);
        have_f = true;
        for (int q = 0; q < INV; ++q) {
          for (int j = 0; j < INV; ++j) X1[j] = Z[j];
          const double zq = Z[q];
          const double step = 1.4901161193847656e-08 * fmax(fabs(zq), 1e-8);
          X1[q] = zq + step;
          const double dq = X1[q] - zq;
          pyro::cell_rhs(P, X1, DZ, c, g, w);
          for (int r = 0; r < INV; ++r) EJ(r, q) = (DZ[r] - F[r]) / dq;
        }
        jstale = false;
        jage = 0;
        jnew = true;
      }
      // M = I - gam J, factorised with partial pivoting
      if (jnew || fabs(gam / glu - 1.0) > 0.3) {
        for (int r = 0; r < INV; ++r)
          for (int q = 0; q < INV; ++q)
            EM(r, q) = (r == q ? 1.0 : 0.0) - gam * EJ(r, q);
        for (int k = 0; k < INV; ++k) {
          int p = k;
          double best = fabs(EM(k, k));
          for (int r = k + 1; r < INV; ++r) {
            const double v = fabs(EM(r, k));
            if (v > best) {
              best = v;
              p = r;
            }
          }
          EP(k) = p;
          if (p != k)
            for (int q = 0; q < INV; ++q) {
              const double tmp = EM(k, q);
              EM(k, q) = EM(p, q);
              EM(p, q) = tmp;
            }
          const double inv = 1.0 / EM(k, k);
          for (int r = k + 1; r < INV; ++r) {
            const double l = EM(r, k) * inv;
            EM(r, k) = l;
            for (int q = k + 1; q < INV; ++q)
              EM(r, q) = fma(-l, EM(k, q), EM(r, q));
          }
        }
        glu = gam;
      }
      // chord Newton
      bool conv = false, fail = false;
      double cr = crate, dl_prev = 1.0;
      for (int it = 0; it < 4; ++it) {
        if (!(it == 0 && have_f)) pyro::cell_rhs(P, Z, F, c, g, w);
        for (int j = 0; j < INV; ++j)
          DZ[j] = Z[j] - (ca * VY(j) - cb * VYP(j)) - gam * F[j];
        for (int k = 0; k < INV; ++k) {
          const int p = EP(k);
          if (p != k) {
            const double tmp = DZ[k];
            DZ[k] = DZ[p];
            DZ[p] = tmp;
          }
        }
        for (int k = 0; k < INV - 1; ++k) {
          const double v = DZ[k];
          for (int r = k + 1; r < INV; ++r) DZ[r] = fma(-EM(r, k), v, DZ[r]);
        }
        for (int k = INV - 1; k >= 0; --k) {
          const double v = DZ[k] / EM(k, k);
          DZ[k] = v;
          for (int r = 0; r < k; ++r) DZ[r] = fma(-EM(r, k), v, DZ[r]);
        }
        double acc = 0.0;
        bool finite = true;
        for (int j = 0; j < INV; ++j) {
          const double zj = Z[j] - DZ[j];
          Z[j] = zj;
          finite = finite && isfinite(zj);
          const double qv = DZ[j] / (rtol * fabs(VY(j)) + atol);
          acc = fma(qv, qv, acc);
        }
        const double dl = sqrt(acc / INV);
        if (it > 0) cr = fmax(0.3 * cr, dl / dl_prev);
        if (!finite || !isfinite(dl) || (it > 0 && dl > 2.0 * dl_prev)) {
          fail = true;
          break;
        }
        if (dl * fmin(cr, 1.0) <= 0.1) {
          conv = true;
          break;
        }
        dl_prev = dl;
      }
      if (!conv) fail = true;
      // local error against the (recomputed) predictor
      double err = 0.0;
      if (conv) {
        double acc = 0.0;
        for (int j = 0; j < INV; ++j) {
          const double y = VY(j), fn = VFN(j);
          const double cq = first ? 0.0 : (VYP(j) - y + fn * hp) / (hp * hp);
          const double zp = y + hu * (fn + cq * hu);
          const double qv = (Z[j] - zp) / (rtol * fabs(y) + atol);
          acc = fma(qv, qv, acc);
        }
        err = (first ? 0.5 : (1.0 + om) / (3.0 * om + 2.0)) * sqrt(acc / INV);
      }
      const bool ok = conv && isfinite(err) && err <= 1.0;
      const bool rej = conv && !ok;
      if (ok) {
        for (int j = 0; j < INV; ++j) {
          const double y = VY(j), yp = VYP(j);
          const double z = Z[j];
          VFN(j) = (z - (ca * y - cb * yp)) / gam;
          VYP(j) = y;
          VY(j) = z;
        }
        t = t + hu;
        hp = hu;
        nsteps += 1;
        crate = cr;
        jage += 1;
        if (jage >= 20) jstale = true;
      } else {
        crate = 1.0;
      }
      natt += 1;
      if (fail) jstale = true;
      const double e = fmax(err, 1e-10);
      double fac;
      if (ok)
        fac = fmin(fmax(0.9 * pow(e, -1.0 / 3.0), 0.2), 2.0);
      else if (rej)
        fac = fmin(fmax(0.9 * pow(e, -1.0 / 3.0), 0.1), 0.9);
      else
        fac = jnew ? 0.25 : 1.0;
      if (!isfinite(fac)) fac = 0.25;
      h = hu * fac;
      bool finite_y = true;
      for (int j = 0; j < INV; ++j) finite_y = finite_y && isfinite(VY(j));
      const bool stuck = (t + h == t) && (t > 0.0);
      if (stuck || h < 1e-30 || natt > max_attempts || !finite_y) {
        failed = true;
        finished = true;
        break;
      }
      if (t >= te * (1.0 - 1e-12)) {
        finished = true;
        break;
      }
    }
    Tt[i] = t;
    Hh[i] = h;
    Hp[i] = hp;
    Glu[i] = glu;
    Crate[i] = crate;
    Nsteps[i] = nsteps;
    Natt[i] = natt;
    Jage[i] = jage;
    Jstale[i] = jstale ? 1 : 0;
    if (failed) Failed[i] = 1;
    if (finished) {
      Active[i] = 0;
      Done[i] = 1;
    }
  }
#undef VY
#undef VYP
#undef VFN
#undef EJ
#undef EM
#undef EP
}

// Shared memory of k_reactor_bdf2 per CTA.
#define BDF2_SMEM ((size_t)(3 * NS + 4 * INV) * IBLOCK * sizeof(double))

PYRO_EXPORT int pyro_reactor_bdf2(
    double* y, double* y_prev, double* f_n, int64_t ld, const double* p,
    double* t, const double* t_end, double* h, double* h_prev, double* g_lu,
    double* crate, int64_t* nsteps, int64_t* nattempts, int64_t* jage,
    unsigned char* active, unsigned char* failed, unsigned char* jstale,
    unsigned char* done, double* J, double* M, int* piv,
    const int64_t* slots, int64_t n, int attempts, double rtol, double atol,
    int64_t max_attempts, cudaStream_t stream) {
  if (n < 0 || (!slots && ld < n) || attempts < 1 || !(rtol > 0.0) ||
      !(atol > 0.0))
    return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!y || !y_prev || !f_n || !p || !t || !t_end || !h || !h_prev ||
      !g_lu || !crate || !nsteps || !nattempts || !jage || !active ||
      !failed || !jstale || !done || !J || !M || !piv)
    return PYRO_ERR_ARGUMENT;
  if (prepare_smem((const void*)k_reactor_bdf2, BDF2_SMEM) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  int64_t blocks = (n + IBLOCK - 1) / IBLOCK;
  const int64_t cap = (int64_t)pyro_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  k_reactor_bdf2<<<(int)blocks, IBLOCK, BDF2_SMEM, stream>>>(
      y, y_prev, f_n, ld, p, t, t_end, h, h_prev, g_lu, crate, nsteps,
      nattempts, jage, active, failed, jstale, done, J, M, piv, slots, n,
      attempts, rtol, atol, max_attempts);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}
