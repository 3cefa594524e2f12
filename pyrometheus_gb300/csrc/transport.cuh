// Mixture-averaged transport of a generated mechanism library (FP64,
// sm_103a): the transport methods of the reference's generated class
// (pyrometheus/codegen/python.py:564-641) with the fit forms and mixture
// rules of pyrometheus/chem_expr.py:190-267.
//
//   mu_k  = sqrt(T) P_k(L)^2,  lam_k = sqrt(T) Q_k(L),
//   D_ij  = sqrt(T) T R_ij(L),   L = ln T, degree-4 fits in L
//   mu    = sum_k x_k mu_k / f_k,
//           f_k = sum_j x_j (1 + sqrt(mu_k/mu_j sqrt(W_j/W_k)))^2
//                   / sqrt(8 (1 + W_k/W_j))                  (Wilke)
//   lam   = (sum_k x_k lam_k + 1 / sum_k x_k/lam_k) / 2
//   D_k   = (mmw - x_k W_k) / (p mmw (sum_i x_i/D_ik - x_k/D_kk)), or
//           D_kk / p where that denominator is not positive
//
// One thread per state.  FP64 is the bound (GB300 retires two FP64 lanes
// per SM per clock), so the formulation removes FP64 work the direct form
// repeats per species pair:
//   * sqrt(mu_k/mu_j sqrt(W_j/W_k)) = a_k / a_j with a_k = |P_k| W_k^-1/4
//     (sqrt(T) cancels), so Wilke's rule needs no square root per pair:
//     f_k = s0_k + a_k (2 s1_k + a_k s2_k) with s0_k = sum_j C_kj x_j,
//     s1_k = sum_j C_kj x_j/a_j, s2_k = sum_j C_kj x_j/a_j^2 and the
//     constant C_kj = 1/sqrt(8 (1 + W_k/W_j)): three FMAs per pair, all
//     terms positive (no cancellation);
//   * the powers of L are formed once per state and every fit is summed in
//     the reference's order c0 + c1 L + c2 L^2 + c3 L^3 + c4 L^4;
//   * with symmetric diffusivity fits (Cantera's are) each pair's 1/R_ij is
//     formed once and added to both x_sum_i and x_sum_j, the reciprocals
//     are formed four at a time by one division (rcp4), and the common
//     1/(sqrt(T) T) is applied once per species.
// Thread-private vectors (mole fractions and the Wilke / x_sum work
// vectors) are shared-memory columns interleaved by thread.
#pragma once

#ifdef PYRO_HAS_TRANSPORT

namespace pyro_tr {

using TCols = pyro::ColsT<TBLOCK>;

__device__ __forceinline__ TCols tcol(double* smem, int q) {
  return TCols{smem + (size_t)q * NS * TBLOCK + threadIdx.x};
}

struct Powers {
  double L, L2, L3, L4;
};

__device__ __forceinline__ Powers powers(double T) {
  Powers p;
  p.L = log(T);
  p.L2 = p.L * p.L;
  p.L3 = p.L2 * p.L;
  p.L4 = p.L2 * p.L2;
  return p;
}

// c0 + c1 L + c2 L^2 + c3 L^3 + c4 L^4, summed left to right
__device__ __forceinline__ double fit(const double* __restrict__ c,
                                      const Powers& p) {
  return fma(__ldg(c + 4), p.L4,
             fma(__ldg(c + 3), p.L3,
                 fma(__ldg(c + 2), p.L2, fma(__ldg(c + 1), p.L, __ldg(c)))));
}

__device__ __forceinline__ const double* diff_fit(int i, int j) {
#if PYRO_TR_SYM
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  return k_tr_diff + 5 * (hi * (hi + 1) / 2 + lo);
#else
  return k_tr_diff + 5 * (i * NS + j);
#endif
}

// |v| in [2^-200, 2^200] (and finite, nonzero)
__device__ __forceinline__ bool rcp_range(double v) {
  const unsigned e = ((unsigned)__double2hiint(v) >> 20) & 0x7ffu;
  return e - (1023u - 200u) <= 400u;
}

// r = 1/R for four values by one division (Montgomery's simultaneous
// inversion, Math. Comp. 48 (1987) 243-264): three products forward, one
// reciprocal, six products back -- 10 FP64 instructions instead of four
// divisions.  Taken only when every value lies in [2^-200, 2^200], so no
// partial product overflows or underflows; otherwise (and for zeros,
// infinities and NaNs) each value is divided on its own, as the reference
// divides every pair.
__device__ __forceinline__ void rcp4(const double R[4], double r[4]) {
  if (rcp_range(R[0]) & rcp_range(R[1]) & rcp_range(R[2]) &
      rcp_range(R[3])) {
    const double p01 = R[0] * R[1], p012 = p01 * R[2];
    double inv = 1.0 / (p012 * R[3]);
    r[3] = inv * p012;
    inv *= R[3];
    r[2] = inv * p01;
    inv *= R[2];
    r[1] = inv * R[0];
    r[0] = inv * R[1];
  } else {
#pragma unroll
    for (int u = 0; u < 4; ++u) r[u] = 1.0 / R[u];
  }
}

// Adds x_k mu_k / f_k for k = k0 .. k0+K-1 (in that order) to acc: the
// K species' Wilke sums run as 3K independent FMA chains over j, which
// keeps the FP64 pipe fed from one warp per scheduler.
template <int K>
__device__ __forceinline__ void wilke_block(int k0, TCols X, TCols V,
                                            TCols Q, const Powers& pw,
                                            double sq, double& acc) {
  double s0[K], s1[K], s2[K];
#pragma unroll
  for (int u = 0; u < K; ++u) s0[u] = s1[u] = s2[u] = 0.0;
  const double* __restrict__ c = k_tr_wilke + k0 * NS;
  for (int j = 0; j < NS; ++j) {
    const double xj = X[j], vj = V[j], qj = Q[j];
#pragma unroll
    for (int u = 0; u < K; ++u) {
      const double ckj = __ldg(c + u * NS + j);
      s0[u] = fma(ckj, xj, s0[u]);
      s1[u] = fma(ckj, vj, s1[u]);
      s2[u] = fma(ckj, qj, s2[u]);
    }
  }
#pragma unroll
  for (int u = 0; u < K; ++u) {
    const double pk = fit(k_tr_visc + 5 * (k0 + u), pw);
    const double a = fabs(pk) * k_tr_wq[k0 + u];
    const double f = fma(a, fma(a, s2[u], 2.0 * s1[u]), s0[u]);
    acc += X[k0 + u] * (sq * (pk * pk)) / f;
  }
}

}  // namespace pyro_tr

// which = 0: species viscosities, 1: species thermal conductivities.
__global__ void __launch_bounds__(BLOCK)
    k_tr_species(int which, const double* __restrict__ Tp, int64_t t_inc,
                 double* __restrict__ out, int64_t ldo, int64_t n) {
  const double* fits = which == 0 ? k_tr_visc : k_tr_cond;
  for (int64_t i = (int64_t)blockIdx.x * BLOCK + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * BLOCK) {
    const double T = pyro_ld(Tp, t_inc, i);
    const pyro_tr::Powers p = pyro_tr::powers(T);
    const double sq = sqrt(T);
    for (int k = 0; k < NS; ++k) {
      const double v = pyro_tr::fit(fits + 5 * k, p);
      out[(int64_t)k * ldo + i] = which == 0 ? sq * (v * v) : sq * v;
    }
  }
}

// D_ij for every pair, out[(i NS + j) ldo + state].
__global__ void __launch_bounds__(BLOCK)
    k_tr_binary(const double* __restrict__ Tp, int64_t t_inc,
                double* __restrict__ out, int64_t ldo, int64_t n) {
  for (int64_t s = (int64_t)blockIdx.x * BLOCK + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * BLOCK) {
    const double T = pyro_ld(Tp, t_inc, s);
    const pyro_tr::Powers p = pyro_tr::powers(T);
    const double sqt = sqrt(T) * T;
    for (int i = 0; i < NS; ++i)
      for (int j = 0; j < NS; ++j)
        out[(int64_t)(i * NS + j) * ldo + s] =
            sqt * pyro_tr::fit(pyro_tr::diff_fit(i, j), p);
  }
}

// Mixture viscosity, conductivity and species diffusivities of each state;
// a null output pointer skips that quantity.
__global__ void __launch_bounds__(TBLOCK)
    k_transport_mixavg(const double* __restrict__ Pp, int64_t p_inc,
                       const double* __restrict__ Tp, int64_t t_inc,
                       const double* __restrict__ Y, int64_t ldy,
                       double* __restrict__ mu_out,
                       double* __restrict__ lam_out,
                       double* __restrict__ d_out, int64_t ldd, int64_t n) {
  extern __shared__ double smem[];
  using pyro_tr::fit;
  const pyro_tr::TCols X = pyro_tr::tcol(smem, 0),
                       V = pyro_tr::tcol(smem, 1),
                       Q = pyro_tr::tcol(smem, 2);
  for (int64_t i = (int64_t)blockIdx.x * TBLOCK + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * TBLOCK) {
    const double T = pyro_ld(Tp, t_inc, i);
    const pyro_tr::Powers pw = pyro_tr::powers(T);
    const double sq = sqrt(T);
    // mole fractions x_k = Y_k / W_k * mmw (python.py:265-285)
    double sy = 0.0;
    for (int k = 0; k < NS; ++k)
      sy = fma(k_inv_mw[k], __ldg(Y + (int64_t)k * ldy + i), sy);
    const double mmw = 1.0 / sy;
    for (int k = 0; k < NS; ++k)
      X[k] = k_inv_mw[k] * __ldg(Y + (int64_t)k * ldy + i) * mmw;

    if (mu_out) {
      // V = x_k / a_k, Q = x_k / a_k^2 (P_k is formed again where it is
      // used: four FMAs per species buy a third fewer shared-memory
      // columns, so more states fit on an SM)
      for (int k = 0; k < NS; ++k) {
        const double pk = fit(k_tr_visc + 5 * k, pw);
        const double b = 1.0 / (fabs(pk) * k_tr_wq[k]);
        const double v = X[k] * b;
        V[k] = v;
        Q[k] = v * b;
      }
      double acc = 0.0;
      int k = 0;
      for (; k + 4 <= NS; k += 4)
        pyro_tr::wilke_block<4>(k, X, V, Q, pw, sq, acc);
      for (; k < NS; ++k) pyro_tr::wilke_block<1>(k, X, V, Q, pw, sq, acc);
      mu_out[i] = acc;
    }

    if (lam_out) {
      double s1 = 0.0, s2 = 0.0;
      for (int k = 0; k < NS; ++k) {
        const double l = sq * fit(k_tr_cond + 5 * k, pw);
        s1 = fma(X[k], l, s1);
        s2 += X[k] / l;
      }
      lam_out[i] = 0.5 * (s1 + 1.0 / s2);
    }

    if (d_out) {
      // V accumulates sum_i x_i / R_ik, Q keeps 1 / R_kk
      const double P = pyro_ld(Pp, p_inc, i);
#if PYRO_TR_SYM
      for (int k = 0; k < NS; ++k) V[k] = 0.0;
      for (int j = 0; j < NS; ++j) {
        const double xj = X[j];
        const double* __restrict__ c = k_tr_diff + 5 * (j * (j + 1) / 2);
        double acc = 0.0;
        int m = 0;
#pragma unroll 2
        for (; m + 4 <= j; m += 4) {
          double R[4], r[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) R[u] = fit(c + 5 * (m + u), pw);
          pyro_tr::rcp4(R, r);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            acc = fma(X[m + u], r[u], acc);
            V[m + u] = fma(xj, r[u], V[m + u]);
          }
        }
        for (; m < j; ++m) {
          const double r = 1.0 / fit(c + 5 * m, pw);
          acc = fma(X[m], r, acc);
          V[m] = fma(xj, r, V[m]);
        }
        const double rjj = 1.0 / fit(c + 5 * j, pw);
        V[j] = fma(xj, rjj, acc);
        Q[j] = rjj;
      }
#else
      for (int j = 0; j < NS; ++j) {
        double acc = 0.0;
        for (int m = 0; m < NS; ++m)
          acc = fma(X[m], 1.0 / fit(k_tr_diff + 5 * (m * NS + j), pw), acc);
        V[j] = acc;
        Q[j] = 1.0 / fit(k_tr_diff + 5 * (j * NS + j), pw);
      }
#endif
      const double sqt = sq * T;
      const double inv15 = 1.0 / sqt;
      for (int k = 0; k < NS; ++k) {
        const double xk = X[k];
        const double denom = (V[k] - xk * Q[k]) * inv15;
        double dk;
        if (denom > 0.0)
          dk = (mmw - xk * k_mw[k]) / (P * mmw * denom);
        else
          dk = sqt * fit(pyro_tr::diff_fit(k, k), pw) / P;
        d_out[(int64_t)k * ldd + i] = dk;
      }
    }
  }
}

#endif  // PYRO_HAS_TRANSPORT

// ---- C ABI -----------------------------------------------------------------

PYRO_EXPORT int pyro_transport_info(int* available, int* symmetric) {
#ifdef PYRO_HAS_TRANSPORT
  if (available) *available = 1;
  if (symmetric) *symmetric = PYRO_TR_SYM;
#else
  if (available) *available = 0;
  if (symmetric) *symmetric = 0;
#endif
  return PYRO_OK;
}

PYRO_EXPORT int pyro_species_transport(int which, const double* T,
                                       int64_t t_inc, double* out,
                                       int64_t ldo, int64_t n,
                                       cudaStream_t stream) {
#ifdef PYRO_HAS_TRANSPORT
  if (n < 0 || which < 0 || which > 1) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!T || !out || ldo < n) return PYRO_ERR_ARGUMENT;
  k_tr_species<<<pyro_grid(n, BLOCK, pyro_sm_count() * BLOCKS_PER_SM), BLOCK,
                 0, stream>>>(which, T, t_inc, out, ldo, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
#else
  (void)which; (void)T; (void)t_inc; (void)out; (void)ldo; (void)n;
  (void)stream;
  return PYRO_ERR_UNSUPPORTED;
#endif
}

PYRO_EXPORT int pyro_binary_diffusivities(const double* T, int64_t t_inc,
                                          double* out, int64_t ldo, int64_t n,
                                          cudaStream_t stream) {
#ifdef PYRO_HAS_TRANSPORT
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!T || !out || ldo < n) return PYRO_ERR_ARGUMENT;
  k_tr_binary<<<pyro_grid(n, BLOCK, pyro_sm_count() * BLOCKS_PER_SM), BLOCK,
                0, stream>>>(T, t_inc, out, ldo, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
#else
  (void)T; (void)t_inc; (void)out; (void)ldo; (void)n; (void)stream;
  return PYRO_ERR_UNSUPPORTED;
#endif
}

PYRO_EXPORT int pyro_transport_mixavg(const double* P, int64_t p_inc,
                                      const double* T, int64_t t_inc,
                                      const double* Y, int64_t ldy,
                                      double* mu, double* lam, double* D,
                                      int64_t ldd, int64_t n,
                                      cudaStream_t stream) {
#ifdef PYRO_HAS_TRANSPORT
  if (n < 0) return PYRO_ERR_ARGUMENT;
  if (n == 0 || (!mu && !lam && !D)) return PYRO_OK;
  if (!T || !Y || ldy < n) return PYRO_ERR_ARGUMENT;
  if (D && (!P || ldd < n)) return PYRO_ERR_ARGUMENT;
  const size_t bytes = (size_t)3 * NS * TBLOCK * sizeof(double);
  if (bytes > 48 * 1024 &&
      cudaFuncSetAttribute(k_transport_mixavg,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)bytes) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  k_transport_mixavg<<<pyro_grid(n, TBLOCK, pyro_sm_count() * TBLOCKS_PER_SM),
                       TBLOCK, bytes, stream>>>(P, p_inc, T, t_inc, Y, ldy,
                                                mu, lam, D, ldd, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
#else
  (void)P; (void)p_inc; (void)T; (void)t_inc; (void)Y; (void)ldy; (void)mu;
  (void)lam; (void)D; (void)ldd; (void)n; (void)stream;
  return PYRO_ERR_UNSUPPORTED;
#endif
}
