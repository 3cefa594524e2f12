// Steady-flamelet residual and block-tridiagonal Jacobian on the device
// (FP64, sm_103a): the assembly of pyrometheus/flamelets/equations.py
// (FlameletEquations.rhs :167-227, jac :228-282, source_terms :313-359)
// with the Laplacian block form of onedim_laplacian.py:144-180, for many
// flamelets at once.
//
// Unknowns per grid point: phi = (h, Y_1..Y_S) (mixture enthalpy per unit
// mass and mass fractions).  Per point, with T from h by Newton (the
// caller's get_temperature_from_enthalpy) and rho = p / (R T sigma),
// sigma = sum_k Y_k / W_k:
//   source   S = (v / rho, W_k w_k / rho)          (v: viscous heating)
//   residual R_i = chi_i / 2 Lap(phi)_i + S_i m_i - BC_i,
//            Lap(phi)_i = (phi_{i-1} - 2 phi_i + phi_{i+1}) / dx^2 inside,
//            phi_i / dx^2 at the two boundary points; m_i = 0 there and
//            BC_i = (h_ox, y_ox) first, (h_fu, y_fu) last, 0 inside
//   blocks   C_i = chi_i / 2 Lap_c,i I + dS/dphi_i (0 at the boundaries),
//            L_i = chi_{i+1} / 2 dx^-2 I when point i+1 is interior,
//            U_i = chi_i / 2 dx^-2 I when point i is interior, else 0.
// The dissipation rates of the boundary points are used as given, as the
// reference does (its _enforce_dirichlet_bcs builds new arrays with
// .at[].set and discards them).
//
// dS/dphi comes from the reactor Jacobian J = d(dT/dt, W w / rho)/d(T, Y)
// at (T, Y, p) (k_reactor_jacobian, written into the C blocks first) by
// the chain rule through T(h, Y): dT/dh = 1 / cp, dT/dY_m = -h_m / cp
// (h_m, cp per unit mass); this is what the reference's jacfwd through its
// Newton loop converges to.  The enthalpy row: d(v/rho) = (v/rho)
// (dT / T + dY_m / (sigma W_m)).
//
// Layout: systems packed along rows as for the block-Thomas solver:
// system s owns rows [row_off[s], row_off[s+1]) (at least 3), sys_of_row
// gives s for every row; per-row arrays [rows], species-major [S][ld];
// blocks [rows][nv][nv] row-major (nv = S + 1); the residual [nv][ldr].
#pragma once

#define FNV (NS + 1)

// Transform the reactor Jacobian held in C in place and write L and U.
// ADJ: the adjoint operator of the EOS-consistency solves instead
// (FlameletEquations.adjoint_operator, equations.py:451-516): interior
// C_i = Lap_c I + (2 / chi_i) (dS/dphi_i)^T, boundary C_i = chi_i / 2
// dx^-2 I, and L, U the Laplacian's own (unscaled) couplings.
//
// A CTA takes tiles of kFbRows rows.  The per-row scalars (T, sigma, cp,
// rho, the species enthalpies per unit mass, the Laplacian couplings) are
// formed one thread per row, so every lane of those FP64 instructions
// works (GB300's FP64 pipe retires a warp instruction per 64 cycles per
// partition whatever its active lanes); then each warp takes rows of the
// tile with its lanes over the block's elements (coalesced).
constexpr int kFbRows = 128;

template <bool ADJ>
__global__ void __launch_bounds__(kFbRows)
    k_flamelet_blocks(const double* __restrict__ Pp, int64_t p_inc,
                      const double* __restrict__ Tt,
                      const double* __restrict__ Y, int64_t ldy,
                      const double* __restrict__ chi,
                      const double* __restrict__ visc,
                      const int64_t* __restrict__ row_off,
                      const int* __restrict__ sys_of_row,
                      const double* __restrict__ inv_dx2,
                      double* __restrict__ L, double* __restrict__ C,
                      double* __restrict__ U, int64_t rows) {
  constexpr int NB = FNV * FNV;
  // per row of the tile: species enthalpies per unit mass, and the scalars
  // 1/cp, v/rho, 1/T, 1/sigma, the C diagonal term, the L and U diagonals,
  // 2/chi; the interior flag
  __shared__ double s_hm[NS][kFbRows];
  __shared__ double s_sc[8][kFbRows];
  __shared__ int s_in[kFbRows];
  __shared__ double s_c0[kFbRows / 32][NS];  // J[1+k][0] / cp of a row
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double* c0_w = s_c0[wid];
  for (int64_t base = (int64_t)blockIdx.x * kFbRows; base < rows;
       base += (int64_t)gridDim.x * kFbRows) {
    const int q = threadIdx.x;
    const int64_t r = base + q;
    if (r < rows) {
      const int s = sys_of_row[r];
      const int64_t r0 = row_off[s], r1 = row_off[s + 1];
      const bool first = r == r0, last = r == r1 - 1;
      const bool interior = !first && !last;
      const double idx2 = inv_dx2[s];
      const double T = Tt[r];
      const double invT = 1.0 / T;
      double sig = 0.0, cpp = 0.0;
      for (int k = 0; k < NS; ++k) {
        const double wk = __ldg(Y + (int64_t)k * ldy + r) * k_inv_mw[k];
        const pyro::Nasa a(k, T > k_tmid[k]);
        const double cpk =
            fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
        const double hrt =
            fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                              a[2] * (1.0 / 3.0)),
                      a[1] * 0.5),
                a[0]) +
            a[5] * invT;
        s_hm[k][q] = GAS_CONSTANT * T * hrt * k_inv_mw[k];
        sig += wk;
        cpp = fma(wk, cpk, cpp);
      }
      const double cp = GAS_CONSTANT * cpp;
      const double rho = pyro_ld(Pp, p_inc, r) / (GAS_CONSTANT * T * sig);
      const double lap_c = interior ? -2.0 * idx2 : idx2;
      const bool next_interior = !last && (r + 1 < r1 - 1);
      s_sc[0][q] = 1.0 / cp;
      s_sc[1][q] = visc[r] / rho;
      s_sc[2][q] = invT;
      s_sc[3][q] = 1.0 / sig;
      s_sc[4][q] = (ADJ && interior) ? lap_c : 0.5 * chi[r] * lap_c;
      s_sc[5][q] =
          next_interior ? (ADJ ? idx2 : 0.5 * chi[r + 1] * idx2) : 0.0;
      s_sc[6][q] = interior ? (ADJ ? idx2 : 0.5 * chi[r] * idx2) : 0.0;
      s_sc[7][q] = ADJ ? 2.0 / chi[r] : 0.0;
      s_in[q] = interior ? 1 : 0;
    }
    __syncthreads();
    for (int q = wid; q < kFbRows && base + q < rows; q += kFbRows / 32) {
      const int64_t rr = base + q;
      double* Cr = C + rr * NB;
      const double inv_cp = s_sc[0][q];
      if (s_in[q]) {
        // species rows: column 0 <- J[1+k][0] / cp, columns m <- J -
        // J[.][0] h_m / cp (each row's column 0 staged first)
        for (int k = lane; k < NS; k += 32)
          c0_w[k] = Cr[(int64_t)(k + 1) * FNV] * inv_cp;
        __syncwarp();
        for (int e = FNV + lane; e < NB; e += 32) {
          const int a = e / FNV, b = e - a * FNV;
          const double c0 = c0_w[a - 1];
          Cr[e] = b == 0 ? c0 : fma(-c0, s_hm[b - 1][q], Cr[e]);
        }
        // enthalpy row
        const double vr = s_sc[1][q], invT = s_sc[2][q];
        for (int m = lane; m < FNV; m += 32) {
          Cr[m] = m == 0 ? vr * invT * inv_cp
                         : vr * (k_inv_mw[m - 1] * s_sc[3][q] -
                                 s_hm[m - 1][q] * inv_cp * invT);
        }
        if (ADJ) {
          // (2 / chi) dS/dphi, transposed in place (each off-diagonal pair
          // swapped by one lane)
          __syncwarp();
          const double sc = s_sc[7][q];
          for (int e = lane; e < NB; e += 32) {
            const int a = e / FNV, b = e - a * FNV;
            if (a < b) {
              const double x = Cr[e], y = Cr[b * FNV + a];
              Cr[e] = sc * y;
              Cr[b * FNV + a] = sc * x;
            } else if (a == b) {
              Cr[e] *= sc;
            }
          }
        }
      } else {
        for (int e = lane; e < NB; e += 32) Cr[e] = 0.0;
      }
      __syncwarp();
      // Laplacian diagonal, and the couplings
      const double dgl = s_sc[4][q], lo = s_sc[5][q], up = s_sc[6][q];
      for (int d = lane; d < FNV; d += 32) Cr[(int64_t)d * FNV + d] += dgl;
      double* Lr = L + rr * NB;
      double* Ur = U + rr * NB;
      for (int e = lane; e < NB; e += 32) {
        const bool diag = (e % (FNV + 1)) == 0;
        Lr[e] = diag ? lo : 0.0;
        Ur[e] = diag ? up : 0.0;
      }
      __syncwarp();
    }
    __syncthreads();  // before the next tile's scalars
  }
}

// thread per row: R T (R = R_u / W_mix) and its gradient with respect to
// phi = (h, Y) at T(h, Y) (local_compressible_eos_rt and its jacfwd,
// equations.py:517-535): d(RT)/dh = R_u sigma / cp,
// d(RT)/dY_m = -R_u sigma h_m / cp + R_u T / W_m (sigma = sum Y/W).
__global__ void __launch_bounds__(128)
    k_flamelet_eos_rt(const double* __restrict__ Tt,
                      const double* __restrict__ Y, int64_t ldy,
                      double* __restrict__ rt, double* __restrict__ J,
                      int64_t ldj, int64_t rows) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const double T = Tt[r];
    double sig = 0.0, cpp = 0.0;
    for (int k = 0; k < NS; ++k) {
      const double wk = __ldg(Y + (int64_t)k * ldy + r) * k_inv_mw[k];
      const pyro::Nasa a(k, T > k_tmid[k]);
      sig += wk;
      cpp = fma(wk,
                fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]),
                cpp);
    }
    const double rs = GAS_CONSTANT * sig;
    rt[r] = GAS_CONSTANT * T / (1.0 / sig);
    if (!J) continue;
    const double inv_cp = 1.0 / (GAS_CONSTANT * cpp);
    const double invT = 1.0 / T;
    J[r] = rs * inv_cp;
    for (int m = 0; m < NS; ++m) {
      const pyro::Nasa a(m, T > k_tmid[m]);
      const double hrt =
          fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                            a[2] * (1.0 / 3.0)),
                    a[1] * 0.5),
              a[0]) +
          a[5] * invT;
      const double hm = GAS_CONSTANT * T * hrt * k_inv_mw[m];
      J[(int64_t)(m + 1) * ldj + r] =
          fma(-rs * inv_cp, hm, GAS_CONSTANT * T * k_inv_mw[m]);
    }
  }
}

// thread per row: the residual R [nv][ldr].
__global__ void __launch_bounds__(128)
    k_flamelet_residual(const double* __restrict__ Pp, int64_t p_inc,
                        const double* __restrict__ Tt,
                        const double* __restrict__ H,
                        const double* __restrict__ Y, int64_t ldy,
                        const double* __restrict__ F, int64_t ldf,
                        const double* __restrict__ chi,
                        const double* __restrict__ visc,
                        const int64_t* __restrict__ row_off,
                        const int* __restrict__ sys_of_row,
                        const double* __restrict__ inv_dx2,
                        const double* __restrict__ h_ox,
                        const double* __restrict__ h_fu,
                        const double* __restrict__ y_ox,
                        const double* __restrict__ y_fu, int64_t ldb,
                        double* __restrict__ R, int64_t ldr, int64_t rows) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int s = sys_of_row[r];
    const int64_t r0 = row_off[s], r1 = row_off[s + 1];
    const bool first = r == r0, last = r == r1 - 1;
    const double idx2 = inv_dx2[s];
    const double hc = 0.5 * chi[r];
    const double T = Tt[r];
    double sig = 0.0;
    for (int k = 0; k < NS; ++k)
      sig = fma(__ldg(Y + (int64_t)k * ldy + r), k_inv_mw[k], sig);
    const double rho = pyro_ld(Pp, p_inc, r) / (GAS_CONSTANT * T * sig);
    // enthalpy
    {
      double v;
      if (first)
        v = hc * (H[r] * idx2) - h_ox[s];
      else if (last)
        v = hc * (H[r] * idx2) - h_fu[s];
      else
        v = hc * ((H[r - 1] - 2.0 * H[r] + H[r + 1]) * idx2) + visc[r] / rho;
      R[r] = v;
    }
    for (int k = 0; k < NS; ++k) {
      const double* yk = Y + (int64_t)k * ldy;
      double v;
      if (first)
        v = hc * (yk[r] * idx2) - y_ox[(int64_t)k * ldb + s];
      else if (last)
        v = hc * (yk[r] * idx2) - y_fu[(int64_t)k * ldb + s];
      else
        v = hc * ((yk[r - 1] - 2.0 * yk[r] + yk[r + 1]) * idx2) +
            F[(int64_t)(k + 1) * ldf + r];
      R[(int64_t)(k + 1) * ldr + r] = v;
    }
  }
}

PYRO_EXPORT int pyro_flamelet_blocks(const double* p, int64_t p_inc,
                                     const double* T, const double* Y,
                                     int64_t ldy, const double* chi,
                                     const double* visc,
                                     const int64_t* row_off,
                                     const int* sys_of_row,
                                     const double* inv_dx2, double* L,
                                     double* C, double* U, int64_t rows,
                                     cudaStream_t stream) {
  if (rows < 0 || ldy < rows) return PYRO_ERR_ARGUMENT;
  if (rows == 0) return PYRO_OK;
  if (!p || !T || !Y || !chi || !visc || !row_off || !sys_of_row ||
      !inv_dx2 || !L || !C || !U)
    return PYRO_ERR_ARGUMENT;
  int64_t blocks = (rows + kFbRows - 1) / kFbRows;
  const int64_t cap = (int64_t)pyro_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  k_flamelet_blocks<false><<<(int)blocks, kFbRows, 0, stream>>>(
      p, p_inc, T, Y, ldy, chi, visc, row_off, sys_of_row, inv_dx2, L, C, U,
      rows);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_flamelet_adjoint_blocks(
    const double* p, int64_t p_inc, const double* T, const double* Y,
    int64_t ldy, const double* chi, const double* visc,
    const int64_t* row_off, const int* sys_of_row, const double* inv_dx2,
    double* L, double* C, double* U, int64_t rows, cudaStream_t stream) {
  if (rows < 0 || ldy < rows) return PYRO_ERR_ARGUMENT;
  if (rows == 0) return PYRO_OK;
  if (!p || !T || !Y || !chi || !visc || !row_off || !sys_of_row ||
      !inv_dx2 || !L || !C || !U)
    return PYRO_ERR_ARGUMENT;
  int64_t blocks = (rows + kFbRows - 1) / kFbRows;
  const int64_t cap = (int64_t)pyro_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  k_flamelet_blocks<true><<<(int)blocks, kFbRows, 0, stream>>>(
      p, p_inc, T, Y, ldy, chi, visc, row_off, sys_of_row, inv_dx2, L, C, U,
      rows);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_flamelet_eos_rt(const double* T, const double* Y,
                                     int64_t ldy, double* rt, double* J,
                                     int64_t ldj, int64_t rows,
                                     cudaStream_t stream) {
  if (rows < 0 || ldy < rows || (J && ldj < rows)) return PYRO_ERR_ARGUMENT;
  if (rows == 0) return PYRO_OK;
  if (!T || !Y || !rt) return PYRO_ERR_ARGUMENT;
  int64_t blocks = (rows + 127) / 128;
  const int64_t cap = (int64_t)pyro_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  k_flamelet_eos_rt<<<(int)blocks, 128, 0, stream>>>(T, Y, ldy, rt, J, ldj,
                                                     rows);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

PYRO_EXPORT int pyro_flamelet_residual(
    const double* p, int64_t p_inc, const double* T, const double* h,
    const double* Y, int64_t ldy, const double* F, int64_t ldf,
    const double* chi, const double* visc, const int64_t* row_off,
    const int* sys_of_row, const double* inv_dx2, const double* h_ox,
    const double* h_fu, const double* y_ox, const double* y_fu, int64_t ldb,
    double* R, int64_t ldr, int64_t rows, cudaStream_t stream) {
  if (rows < 0 || ldy < rows || ldf < rows || ldr < rows || ldb < 1)
    return PYRO_ERR_ARGUMENT;
  if (rows == 0) return PYRO_OK;
  if (!p || !T || !h || !Y || !F || !chi || !visc || !row_off ||
      !sys_of_row || !inv_dx2 || !h_ox || !h_fu || !y_ox || !y_fu || !R)
    return PYRO_ERR_ARGUMENT;
  int64_t blocks = (rows + 127) / 128;
  const int64_t cap = (int64_t)pyro_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  k_flamelet_residual<<<(int)blocks, 128, 0, stream>>>(
      p, p_inc, T, h, Y, ldy, F, ldf, chi, visc, row_off, sys_of_row,
      inv_dx2, h_ox, h_fu, y_ox, y_fu, ldb, R, ldr, rows);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

// one warp per row: the matrix-free flamelet Jacobian action
// A v = chi / 2 Lap(v) + dS/dphi v (FlameletEquations.jacobian_action,
// equations.py:411-450), with every point's source Jacobian -- the two
// boundary points included, unlike the blocks -- and the Laplacian's
// boundary rows v / dx^2.  dS/dphi v comes from the reactor Jacobian J at
// (T, Y, p) without forming dS/dphi: with a = (v_h - sum_m h_m v_m) / cp
// (the temperature change along v), the species rows are J (a, v_Y) and
// the enthalpy row (v / rho) (a / T + sum_m v_m / (sigma W_m)).
__global__ void __launch_bounds__(128)
    k_flamelet_jacobian_action(
        const double* __restrict__ Pp, int64_t p_inc,
        const double* __restrict__ Tt, const double* __restrict__ Y,
        int64_t ldy, const double* __restrict__ J,
        const double* __restrict__ V, int64_t ldv,
        const double* __restrict__ chi, const double* __restrict__ visc,
        const int64_t* __restrict__ row_off,
        const int* __restrict__ sys_of_row,
        const double* __restrict__ inv_dx2, double* __restrict__ A,
        int64_t lda, int64_t rows) {
  const int lane = threadIdx.x & 31;
  constexpr int NB = FNV * FNV;
  __shared__ double s_z[4][FNV];
  double* z = s_z[threadIdx.x >> 5];
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
       r < rows; r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int s = sys_of_row[r];
    const int64_t r0 = row_off[s], r1 = row_off[s + 1];
    const bool interior = r != r0 && r != r1 - 1;
    const double idx2 = inv_dx2[s];
    const double T = Tt[r];
    const double invT = 1.0 / T;
    double sig = 0.0, cpp = 0.0, hv = 0.0, wv = 0.0;
    for (int k = lane; k < NS; k += 32) {
      const double wk = __ldg(Y + (int64_t)k * ldy + r) * k_inv_mw[k];
      const pyro::Nasa a(k, T > k_tmid[k]);
      const double cpk =
          fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
      const double hrt =
          fma(T, fma(T, fma(T, fma(T, a[4] * 0.2, a[3] * 0.25),
                            a[2] * (1.0 / 3.0)),
                    a[1] * 0.5),
              a[0]) +
          a[5] * invT;
      const double vk = __ldg(V + (int64_t)(k + 1) * ldv + r);
      sig += wk;
      cpp = fma(wk, cpk, cpp);
      hv = fma(GAS_CONSTANT * T * hrt * k_inv_mw[k], vk, hv);
      wv = fma(k_inv_mw[k], vk, wv);
      z[k + 1] = vk;
    }
    const double sigma = pyro::warp_sum(sig);
    const double cp = GAS_CONSTANT * pyro::warp_sum(cpp);
    const double hvs = pyro::warp_sum(hv), wvs = pyro::warp_sum(wv);
    const double vh = __ldg(V + r);
    const double a = (vh - hvs) / cp;
    if (lane == 0) z[0] = a;
    __syncwarp();
    const double rho = pyro_ld(Pp, p_inc, r) / (GAS_CONSTANT * T * sigma);
    const double* __restrict__ Jr = J + r * NB;
    const double half_chi = 0.5 * chi[r];
    // chi / 2 Lap(v) for component q at this row
    auto lap = [&](int q) {
      const double vc = __ldg(V + (int64_t)q * ldv + r);
      if (!interior) return vc * idx2;
      return (__ldg(V + (int64_t)q * ldv + r - 1) - 2.0 * vc +
              __ldg(V + (int64_t)q * ldv + r + 1)) * idx2;
    };
    for (int k = 0; k < NS; ++k) {
      const double* __restrict__ row = Jr + (int64_t)(k + 1) * FNV;
      double acc = 0.0;
      for (int m = lane; m < FNV; m += 32) acc = fma(__ldg(row + m), z[m], acc);
      acc = pyro::warp_sum(acc);
      if (lane == 0)
        A[(int64_t)(k + 1) * lda + r] = fma(half_chi, lap(k + 1), acc);
    }
    if (lane == 0) {
      const double vr = visc[r] / rho;
      A[r] = fma(half_chi, lap(0), vr * (a * invT + wvs / sigma));
    }
    __syncwarp();
  }
}

PYRO_EXPORT int pyro_flamelet_jacobian_action(
    const double* p, int64_t p_inc, const double* T, const double* Y,
    int64_t ldy, const double* J, const double* V, int64_t ldv,
    const double* chi, const double* visc, const int64_t* row_off,
    const int* sys_of_row, const double* inv_dx2, double* A, int64_t lda,
    int64_t rows, cudaStream_t stream) {
  if (rows < 0 || ldy < rows || ldv < rows || lda < rows)
    return PYRO_ERR_ARGUMENT;
  if (rows == 0) return PYRO_OK;
  if (!p || !T || !Y || !J || !V || !chi || !visc || !row_off ||
      !sys_of_row || !inv_dx2 || !A)
    return PYRO_ERR_ARGUMENT;
  int64_t blocks = (rows * 32 + 127) / 128;
  const int64_t cap = (int64_t)pyro_sm_count() * 32;
  if (blocks > cap) blocks = cap;
  k_flamelet_jacobian_action<<<(int)blocks, 128, 0, stream>>>(
      p, p_inc, T, Y, ldy, J, V, ldv, chi, visc, row_off, sys_of_row, inv_dx2,
      A, lda, rows);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}
