// Batched dense LU factorisation (partial pivoting) and solves for many
// independent small FP64 systems (sm_103a): the per-cell Newton matrices
// M = I - gamma J of the implicit 0-D reactor integrator.  The reference
// solves one reactor's Newton system at a time with jnp.linalg.solve
// (examples/free_flame/time_integ.py:94, LAPACK getrf + getrs); here every
// cell of a batch is factorised in one launch and the factors are kept, so
// the Newton iterations of the following steps only pay for the solves.
//
// Work split: one warp per system, its matrix staged in shared memory with
// a padded row (ld = nv + 1).  Factorisation step k: the warp finds the
// pivot row by a shuffle argmax over lanes (rows), swaps whole rows (the
// LAPACK convention: L's multipliers move with their rows), scales the
// column below the pivot, then each lane owns trailing columns
// j = k+1+lane, k+33+lane and updates them row by row (the multiplier
// A[i][k] is a shared-memory broadcast, A[i][j] a conflict-free row
// segment).  Systems are taken in a grid-stride loop; no waits between
// warps or CTAs.
//
// Layout: M[n][nv][nv] row-major (factorised in place: unit-lower L below
// the diagonal, U on and above), piv[n][nv] (row swapped with k at step
// k); right-hand sides and solutions are addressed with separate system and
// variable strides so both [n][nv] and species-major [nv][n] arrays work.
#include <cstdint>
#include <cuda_runtime.h>

#include "pyro_common.cuh"

namespace {

constexpr int kWarps = 4;  // systems per CTA

__global__ void __launch_bounds__(kWarps * 32)
    k_lu_factor(double* __restrict__ M, int* __restrict__ piv,
                const unsigned char* __restrict__ mask, int n, int nv,
                int* __restrict__ status) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int ld = nv + 1;
  double* A = smem + (size_t)warp * nv * ld;
  for (int64_t s = (int64_t)blockIdx.x * kWarps + warp; s < n;
       s += (int64_t)gridDim.x * kWarps) {
    if (mask && !mask[s]) continue;
    double* Ms = M + s * nv * nv;
    for (int e = lane; e < nv * nv; e += 32) {
      const int i = e / nv;
      A[i * ld + (e - i * nv)] = Ms[e];
    }
    __syncwarp();
    int* ps = piv + s * nv;
    bool singular = false;
    for (int k = 0; k < nv; ++k) {
      // pivot: first row of largest |A[i][k]|, i >= k
      double best = -1.0;
      int bi = k;
      for (int i = k + lane; i < nv; i += 32) {
        const double v = fabs(A[i * ld + k]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) ps[k] = bi;
      if (!(best > 0.0)) {  // zero (or NaN) column: leave the rest as is
        singular = true;
        for (int kk = k + 1 + lane; kk < nv; kk += 32) ps[kk] = kk;
        break;
      }
      if (bi != k)
        for (int j = lane; j < nv; j += 32) {
          const double t = A[k * ld + j];
          A[k * ld + j] = A[bi * ld + j];
          A[bi * ld + j] = t;
        }
      __syncwarp();
      const double inv = 1.0 / A[k * ld + k];
      for (int i = k + 1 + lane; i < nv; i += 32) A[i * ld + k] *= inv;
      __syncwarp();
      const int j0 = k + 1 + lane, j1 = k + 33 + lane;
      const double u0 = j0 < nv ? A[k * ld + j0] : 0.0;
      const double u1 = j1 < nv ? A[k * ld + j1] : 0.0;
      for (int i = k + 1; i < nv; ++i) {
        const double l = A[i * ld + k];
        if (j0 < nv) A[i * ld + j0] = fma(-l, u0, A[i * ld + j0]);
        if (j1 < nv) A[i * ld + j1] = fma(-l, u1, A[i * ld + j1]);
      }
      __syncwarp();
    }
    __syncwarp();
    for (int e = lane; e < nv * nv; e += 32) {
      const int i = e / nv;
      Ms[e] = A[i * ld + (e - i * nv)];
    }
    if (singular && lane == 0 && status) atomicOr(status, 1);
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kWarps * 32)
    k_lu_solve(const double* __restrict__ LU, const int* __restrict__ piv,
               const unsigned char* __restrict__ mask,
               const double* b, int64_t b_ss, int64_t b_vs, double* x,
               int64_t x_ss, int64_t x_vs, int n,
               int nv) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int ld = nv + 1;
  double* A = smem + (size_t)warp * (nv * ld + nv);
  double* r = A + nv * ld;
  for (int64_t s = (int64_t)blockIdx.x * kWarps + warp; s < n;
       s += (int64_t)gridDim.x * kWarps) {
    if (mask && !mask[s]) continue;
    const double* Ls = LU + s * nv * nv;
    for (int e = lane; e < nv * nv; e += 32) {
      const int i = e / nv;
      A[i * ld + (e - i * nv)] = __ldg(Ls + e);
    }
    for (int i = lane; i < nv; i += 32) r[i] = b[s * b_ss + i * b_vs];
    __syncwarp();
    if (lane == 0) {
      const int* ps = piv + s * nv;
      for (int k = 0; k < nv; ++k) {
        const int p = __ldg(ps + k);
        if (p != k && p > k && p < nv) {
          const double t = r[k];
          r[k] = r[p];
          r[p] = t;
        }
      }
    }
    __syncwarp();
    // L y = P b (unit lower), lanes over rows below k
    for (int k = 0; k < nv - 1; ++k) {
      const double rk = r[k];
      for (int i = k + 1 + lane; i < nv; i += 32)
        r[i] = fma(-A[i * ld + k], rk, r[i]);
      __syncwarp();
    }
    // U x = y
    for (int k = nv - 1; k >= 0; --k) {
      if (lane == 0) r[k] = r[k] / A[k * ld + k];
      __syncwarp();
      const double rk = r[k];
      for (int i = lane; i < k; i += 32) r[i] = fma(-A[i * ld + k], rk, r[i]);
      __syncwarp();
    }
    for (int i = lane; i < nv; i += 32) x[s * x_ss + i * x_vs] = r[i];
    __syncwarp();
  }
}

int grid_for(int64_t n) {
  int64_t g = (n + kWarps - 1) / kWarps;
  const int64_t cap = (int64_t)pyro_sm_count() * 32;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

int set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024 &&
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)bytes) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  return PYRO_OK;
}

}  // namespace

// Factorise n matrices M[n][nv][nv] in place (P M = L U, partial pivoting);
// piv[n][nv] receives the row swapped with k at step k.  mask (optional,
// n bytes): only systems with a non-zero byte are touched.  status
// (optional device int): bit 0 set if a pivot column was zero (that
// system's factors are incomplete).  Asynchronous on `stream`.
PYRO_EXPORT int pyro_batched_lu_factor(double* M, int* piv,
                                       const unsigned char* mask, int n,
                                       int nv, int* status,
                                       cudaStream_t stream) {
  if (n < 0 || nv < 1 || nv > 64) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!M || !piv) return PYRO_ERR_ARGUMENT;
  const size_t smem = (size_t)kWarps * nv * (nv + 1) * sizeof(double);
  if (set_smem((const void*)k_lu_factor, smem) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  k_lu_factor<<<grid_for(n), kWarps * 32, smem, stream>>>(M, piv, mask, n,
                                                          nv, status);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

// Solve M_s x_s = b_s for every (unmasked) system with the factors of
// pyro_batched_lu_factor.  b and x are addressed as b[s * b_ss + i * b_vs]
// (b_ss = nv, b_vs = 1 for [n][nv]; b_ss = 1, b_vs = n for species-major
// [nv][n]); x may alias b only with identical strides.  Masked-out systems'
// x are left untouched.  Asynchronous on `stream`.
PYRO_EXPORT int pyro_batched_lu_solve(const double* LU, const int* piv,
                                      const unsigned char* mask,
                                      const double* b, int64_t b_ss,
                                      int64_t b_vs, double* x, int64_t x_ss,
                                      int64_t x_vs, int n, int nv,
                                      cudaStream_t stream) {
  if (n < 0 || nv < 1 || nv > 64) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!LU || !piv || !b || !x) return PYRO_ERR_ARGUMENT;
  const size_t smem =
      (size_t)kWarps * ((size_t)nv * (nv + 1) + nv) * sizeof(double);
  if (set_smem((const void*)k_lu_solve, smem) != PYRO_OK)
    return PYRO_ERR_LAUNCH;
  k_lu_solve<<<grid_for(n), kWarps * 32, smem, stream>>>(
      LU, piv, mask, b, b_ss, b_vs, x, x_ss, x_vs, n, nv);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}
