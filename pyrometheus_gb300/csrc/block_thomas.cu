// Batched block-Thomas solver for block-tridiagonal systems of uneven
// lengths (FP64, sm_103a): the flamelet Newton/time-step linear solve
// (pyrometheus/flamelets/linear_solver.py:6-103).
//
// For one system with diagonal blocks C_i (i < N), sub-diagonal L_i and
// super-diagonal U_i (i < N-1), right-hand side b_i:
//
//   forward:  C'_0 = C_0, b'_0 = b_0,
//             S_i = C'_i^-1 U_i,  t_i = C'_i^-1 b'_i,
//             C'_{i+1} = C_{i+1} - L_i S_i,  b'_{i+1} = b_{i+1} - L_i t_i
//   backward: x_{N-1} = t_{N-1},  x_i = C'_i^-1 (b'_i - U_i x_{i+1})
//
// which is the reference's recurrence.  Each C'_i is LU-factorised once
// with partial pivoting (the LAPACK getrf behind jnp.linalg.solve); its
// factors, pivots and b'_i are kept for the backward solve instead of
// factorising again, as the reference does.
//
// Work split: one CTA per system, the working blocks (C', L, U -> S and the
// previous S) in shared memory, threads parallel over matrix elements /
// right-hand-side columns; a persistent grid takes systems from an atomic
// counter in longest-first order (LPT), so uneven lengths balance across
// SMs in one launch.  Layout (packed, row-major blocks): system s owns rows
// [row_off[s], row_off[s+1]) of C[rows][nv][nv], L, U (the last row's L/U
// unused), b[rows][nv], x[rows][nv]; work holds, per row, the LU factors
// of C'_i, b'_i and the pivots: rows * (nv*nv + 2*nv) doubles.  No waits on other CTAs; the counter is reset
// by the host before each launch.
#include <cstdint>
#include <cuda_runtime.h>

#include "pyro_common.cuh"

namespace {

__device__ __forceinline__ void load_block(double* dst, int ld,
                                           const double* __restrict__ src,
                                           int nv) {
  for (int e = threadIdx.x; e < nv * nv; e += blockDim.x) {
    const int i = e / nv, j = e - (e / nv) * nv;
    dst[i * ld + j] = __ldg(src + e);
  }
}

// In-place LU with partial pivoting of A (nv x nv); piv[k] = row swapped
// with k.  Returns through *singular (shared) when a pivot is zero.
__device__ void lu_factor(double* A, int ld, int nv, int* piv,
                          int* singular) {
  __shared__ double red_v[32];
  __shared__ int red_i[32];
  for (int k = 0; k < nv; ++k) {
    // argmax |A[i][k]|, i >= k (first warp)
    if (threadIdx.x < 32) {
      double best = -1.0;
      int bi = k;
      for (int i = k + threadIdx.x; i < nv; i += 32) {
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
      if (threadIdx.x == 0) {
        red_v[0] = best;
        // the pivot's reciprocal, once for the CTA (the FP64 pipe is
        // narrow: a division repeated by every thread costs more than the
        // whole elimination step of a small block)
        red_v[1] = 1.0 / A[bi * ld + k];
        red_i[0] = bi;
        piv[k] = bi;
        if (best == 0.0) *singular = 1;
      }
    }
    __syncthreads();
    const int p = red_i[0];
    const double inv = red_v[1];
    if (p != k) {
      for (int j = threadIdx.x; j < nv; j += blockDim.x) {
        const double t = A[k * ld + j];
        A[k * ld + j] = A[p * ld + j];
        A[p * ld + j] = t;
      }
      __syncthreads();
    }
    for (int i = k + 1 + threadIdx.x; i < nv; i += blockDim.x)
      A[i * ld + k] *= inv;
    __syncthreads();
    const int m = nv - k - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = k + 1 + e / m, j = k + 1 + (e - (e / m) * m);
      A[i * ld + j] = fma(-A[i * ld + k], A[k * ld + j], A[i * ld + j]);
    }
    __syncthreads();
  }
}

// Solve A X = R for ncol right-hand-side columns of R (in place) with the
// factors and pivots of lu_factor.
__device__ void lu_solve(const double* A, double* R, int ld, int nv,
                         int ncol, int col0, const int* piv) {
  // row permutation
  if (threadIdx.x < 32) {
    for (int k = 0; k < nv; ++k) {
      const int p = piv[k];
      if (p != k)
        for (int c = col0 + threadIdx.x; c < col0 + ncol; c += 32) {
          const double t = R[k * ld + c];
          R[k * ld + c] = R[p * ld + c];
          R[p * ld + c] = t;
        }
      __syncwarp();
    }
  }
  __syncthreads();
  // forward, unit lower
  for (int k = 0; k < nv - 1; ++k) {
    const int m = nv - k - 1;
    for (int e = threadIdx.x; e < m * ncol; e += blockDim.x) {
      const int i = k + 1 + e / ncol, c = col0 + (e - (e / ncol) * ncol);
      R[i * ld + c] = fma(-A[i * ld + k], R[k * ld + c], R[i * ld + c]);
    }
    __syncthreads();
  }
  // backward, upper (the diagonal reciprocals once, in parallel)
  __shared__ double s_invd[64];
  for (int k = threadIdx.x; k < nv; k += blockDim.x)
    s_invd[k] = 1.0 / A[k * ld + k];
  __syncthreads();
  for (int k = nv - 1; k >= 0; --k) {
    const double inv = s_invd[k];
    for (int c = col0 + threadIdx.x; c < col0 + ncol; c += blockDim.x)
      R[k * ld + c] *= inv;
    __syncthreads();
    for (int e = threadIdx.x; e < k * ncol; e += blockDim.x) {
      const int i = e / ncol, c = col0 + (e - (e / ncol) * ncol);
      R[i * ld + c] = fma(-A[i * ld + k], R[k * ld + c], R[i * ld + c]);
    }
    __syncthreads();
  }
}

// One system (rows r0 .. r0+N-1): forward elimination, then the backward
// solves with the kept factors.  All threads of the CTA take part.  Two
// shared blocks: A (C'_i and its factors) and Q, which holds S_{i-1} |
// t_{i-1} for the update C'_i = C_i - L_{i-1} S_{i-1} (L_{i-1} is read
// from global memory: a CTA's threads share each element through L1), then
// U_i | b'_i, solved in place into S_i | t_i for the next row.  Two blocks
// instead of four let four CTAs share an SM at nv = 54.
__device__ void solve_system(const double* __restrict__ Lm,
                             const double* __restrict__ Cm,
                             const double* __restrict__ Um,
                             const double* __restrict__ B,
                             double* __restrict__ X, int64_t r0, int N,
                             int nv, double* __restrict__ work,
                             double* smem, int* s_sing) {
  const int ld = nv + 1;
  double* A = smem;          // C'_i | b'_i, then LU factors | b'_i
  double* Q = A + nv * ld;   // S_{i-1} | t_{i-1}, then U_i | b'_i -> S_i | t_i
  int* piv = (int*)(Q + nv * ld);
  const int64_t wrow = (int64_t)nv * nv + 2 * nv;
  for (int i = 0; i < N; ++i) {
    const int64_t row = r0 + i;
    load_block(A, ld, Cm + row * nv * nv, nv);
    for (int j = threadIdx.x; j < nv; j += blockDim.x)
      A[j * ld + nv] = __ldg(B + row * nv + j);  // b in column nv of A
    __syncthreads();
    if (i > 0) {
      // C' = C - L S_prev ; b' = b - L t_prev (t_prev in column nv of Q)
      const double* __restrict__ Lb = Lm + (row - 1) * nv * nv;
      for (int e = threadIdx.x; e < nv * ld; e += blockDim.x) {
        const int r = e / ld, c = e - (e / ld) * ld;
        double acc = A[r * ld + c];
        for (int k = 0; k < nv; ++k)
          acc = fma(-__ldg(Lb + r * nv + k), Q[k * ld + c], acc);
        A[r * ld + c] = acc;
      }
      __syncthreads();
    }
    // right-hand sides: U_i (if any) and b'_i
    const bool has_u = i < N - 1;
    if (has_u) load_block(Q, ld, Um + row * nv * nv, nv);
    for (int j = threadIdx.x; j < nv; j += blockDim.x)
      Q[j * ld + nv] = A[j * ld + nv];
    __syncthreads();
    lu_factor(A, ld, nv, piv, s_sing);
    // keep the factors, b'_i and the pivots for the backward solve
    double* w = work + row * wrow;
    for (int e = threadIdx.x; e < nv * ld; e += blockDim.x) {
      const int r = e / ld, c = e - (e / ld) * ld;
      if (c < nv)
        w[r * nv + c] = A[e];
      else
        w[nv * nv + r] = A[e];
    }
    for (int k = threadIdx.x; k < nv; k += blockDim.x)
      w[nv * nv + nv + k] = (double)piv[k];
    if (has_u)
      lu_solve(A, Q, ld, nv, nv + 1, 0, piv);
    else
      lu_solve(A, Q, ld, nv, 1, nv, piv);
  }
  // backward: x_{N-1} = t_{N-1}; x_i = C'_i^-1 (b'_i - U_i x_{i+1}).
  // x_{i+1} lives in the first nv entries of Q (row 0 of the block); the
  // right-hand side column nv sits at indices >= nv.
  double* xs = Q;
  {
    const int64_t row = r0 + N - 1;
    for (int j = threadIdx.x; j < nv; j += blockDim.x) {
      const double v = Q[j * ld + nv];
      X[row * nv + j] = v;
      xs[j] = v;
    }
    __syncthreads();
  }
  for (int i = N - 2; i >= 0; --i) {
    const int64_t row = r0 + i;
    const double* w = work + row * wrow;
    const double* Ui = Um + row * nv * nv;
    for (int e = threadIdx.x; e < nv * nv; e += blockDim.x) {
      const int r = e / nv, c = e - (e / nv) * nv;
      A[r * ld + c] = w[e];
    }
    for (int j = threadIdx.x; j < nv; j += blockDim.x) {
      double v = w[nv * nv + j];
      for (int k = 0; k < nv; ++k) v = fma(-__ldg(Ui + j * nv + k), xs[k], v);
      Q[j * ld + nv] = v;  // column nv: disjoint from xs
      piv[j] = (int)w[nv * nv + nv + j];
    }
    __syncthreads();
    lu_solve(A, Q, ld, nv, 1, nv, piv);
    for (int j = threadIdx.x; j < nv; j += blockDim.x) {
      const double v = Q[j * ld + nv];
      X[row * nv + j] = v;
      xs[j] = v;
    }
    __syncthreads();
  }
}

__global__ void k_block_thomas(const double* __restrict__ Lm,
                               const double* __restrict__ Cm,
                               const double* __restrict__ Um,
                               const double* __restrict__ B,
                               double* __restrict__ X,
                               const int64_t* __restrict__ row_off,
                               const int* __restrict__ order, int nsys,
                               int nv, double* __restrict__ work,
                               int* __restrict__ counter,
                               int* __restrict__ status) {
  extern __shared__ double smem[];
  __shared__ int s_sys;
  __shared__ int s_sing;
  for (;;) {
    if (threadIdx.x == 0) {
      s_sys = atomicAdd(counter, 1);
      s_sing = 0;
    }
    __syncthreads();
    const int q = s_sys;
    if (q >= nsys) break;
    const int s = order[q];
    const int64_t r0 = row_off[s];
    const int64_t n64 = row_off[s + 1] - r0;
    if (n64 <= 0) {  // an empty row range: skipped and flagged
      if (threadIdx.x == 0 && status) atomicOr(status, 2);
      __syncthreads();
      continue;
    }
    solve_system(Lm, Cm, Um, B, X, r0, (int)n64, nv, work, smem, &s_sing);
    if (threadIdx.x == 0 && s_sing && status) atomicOr(status, 1);
    __syncthreads();
  }
}


// ------------------------------------------------------------------------
// Small blocks (nv <= 16): one thread per system.
//
// On GB300 a warp-wide FP64 instruction occupies the FP64 pipe for the same
// time however few of its lanes are active, so the CTA-per-system kernel
// above, whose 10 x 10 steps keep only a few lanes busy, is bound by
// partially empty FP64 instructions.  Here each thread runs one system's
// whole recurrence (same algorithm, same per-row workspace layout), so every
// FP64 instruction does 32 useful operations; the thread's blocks live in
// shared memory interleaved by thread ([element][thread]: a warp's accesses
// to one element are 32 consecutive doubles, conflict-free).  Systems are
// handed out in the caller's order (longest first), so the threads of a
// warp get systems of similar length.
template <int NV>
__global__ void __launch_bounds__(64)
    k_block_thomas_small(const double* __restrict__ Lm,
                         const double* __restrict__ Cm,
                         const double* __restrict__ Um,
                         const double* __restrict__ B, double* __restrict__ X,
                         const int64_t* __restrict__ row_off,
                         const int* __restrict__ order, int nsys,
                         double* __restrict__ work, int* __restrict__ status) {
  extern __shared__ double smem[];
  constexpr int LD = NV + 1;
  constexpr int BLK = NV * LD;
  const int T = blockDim.x;
  const int q = blockIdx.x * T + threadIdx.x;
  if (q >= nsys) return;  // no block-wide synchronisation below
  double* A = smem + threadIdx.x;  // C'_i | b'_i, then LU | b'_i
  double* R = A + (size_t)BLK * T;  // U_i | b'_i -> S_i | t_i
  double* P = R + (size_t)BLK * T;  // S_{i-1} | t_{i-1}
#define EA(i, j) A[((i) * LD + (j)) * T]
#define ER(i, j) R[((i) * LD + (j)) * T]
#define EP(i, j) P[((i) * LD + (j)) * T]
  const int s = order[q];
  const int64_t r0 = row_off[s];
  const int64_t n64 = row_off[s + 1] - r0;
  if (n64 <= 0) {  // an empty row range: skipped and flagged
    if (status) atomicOr(status, 2);
    return;
  }
  const int N = (int)n64;
  constexpr int64_t WROW = (int64_t)NV * NV + 2 * NV;
  bool singular = false;
  for (int i = 0; i < N; ++i) {
    const int64_t row = r0 + i;
    const double* Ci = Cm + row * NV * NV;
    double* w = work + row * WROW;
    for (int r = 0; r < NV; ++r) {
#pragma unroll
      for (int c = 0; c < NV; ++c) EA(r, c) = __ldg(Ci + r * NV + c);
      EA(r, NV) = __ldg(B + row * NV + r);
    }
    if (i > 0) {
      // C' = C - L S_prev ; b' = b - L t_prev
      const double* Li = Lm + (row - 1) * NV * NV;
      for (int r = 0; r < NV; ++r) {
        double l[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) l[k] = __ldg(Li + r * NV + k);
#pragma unroll
        for (int c = 0; c < LD; ++c) {
          double acc = EA(r, c);
#pragma unroll
          for (int k = 0; k < NV; ++k) acc = fma(-l[k], EP(k, c), acc);
          EA(r, c) = acc;
        }
      }
    }
    // LU with partial pivoting of the NV x NV part (b' column untouched);
    // the pivots go straight to the workspace row
    for (int k = 0; k < NV; ++k) {
      int p = k;
      double best = fabs(EA(k, k));
      for (int r = k + 1; r < NV; ++r) {
        const double v = fabs(EA(r, k));
        if (v > best) {
          best = v;
          p = r;
        }
      }
      w[NV * NV + NV + k] = (double)p;
      if (best == 0.0) singular = true;
      if (p != k) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
          const double t = EA(k, c);
          EA(k, c) = EA(p, c);
          EA(p, c) = t;
        }
      }
      const double inv = 1.0 / EA(k, k);
      for (int r = k + 1; r < NV; ++r) {
        const double lrk = EA(r, k) * inv;
        EA(r, k) = lrk;
        for (int c = k + 1; c < NV; ++c)
          EA(r, c) = fma(-lrk, EA(k, c), EA(r, c));
      }
    }
    // keep the factors and b'_i for the backward solve
    for (int r = 0; r < NV; ++r) {
#pragma unroll
      for (int c = 0; c < NV; ++c) w[r * NV + c] = EA(r, c);
      w[NV * NV + r] = EA(r, NV);
    }
    // S_i | t_i = C'_i^-1 (U_i | b'_i)  (only t_i on the last row)
    const bool has_u = i < N - 1;
    const double* Ui = Um + row * NV * NV;
    for (int r = 0; r < NV; ++r) {
      if (has_u) {
#pragma unroll
        for (int c = 0; c < NV; ++c) ER(r, c) = __ldg(Ui + r * NV + c);
      }
      ER(r, NV) = EA(r, NV);
    }
    for (int k = 0; k < NV; ++k) {
      const int p = (int)w[NV * NV + NV + k];
      if (p != k) {
        for (int c = has_u ? 0 : NV; c < LD; ++c) {
          const double t = ER(k, c);
          ER(k, c) = ER(p, c);
          ER(p, c) = t;
        }
      }
    }
    for (int k = 0; k < NV - 1; ++k)
      for (int r = k + 1; r < NV; ++r) {
        const double l = EA(r, k);
        for (int c = has_u ? 0 : NV; c < LD; ++c)
          ER(r, c) = fma(-l, ER(k, c), ER(r, c));
      }
    for (int k = NV - 1; k >= 0; --k) {
      const double inv = 1.0 / EA(k, k);
      for (int c = has_u ? 0 : NV; c < LD; ++c) ER(k, c) *= inv;
      for (int r = 0; r < k; ++r) {
        const double u = EA(r, k);
        for (int c = has_u ? 0 : NV; c < LD; ++c)
          ER(r, c) = fma(-u, ER(k, c), ER(r, c));
      }
    }
    double* tmp = P;
    P = R;
    R = tmp;
  }
  // backward: x_{N-1} = t_{N-1}; x_i = C'_i^-1 (b'_i - U_i x_{i+1}), with
  // x_{i+1} kept in the R block's last column
  {
    const int64_t row = r0 + N - 1;
    for (int r = 0; r < NV; ++r) {
      const double v = EP(r, NV);
      ER(r, NV) = v;
      X[row * NV + r] = v;
    }
  }
  for (int i = N - 2; i >= 0; --i) {
    const int64_t row = r0 + i;
    const double* w = work + row * WROW;
    const double* Ui = Um + row * NV * NV;
    // A's last column <- b'_i - U_i x_{i+1}
    for (int r = 0; r < NV; ++r) {
      double a = w[NV * NV + r];
#pragma unroll
      for (int k = 0; k < NV; ++k)
        a = fma(-__ldg(Ui + r * NV + k), ER(k, NV), a);
      EA(r, NV) = a;
    }
    for (int k = 0; k < NV; ++k) {
      const int p = (int)w[NV * NV + NV + k];
      if (p != k) {
        const double t = EA(k, NV);
        EA(k, NV) = EA(p, NV);
        EA(p, NV) = t;
      }
    }
    for (int k = 0; k < NV - 1; ++k) {
      const double v = EA(k, NV);
      for (int r = k + 1; r < NV; ++r)
        EA(r, NV) = fma(-w[r * NV + k], v, EA(r, NV));
    }
    for (int k = NV - 1; k >= 0; --k) {
      const double v = EA(k, NV) / w[k * NV + k];
      EA(k, NV) = v;
      for (int r = 0; r < k; ++r)
        EA(r, NV) = fma(-w[r * NV + k], v, EA(r, NV));
    }
    for (int r = 0; r < NV; ++r) {
      const double v = EA(r, NV);
      ER(r, NV) = v;
      X[row * NV + r] = v;
    }
  }
  if (singular && status) atomicOr(status, 1);
#undef EA
#undef ER
#undef EP
}

template <int NV>
int launch_small(const double* L, const double* C, const double* U,
                 const double* b, double* x, const int64_t* row_off,
                 const int* order, int nsys, double* work, int* status,
                 int threads, cudaStream_t stream) {
  const size_t smem = (size_t)3 * NV * (NV + 1) * threads * sizeof(double);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute((const void*)k_block_thomas_small<NV>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  const int grid = (nsys + threads - 1) / threads;
  k_block_thomas_small<NV><<<grid, threads, smem, stream>>>(
      L, C, U, b, x, row_off, order, nsys, work, status);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

}  // namespace

// Doubles of workspace pyro_block_thomas needs for `rows` packed rows: per
// row the factors, b' and the pivots; for nv <= 16 (the segmented kernel)
// then S_i | t_i of every row after them.
PYRO_EXPORT int64_t pyro_block_thomas_work_doubles(int nv, int64_t rows) {
  const int64_t st = nv <= 16 ? (int64_t)nv * (nv + 1) : 0;
  return rows * ((int64_t)nv * nv + 2 * nv + st);
}

// Shared memory of one CTA for block size nv.
PYRO_EXPORT int64_t pyro_block_thomas_smem_bytes(int nv) {
  return (int64_t)2 * nv * (nv + 1) * 8 + (int64_t)nv * 4;
}

// Solve nsys block-tridiagonal systems (packed as described above).
// order: a permutation of 0..nsys-1 (longest first balances best); counter
// and status: device ints (counter is zeroed here, status gets bit 0 set
// for a zero pivot and bit 1 for a system with an empty row range, which is
// skipped); threads: CTA size (multiple of 32, <= 1024); ctas: grid size
// (0: as many as fit, resident).  Asynchronous on `stream`.
PYRO_EXPORT int pyro_block_thomas(const double* L, const double* C,
                                  const double* U, const double* b, double* x,
                                  const int64_t* row_off, const int* order,
                                  int nsys, int nv, double* work, int* counter,
                                  int* status, int threads, int ctas,
                                  cudaStream_t stream) {
  if (nsys < 0 || nv < 1 || nv > 64 || threads < 32 || threads > 1024 ||
      threads % 32)
    return PYRO_ERR_ARGUMENT;
  if (nsys == 0) return PYRO_OK;
  if (!L || !C || !U || !b || !x || !row_off || !order || !work || !counter)
    return PYRO_ERR_ARGUMENT;
  const size_t smem = (size_t)pyro_block_thomas_smem_bytes(nv);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute((const void*)k_block_thomas,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  if (ctas <= 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, k_block_thomas, threads, smem) != cudaSuccess ||
        per_sm < 1) {
      (void)cudaGetLastError();
      per_sm = 1;
    }
    ctas = per_sm * pyro_sm_count();
  }
  if (ctas > nsys) ctas = nsys;
  if (cudaMemsetAsync(counter, 0, sizeof(int), stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  k_block_thomas<<<ctas, threads, smem, stream>>>(L, C, U, b, x, row_off,
                                                  order, nsys, nv, work,
                                                  counter, status);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

// pyro_block_thomas for blocks of size nv <= 16 with one thread per system
// (same arguments minus the counter; threads = systems per CTA, 32 or 64).
// The workspace layout is the same as pyro_block_thomas's.
PYRO_EXPORT int pyro_block_thomas_small(const double* L, const double* C,
                                        const double* U, const double* b,
                                        double* x, const int64_t* row_off,
                                        const int* order, int nsys, int nv,
                                        double* work, int* status,
                                        int threads, cudaStream_t stream) {
  if (nsys < 0 || nv < 1 || nv > 16 || (threads != 32 && threads != 64))
    return PYRO_ERR_ARGUMENT;
  if (nsys == 0) return PYRO_OK;
  if (!L || !C || !U || !b || !x || !row_off || !order || !work)
    return PYRO_ERR_ARGUMENT;
  if ((size_t)3 * nv * (nv + 1) * threads * sizeof(double) > 227 * 1024)
    return PYRO_ERR_ARGUMENT;
  switch (nv) {
#define PYRO_BT_SMALL(NV)                                                    \
  case NV:                                                                   \
    return launch_small<NV>(L, C, U, b, x, row_off, order, nsys, work,       \
                            status, threads, stream);
    PYRO_BT_SMALL(1) PYRO_BT_SMALL(2) PYRO_BT_SMALL(3) PYRO_BT_SMALL(4)
    PYRO_BT_SMALL(5) PYRO_BT_SMALL(6) PYRO_BT_SMALL(7) PYRO_BT_SMALL(8)
    PYRO_BT_SMALL(9) PYRO_BT_SMALL(10) PYRO_BT_SMALL(11) PYRO_BT_SMALL(12)
    PYRO_BT_SMALL(13) PYRO_BT_SMALL(14) PYRO_BT_SMALL(15) PYRO_BT_SMALL(16)
#undef PYRO_BT_SMALL
    default:
      return PYRO_ERR_ARGUMENT;
  }
}

// ------------------------------------------------------------------------
// Small blocks, several systems per warp (nv <= 16).
//
// A warp-wide FP64 instruction costs GB300's narrow FP64 pipe the same
// however many of its lanes are active (each SM partition retires one every
// 64 cycles, and a dependent one no sooner), so small blocks need every lane
// busy, and the CTA-per-system kernel above, whose 10 x 10 steps keep a few
// lanes busy between barriers, cannot.  Here a system takes a segment of NV
// consecutive lanes (P = 32 / NV segments per warp: three at nv = 10) and
// lane r of a segment holds row r of the system's working blocks in
// registers; nothing synchronises beyond the warp.
//
// Balance.  With the FP64 pipe of an SM partition the bound, the solve
// takes as long as the busiest partition's FP64 instructions, so the work
// is spread in units of one system per segment, not one warp's worth: the
// grid is persistent (one warp per SM partition by default) and a segment
// whose system is done takes the next one from the caller's order (longest
// first), so every segment stays busy until the queue is empty.  Segments
// of one warp are then at different rows of different systems, in lockstep
// only as instruction streams; the forward and backward sweeps are two
// kernels (two launches on the stream) so that every warp step runs one
// sweep's instructions for all its segments.
//
// Forward sweep, per block row: C'_i | b'_i = (C_i | b_i) - L_{i-1}
// (S_{i-1} | t_{i-1}) with S_{i-1} | t_{i-1} read from warp-private shared
// memory; then one elimination pass over [C'_i | U_i | b'_i] with partial
// pivoting.  Row interchanges are relabellings (a lane keeps its row and
// tracks the position LAPACK's swaps would move it to); the pivot is the
// largest |a| of the eligible rows, ties to the lowest position, as getrf
// chooses it (up to candidates equal to 2^-16 relative, see pivot_key).
// Below the pivot the pass is LU's elimination (its multipliers and the
// pivot rows are exactly getrf's factors, kept in the workspace in the
// layout of the kernels above); above the pivot it also eliminates
// (Gauss-Jordan), which in SIMT costs nothing extra: the lanes of rows above
// the pivot run the same instructions as the others.  Each lane's
// right-hand-side row, scaled by its pivot's reciprocal, is then row
// `pivot step` of S_i | t_i, kept in shared memory for the next row and in
// the workspace for the backward sweep; t_{N-1} = x_{N-1} goes to x.  The
// backward sweep is x_i = t_i - S_i x_{i+1}, the reference's x_i = C'_i^-1
// (b'_i - U_i x_{i+1}) with C'_i^-1 applied in the forward sweep; the LU
// factors are kept as well, for pyro_block_thomas_resolve.

namespace {

// warps per CTA of the sweeps: four, so that a CTA's warps sit on the four
// partitions of its SM
constexpr int kSegWarps = 4;

template <int NV>
struct SegCfg {
  static constexpr int P = 32 / NV;         // systems per warp
  static constexpr int RS = NV + 1;         // shared row stride (S | t)
  static constexpr int SMEM = P * NV * RS;  // doubles per warp
};

// Pivot key of an eligible row: the top 27 bits of |v|'s bit pattern
// (exponent and 16 mantissa bits, which order like |v|), then 15 - position
// in the low 4 bits, so one unsigned max picks the largest |v| and, among
// candidates equal to 2^-16 relative, the lowest position -- getrf's
// choice up to those near-ties.  NaN and zero rank lowest (key bits 0);
// rows already pivoted are not candidates (key 0, below every candidate
// through the position bits being at most 15 and eligibility ORed in).
__device__ __forceinline__ unsigned pivot_key(double v, int pos) {
  const unsigned long long b =
      (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
  const unsigned top =
      b > 0x7ff0000000000000ULL ? 0u : (unsigned)(b >> 36);  // 27 bits
  return (top << 5) | 16u | (unsigned)(15 - pos);
}

// Lane geometry of the segmented kernels: segment, row in it, first lane,
// and the segment as a lane mask (the lanes past the last segment, 32 mod
// NV of them, own no system and form one group of their own).
template <int NV>
struct SegLane {
  int lane, seg, r, base;
  bool in_seg;
  unsigned mask;
  __device__ SegLane() {
    constexpr int P = SegCfg<NV>::P;
    lane = threadIdx.x & 31;
    seg = lane / NV;
    r = lane - seg * NV;
    base = seg * NV;
    in_seg = seg < P;
    mask = in_seg ? (((1u << NV) - 1u) << base)
                  : (P * NV >= 32 ? 0u : ~((1u << (P * NV)) - 1u));
  }
};

// Queue step of the segmented kernels: every segment that needs a system
// takes the next position of the order (one atomic per segment, read by
// its lanes); returns the position, or nsys and beyond when the queue is
// empty.  All lanes of the warp call it.
template <int NV>
__device__ __forceinline__ int seg_fetch(const SegLane<NV>& g, bool need,
                                         int* __restrict__ counter) {
  int q = 0;
  if (need && g.r == 0) q = atomicAdd(counter, 1);
  return __shfl_sync(0xffffffffu, q, g.in_seg ? g.base : 0);
}

// Segmented maximum of a 32-bit key: every lane gets the largest key of its
// segment.  Up to four segments per warp, one full-warp redux.sync per
// segment (the others contributing 0), independent of one another; more
// segments, shuffle rounds with offsets 1, 2, 4, 8 inside the segment
// (after them each lane holds the largest key of positions [r, r +
// 2^rounds) mod NV).
template <int NV>
__device__ __forceinline__ unsigned seg_max(const SegLane<NV>& g,
                                            unsigned key) {
  using Cfg = SegCfg<NV>;
  unsigned best = 0u;
  if constexpr (Cfg::P <= 4) {
#pragma unroll
    for (int s = 0; s < Cfg::P; ++s) {
      const unsigned m = __reduce_max_sync(0xffffffffu, g.seg == s ? key : 0u);
      if (g.seg == s) best = m;
    }
  } else {
    constexpr int rounds = NV <= 1 ? 0 : NV <= 2 ? 1 : NV <= 4 ? 2 : 3;
    best = key;
#pragma unroll
    for (int o = 0, off = 1; o < rounds; ++o, off <<= 1) {
      const int rr = g.r + off;
      const int src = g.base + (rr >= NV ? rr - NV : rr);
      best = max(best, __shfl_sync(0xffffffffu, best, src));
    }
  }
  return best;
}

// L2 prefetch of the 8 n bytes at p (both ends, which may sit in two
// lines).
template <int N>
__device__ __forceinline__ void prefetch_row(const double* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p + N - 1));
}

// Elimination of one block row held by a segment, lane r holding row r of
// [A | R] in a[0..NV) | a[NV..NC): Gauss-Jordan with relabelled partial
// pivoting, software-pipelined -- as soon as step k has updated column
// k + 1, the pivot of step k + 1 is searched (key maximum over the segment,
// ballot) and every lane takes the reciprocal of its own candidate (the
// pivot lane's is shuffled out), all under step k's remaining updates.  On
// entry `best` is the segment maximum of column 0's keys and `rc` this
// lane's pyro_rcp3(a[0]).  On return lu holds this lane's row of getrf's
// factors (its position in getrf's row order is myk), mypiv getrf's pivot
// of step r, and a[NV..NC) * myinv is row myk of A^-1 R; singular is set on
// a zero pivot of an active segment.
template <int NV, int NC>
__device__ __forceinline__ void seg_eliminate(const SegLane<NV>& g, bool act,
                                              double (&a)[NC], unsigned best,
                                              double rc, double (&lu)[NV],
                                              int& myk, int& mypiv,
                                              double& myinv, bool& singular) {
  constexpr unsigned full = 0xffffffffu;
  const int r = g.r, lane = g.lane;
  int pos = r;
  bool elig = true;
  myk = 0;
  mypiv = 0;
  myinv = 0.0;
  int bp = 15 - (int)(best & 15u);
  int bl = __ffs(__ballot_sync(full, pos == bp) & g.mask) - 1;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    if ((best >> 5) == 0 && act) singular = true;
    if (r == k) mypiv = bp;
    const bool is_piv = lane == bl;
    const double inv = __shfl_sync(full, rc, bl);
    const double m = is_piv ? 0.0 : a[k] * inv;
    if (elig && !is_piv) lu[k] = m;  // getrf's multiplier
    if (is_piv) {
#pragma unroll
      for (int j = k; j < NV; ++j) lu[j] = a[j];  // getrf's U row
      myinv = inv;
      myk = k;
    }
    if (pos == k) pos = bp;
    if (is_piv) {
      pos = k;
      elig = false;
    }
    int nbl = bl;
    if (k + 1 < NV) {
      const double p1 = __shfl_sync(full, a[k + 1], bl);
      a[k + 1] = fma(-m, p1, a[k + 1]);
      best = seg_max(g, elig ? pivot_key(a[k + 1], pos) : 0u);
      rc = pyro_rcp3(a[k + 1]);
      bp = 15 - (int)(best & 15u);
      nbl = __ffs(__ballot_sync(full, elig && pos == bp) & g.mask) - 1;
    }
#pragma unroll
    for (int j = (k + 1 < NV ? k + 2 : k + 1); j < NC; ++j) {
      const double pj = __shfl_sync(full, a[j], bl);
      a[j] = fma(-m, pj, a[j]);
    }
    bl = nbl;
  }
}

// Rows and split of a system of the two-ended sweeps: N rows, the middle
// row m = N / 2; unit 0 eliminates rows 0 .. m-1 downwards, unit 1 rows
// N-1 .. m+1 upwards.
__device__ __forceinline__ int seg_unit_rows(int N, int dir) {
  const int m = N >> 1;
  const int c = dir == 0 ? m : N - 1 - m;
  return c > 0 ? c : 0;
}

// Forward sweeps: every segment takes units (system, direction) from the
// queue -- position q is direction q & 1 of system order[q >> 1] -- and
// eliminates the unit's rows in order.  Step t of a downward unit is row
// i = t: C'_i | b'_i = (C_i | b_i) - L_{i-1} (S_{i-1} | t_{i-1}), then the
// elimination over [C'_i | U_i | b'_i]; of an upward unit row i = N-1-t:
// C^_i | b^_i = (C_i | b_i) - U_i (S^_{i+1} | t^_{i+1}), then the
// elimination over [C^_i | L_{i-1} | b^_i].  The factors go to row i of the
// workspace, S_i | t_i (or S^_i | t^_i) to the S | t region and, for the
// unit's next row, to the warp's shared memory.
template <int NV>
__global__ void __launch_bounds__(kSegWarps * 32)
    k_block_thomas_seg(const double* __restrict__ Lm,
                       const double* __restrict__ Cm,
                       const double* __restrict__ Um,
                       const double* __restrict__ B,
                       const int64_t* __restrict__ row_off,
                       const int* __restrict__ order, int nsys,
                       double* __restrict__ work, int* __restrict__ counter,
                       int* __restrict__ status) {
  using Cfg = SegCfg<NV>;
  constexpr int RS = Cfg::RS, NC = 2 * NV + 1;
  constexpr int64_t NN = (int64_t)NV * NV, WROW = NN + 2 * NV,
                    SROW = (int64_t)NV * RS;
  constexpr unsigned full = 0xffffffffu;
  __shared__ double s_st[kSegWarps][Cfg::SMEM];
  const SegLane<NV> g;
  const int r = g.r;
  // lanes past the last segment read segment 0's rows, never write them
  double* st = s_st[threadIdx.x >> 5] + (g.in_seg ? g.seg : 0) * NV * RS;
  // the previous row's S | t is kept finite between units (zero before the
  // first and after every last row), so the update runs branch-free with
  // zero couplings on a unit's first row
  for (int e = g.lane; e < Cfg::SMEM; e += 32)
    s_st[threadIdx.x >> 5][e] = 0.0;
  __syncwarp();
  double* __restrict__ sg = work + row_off[nsys] * WROW;
  bool live = g.in_seg;  // the segment may still take units
  int N = 0, dir = 0, cnt = 0, t = 0;
  int64_t r0 = 0;
  bool singular = false;
  for (;;) {
    const bool need = live && t >= cnt;
    const int q = seg_fetch(g, need, counter);
    if (need) {
      if (q >= 2 * nsys) {
        live = false;
      } else {
        const int s = order[q >> 1];
        dir = q & 1;
        r0 = row_off[s];
        const int64_t n64 = row_off[s + 1] - r0;
        // an empty (or inverted) row range is skipped and flagged
        N = n64 > 0 ? (int)n64 : 0;
        cnt = seg_unit_rows(N, dir);
        t = 0;
        if (n64 <= 0 && dir == 0 && r == 0 && status) atomicOr(status, 2);
      }
    }
    if (!__any_sync(full, live)) break;
    const bool act = live && t < cnt;
    const bool down = dir == 0;
    const int i = down ? t : N - 1 - t;
    const int64_t row = r0 + i;
    // coupling to the row eliminated before (L_{i-1} down, U_i up) and the
    // right-hand-side block (U_i down, L_{i-1} up)
    const double* __restrict__ Pm = down ? Lm : Um;
    const double* __restrict__ Qm = down ? Um : Lm;
    const int64_t prow = down ? row - 1 : row, qrow = down ? row : row - 1;
    double a[NC], l[NV];
    if (act) {
      if (t + 1 < cnt) {
        // the next row's blocks to L2 while this one is worked on
        const int64_t step = down ? 1 : -1;
        prefetch_row<NV>(Cm + (row + step) * NN + r * NV);
        prefetch_row<NV>(Pm + (prow + step) * NN + r * NV);
        prefetch_row<NV>(Qm + (qrow + step) * NN + r * NV);
      }
      const double* __restrict__ Ci = Cm + row * NN + r * NV;
      const double* __restrict__ Qi = Qm + qrow * NN + r * NV;
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        a[j] = __ldg(Ci + j);
        a[NV + j] = __ldg(Qi + j);
      }
      a[2 * NV] = __ldg(B + row * NV + r);
      // (a unit's first row has no coupling; its address stays in bounds)
      const double* __restrict__ Pi = Pm + (t > 0 ? prow : row) * NN + r * NV;
#pragma unroll
      for (int k = 0; k < NV; ++k) l[k] = t > 0 ? __ldg(Pi + k) : 0.0;
    } else {
#pragma unroll
      for (int j = 0; j < NC; ++j) a[j] = 0.0;
#pragma unroll
      for (int k = 0; k < NV; ++k) l[k] = 0.0;
    }
    // C' = C - P S_prev, b' = b - P t_prev (S | t in shared memory), column
    // 0 first so that its pivot search starts under the other columns'
    // updates
#pragma unroll
    for (int k = 0; k < NV; ++k) a[0] = fma(-l[k], st[k * RS], a[0]);
    const unsigned best = seg_max(g, pivot_key(a[0], r));
    const double rc = pyro_rcp3(a[0]);
#pragma unroll
    for (int j = 1; j < NV; ++j) {
#pragma unroll
      for (int k = 0; k < NV; ++k) a[j] = fma(-l[k], st[k * RS + j], a[j]);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k)
      a[2 * NV] = fma(-l[k], st[k * RS + NV], a[2 * NV]);
    double* __restrict__ w = work + row * WROW;
    if (act) w[NN + r] = a[2 * NV];  // b'_i, original row order
    __syncwarp();
    int myk, mypiv;
    double myinv, lu[NV];
    seg_eliminate<NV, NC>(g, act, a, best, rc, lu, myk, mypiv, myinv,
                          singular);
    if (act) {
      // factors in getrf's row order (position myk), pivots as swaps
      double* __restrict__ wf = w + myk * NV;
#pragma unroll
      for (int j = 0; j < NV; ++j) wf[j] = lu[j];
      w[NN + NV + r] = (double)mypiv;
      // row myk of S_i | t_i: for the unit's next row (shared memory, zeros
      // after its last row) and the backward sweeps (workspace)
      const bool last = t == cnt - 1;
      double* __restrict__ sgr = sg + row * SROW + myk * RS;
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        const double sj = a[NV + j] * myinv;
        st[myk * RS + j] = last ? 0.0 : sj;
        sgr[j] = sj;
      }
      const double tk = a[2 * NV] * myinv;
      st[myk * RS + NV] = last ? 0.0 : tk;
      sgr[NV] = tk;
      if (last) {
        if (singular && r == 0 && status) atomicOr(status, 1);
        singular = false;
      }
      ++t;
    }
    __syncwarp();
  }
}

// Middle rows: for every system, row m = N / 2 couples to both sweeps,
// (C_m - L_{m-1} S_{m-1} - U_m S^_{m+1}) x_m = b_m - L_{m-1} t_{m-1} -
// U_m t^_{m+1} (a missing side drops out); one elimination per system,
// factors kept at row m, x_m to x.
template <int NV>
__global__ void __launch_bounds__(kSegWarps * 32)
    k_block_thomas_seg_mid(const double* __restrict__ Lm,
                           const double* __restrict__ Cm,
                           const double* __restrict__ Um,
                           const double* __restrict__ B,
                           double* __restrict__ X,
                           const int64_t* __restrict__ row_off,
                           const int* __restrict__ order, int nsys,
                           double* __restrict__ work,
                           int* __restrict__ counter,
                           int* __restrict__ status) {
  constexpr int RS = SegCfg<NV>::RS, NC = NV + 1;
  constexpr int64_t NN = (int64_t)NV * NV, WROW = NN + 2 * NV,
                    SROW = (int64_t)NV * RS;
  constexpr unsigned full = 0xffffffffu;
  const SegLane<NV> g;
  const int r = g.r;
  const double* __restrict__ sg = work + row_off[nsys] * WROW;
  bool live = g.in_seg;
  for (;;) {
    const int q = seg_fetch(g, live, counter);
    int N = 0;
    int64_t r0 = 0;
    if (live) {
      if (q >= nsys) {
        live = false;
      } else {
        const int s = order[q];
        r0 = row_off[s];
        const int64_t n64 = row_off[s + 1] - r0;
        N = n64 > 0 ? (int)n64 : 0;
      }
    }
    if (!__any_sync(full, live)) break;
    const bool act = live && N > 0;
    const int m = N >> 1;
    const int64_t row = r0 + m;
    double a[NC];
    if (act) {
      const double* __restrict__ Ci = Cm + row * NN + r * NV;
#pragma unroll
      for (int j = 0; j < NV; ++j) a[j] = __ldg(Ci + j);
      a[NV] = __ldg(B + row * NV + r);
      if (m >= 1) {
        const double* __restrict__ Li = Lm + (row - 1) * NN + r * NV;
        const double* __restrict__ S = sg + (row - 1) * SROW;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const double lk = __ldg(Li + k);
#pragma unroll
          for (int j = 0; j < NC; ++j) a[j] = fma(-lk, S[k * RS + j], a[j]);
        }
      }
      if (m + 1 <= N - 1) {
        const double* __restrict__ Ui = Um + row * NN + r * NV;
        const double* __restrict__ S = sg + (row + 1) * SROW;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const double uk = __ldg(Ui + k);
#pragma unroll
          for (int j = 0; j < NC; ++j) a[j] = fma(-uk, S[k * RS + j], a[j]);
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < NC; ++j) a[j] = 0.0;
    }
    double* __restrict__ w = work + row * WROW;
    if (act) w[NN + r] = a[NV];
    const unsigned best = seg_max(g, pivot_key(a[0], r));
    const double rc = pyro_rcp3(a[0]);
    int myk, mypiv;
    double myinv, lu[NV];
    bool singular = false;
    seg_eliminate<NV, NC>(g, act, a, best, rc, lu, myk, mypiv, myinv,
                          singular);
    if (act) {
      double* __restrict__ wf = w + myk * NV;
#pragma unroll
      for (int j = 0; j < NV; ++j) wf[j] = lu[j];
      w[NN + NV + r] = (double)mypiv;
      X[row * NV + myk] = a[NV] * myinv;
      if (singular && r == 0 && status) atomicOr(status, 1);
    }
  }
}

// Backward sweeps from the middle row: unit (system, direction) as in the
// forward kernel; downwards x_i = t_i - S_i x_{i+1} for i = m-1 .. 0,
// upwards x_i = t^_i - S^_i x_{i-1} for i = m+1 .. N-1, starting from x_m.
template <int NV>
__global__ void __launch_bounds__(kSegWarps * 32)
    k_block_thomas_seg_back(double* __restrict__ X,
                            const int64_t* __restrict__ row_off,
                            const int* __restrict__ order, int nsys,
                            const double* __restrict__ work,
                            int* __restrict__ counter) {
  constexpr int RS = SegCfg<NV>::RS;
  constexpr int64_t WROW = (int64_t)NV * NV + 2 * NV, SROW = (int64_t)NV * RS;
  constexpr unsigned full = 0xffffffffu;
  const SegLane<NV> g;
  const int r = g.r, base = g.base;
  const double* __restrict__ sg = work + row_off[nsys] * WROW;
  bool live = g.in_seg;
  int cnt = 0, t = 0, dir = 0, m = 0;
  int64_t r0 = 0;
  double x = 0.0;  // this lane's entry of the previous row's x
  for (;;) {
    const bool need = live && t >= cnt;
    const int q = seg_fetch(g, need, counter);
    if (need) {
      if (q >= 2 * nsys) {
        live = false;
      } else {
        const int s = order[q >> 1];
        dir = q & 1;
        r0 = row_off[s];
        const int64_t n64 = row_off[s + 1] - r0;
        const int N = n64 > 0 ? (int)n64 : 0;
        m = N >> 1;
        cnt = seg_unit_rows(N, dir);
        t = 0;
        if (cnt > 0) x = X[(r0 + m) * NV + r];
      }
    }
    if (!__any_sync(full, live)) break;
    const bool act = live && t < cnt;
    const int64_t row = r0 + (act ? (dir == 0 ? m - 1 - t : m + 1 + t) : 0);
    double v = 0.0, srow[NV];
    if (act) {
      const double* __restrict__ p = sg + row * SROW + r * RS;
      if (t + 1 < cnt) prefetch_row<RS>(dir == 0 ? p - SROW : p + SROW);
#pragma unroll
      for (int j = 0; j < NV; ++j) srow[j] = p[j];
      v = p[NV];
    } else {
#pragma unroll
      for (int j = 0; j < NV; ++j) srow[j] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double xk = __shfl_sync(full, x, base + k);
      v = fma(-srow[k], xk, v);
    }
    if (act) {
      x = v;
      X[row * NV + r] = v;
      ++t;
    }
  }
}

// y = F^-1 v inside a segment: F's getrf factors (lane r holding factor
// row r, f, and its diagonal d) and pivots, v in original row order on the
// lanes; returns this lane's entry of y (variable order).
template <int NV>
__device__ __forceinline__ double seg_lu_solve(const SegLane<NV>& g,
                                               const double (&f)[NV],
                                               double d, int perm_src,
                                               double v) {
  constexpr unsigned full = 0xffffffffu;
  const int r = g.r, base = g.base;
  double y = __shfl_sync(full, v, base + perm_src);
  // unit lower: y_r -= L[r][k] y_k, k < r
#pragma unroll
  for (int k = 0; k < NV - 1; ++k) {
    const double yk = __shfl_sync(full, y, base + k);
    if (r > k) y = fma(-f[k], yk, y);
  }
  // upper: y_r = (y_r - sum_{k > r} U[r][k] y_k) / U[r][r]
  const double inv = pyro_rcp3(d);
#pragma unroll
  for (int k = NV - 1; k >= 0; --k) {
    if (r == k) y *= inv;
    const double yk = __shfl_sync(full, y, base + k);
    if (r < k) y = fma(-f[k], yk, y);
  }
  return y;
}

// Re-solve after pyro_block_thomas_seg, with its kept factors (two-ended,
// like the solve): per system and right-hand side, in steps
// v = base - M y [then y = F^-1 v], y the previous step's result:
//   1  rows i = 0 .. m-1:        base b_i, M = L_{i-1} (none at i = 0), F_i
//   2  row m:                    base b_m, M = L_{m-1} (none at m = 0)
//   3  rows i = N-1 .. m+1:      base b_i, M = U_i (none at i = N-1), F_i
//   4  row m:                    base step 2's v, M = U_m (none without
//                                rows below m), F_m: x_m
//   5  rows i = m-1 .. 0:        base t_i, M = S_i (y = x_m first)
//   6  rows i = m+1 .. N-1:      base t^_i, M = S^_i (y = x_m first)
// with the intermediate vectors in x.  Every segment runs one step per
// warp step, at its own system, right-hand side and phase.
template <int NV>
__global__ void __launch_bounds__(kSegWarps * 32)
    k_block_thomas_seg_resolve(const double* __restrict__ Lm,
                               const double* __restrict__ Um,
                               const double* __restrict__ B,
                               double* __restrict__ X, int nrhs,
                               int64_t rhs_stride,
                               const int64_t* __restrict__ row_off,
                               const int* __restrict__ order, int nsys,
                               const double* __restrict__ work,
                               int* __restrict__ counter,
                               int* __restrict__ status) {
  constexpr int RS = SegCfg<NV>::RS;
  constexpr int64_t NN = (int64_t)NV * NV, WROW = NN + 2 * NV,
                    SROW = (int64_t)NV * RS;
  constexpr unsigned full = 0xffffffffu;
  const SegLane<NV> g;
  const int r = g.r, base = g.base;
  const double* __restrict__ sg = work + row_off[nsys] * WROW;
  bool live = g.in_seg, busy = false;
  int N = 0, m = 0, c = 0, ph = 0, i = 0;
  int64_t r0 = 0;
  double y = 0.0, xm = 0.0;
  for (;;) {
    const bool need = live && !busy;
    const int q = seg_fetch(g, need, counter);
    if (need) {
      if (q >= nsys) {
        live = false;
      } else {
        const int s = order[q];
        r0 = row_off[s];
        const int64_t n64 = row_off[s + 1] - r0;
        N = n64 > 0 ? (int)n64 : 0;
        if (n64 <= 0 && r == 0 && status) atomicOr(status, 2);
        m = N >> 1;
        c = 0;
        ph = 1;
        i = 0;
        busy = N > 0;
      }
    }
    if (!__any_sync(full, live)) break;
    // skip the empty phases (1: no rows above m; 3: none below; 5, 6
    // likewise) and move to the next right-hand side after phase 6
    if (busy && ph == 1 && i >= m) { ph = 2; i = m; }
    if (busy && ph == 3 && i < m + 1) { ph = 4; i = m; }
    if (busy && ph == 5 && i < 0) { ph = 6; i = m + 1; y = xm; }
    if (busy && ph == 6 && i > N - 1) {
      if (++c < nrhs) {
        ph = m >= 1 ? 1 : 2;
        i = 0;
      } else {
        busy = false;
      }
    }
    const bool act = live && busy;
    const int64_t row = r0 + i;
    const double* __restrict__ Bc = B + (int64_t)c * rhs_stride;
    double* __restrict__ Xc = X + (int64_t)c * rhs_stride;
    // the step's base, coupling rows and whether it solves with F_row
    double v = 0.0, mrow[NV];
    bool solve = false, coupled = false;
    if (act) {
      const double* __restrict__ M = nullptr;
      int64_t mstride = NV;
      if (ph == 1) {
        v = __ldg(Bc + row * NV + r);
        if (i > 0) M = Lm + (row - 1) * NN;
        solve = true;
      } else if (ph == 2) {
        v = __ldg(Bc + row * NV + r);
        if (m >= 1) M = Lm + (row - 1) * NN;
      } else if (ph == 3) {
        v = __ldg(Bc + row * NV + r);
        if (i < N - 1) M = Um + row * NN;
        solve = true;
      } else if (ph == 4) {
        v = Xc[row * NV + r];
        if (m + 1 <= N - 1) M = Um + row * NN;
        solve = true;
      } else {
        v = Xc[row * NV + r];
        M = sg + row * SROW;
        mstride = RS;
      }
      coupled = M != nullptr;
      const double* __restrict__ Mr = (coupled ? M : Bc + row * NV) +
                                      (coupled ? r * mstride : 0);
#pragma unroll
      for (int k = 0; k < NV; ++k) mrow[k] = coupled ? Mr[k] : 0.0;
    } else {
#pragma unroll
      for (int k = 0; k < NV; ++k) mrow[k] = 0.0;
    }
    // an uncoupled step takes nothing from y (which may hold a previous
    // system's non-finite result)
    const double ys = coupled ? y : 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double yk = __shfl_sync(full, ys, base + k);
      v = fma(-mrow[k], yk, v);
    }
    // y = F^-1 v where the step solves (the other segments' lanes pass v)
    if (__any_sync(full, solve)) {
      const double* __restrict__ w = work + row * WROW;
      double f[NV], d = 1.0;
      int perm_src = r;
      if (solve) {
#pragma unroll
        for (int j = 0; j < NV; ++j) f[j] = w[r * NV + j];
        d = f[0];
#pragma unroll
        for (int j = 1; j < NV; ++j)
          if (j == r) d = f[j];
        // original row held at position r after getrf's swaps
        int j = r;
#pragma unroll
        for (int k = NV - 1; k >= 0; --k) {
          const int pk = (int)w[NN + NV + k];
          if (j == k)
            j = pk;
          else if (j == pk)
            j = k;
        }
        perm_src = j;
      } else {
#pragma unroll
        for (int j = 0; j < NV; ++j) f[j] = 0.0;
      }
      const double yl = seg_lu_solve<NV>(g, f, d, perm_src, v);
      if (solve) v = yl;
    }
    if (act) {
      Xc[row * NV + r] = v;
      y = v;
      if (ph == 1) {
        ++i;
      } else if (ph == 2) {
        ph = 3;
        i = N - 1;
      } else if (ph == 3) {
        --i;
      } else if (ph == 4) {
        xm = v;
        ph = 5;
        i = m - 1;
      } else if (ph == 5) {
        --i;
      } else {
        ++i;
      }
    }
  }
}

template <int NV>
int seg_grid(const void* kernel, int nunits, int ctas) {
  const int per_cta = kSegWarps * SegCfg<NV>::P;
  const int need = (nunits + per_cta - 1) / per_cta;
  if (ctas <= 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, kernel, kSegWarps * 32, 0) != cudaSuccess ||
        per_sm < 1) {
      (void)cudaGetLastError();
      per_sm = 1;
    }
    ctas = per_sm * pyro_sm_count();
  }
  return ctas < need ? ctas : need;
}

template <int NV>
int launch_seg(const double* L, const double* C, const double* U,
               const double* b, double* x, const int64_t* row_off,
               const int* order, int nsys, double* work, int* counter,
               int* status, int ctas, cudaStream_t stream) {
  // forward grid: by default two warps per SM partition (one's shuffle,
  // redux and reciprocal latencies under the other's FP64 work) when the
  // sweeps come to three per lane segment of one warp per partition or
  // more, else one (forward sweeps at nv = 10, sweeps of 32..512 rows,
  // one / two warps: 2,048 sweeps 7.7 / 9.9 ms, 4,096 10.4 / 11.5 ms,
  // 6,000 14.5 / 11.5 ms, 8,192 19.2 / 15.3 ms, three warps 17.0 ms)
  const int units = 2 * nsys;
  if (ctas <= 0) {
    const int segs_per_warp_slot = pyro_sm_count() * 4 * SegCfg<NV>::P;
    const int w = units >= 3 * segs_per_warp_slot ? 2 : 1;
    ctas = pyro_sm_count() * w * 4 / kSegWarps;
  }
  const int fwd = seg_grid<NV>((const void*)k_block_thomas_seg<NV>, units,
                               ctas);
  const int mid = seg_grid<NV>((const void*)k_block_thomas_seg_mid<NV>, nsys,
                               0);
  const int back = seg_grid<NV>((const void*)k_block_thomas_seg_back<NV>,
                                units, 0);
  if (cudaMemsetAsync(counter, 0, sizeof(int), stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  k_block_thomas_seg<NV><<<fwd, kSegWarps * 32, 0, stream>>>(
      L, C, U, b, row_off, order, nsys, work, counter, status);
  PYRO_CHECK_LAUNCH();
  if (cudaMemsetAsync(counter, 0, sizeof(int), stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  k_block_thomas_seg_mid<NV><<<mid, kSegWarps * 32, 0, stream>>>(
      L, C, U, b, x, row_off, order, nsys, work, counter, status);
  PYRO_CHECK_LAUNCH();
  if (cudaMemsetAsync(counter, 0, sizeof(int), stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  k_block_thomas_seg_back<NV><<<back, kSegWarps * 32, 0, stream>>>(
      x, row_off, order, nsys, work, counter);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

template <int NV>
int launch_seg_resolve(const double* L, const double* U, const double* B,
                       double* X, int nrhs, int64_t rhs_stride,
                       const int64_t* row_off, const int* order, int nsys,
                       const double* work, int* counter, int* status,
                       cudaStream_t stream) {
  const int grid = seg_grid<NV>(
      (const void*)k_block_thomas_seg_resolve<NV>, nsys, 0);
  if (cudaMemsetAsync(counter, 0, sizeof(int), stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  k_block_thomas_seg_resolve<NV><<<grid, kSegWarps * 32, 0, stream>>>(
      L, U, B, X, nrhs, rhs_stride, row_off, order, nsys, work, counter,
      status);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

}  // namespace

// pyro_block_thomas for blocks of size nv <= 16 with 32 / nv systems per
// warp, one lane per block row (see above).  Same arguments and workspace
// size as pyro_block_thomas (the factors two-ended: re-solve with
// pyro_block_thomas_seg_resolve); three launches (sweeps to the middle
// rows, middle rows, sweeps back); the CTA size is fixed (four warps);
// ctas: forward grid size (0 = one or two warps per SM partition by the
// batch size).
PYRO_EXPORT int pyro_block_thomas_seg(const double* L, const double* C,
                                      const double* U, const double* b,
                                      double* x, const int64_t* row_off,
                                      const int* order, int nsys, int nv,
                                      double* work, int* counter, int* status,
                                      int ctas, cudaStream_t stream) {
  if (nsys < 0 || nv < 1 || nv > 16) return PYRO_ERR_ARGUMENT;
  if (nsys == 0) return PYRO_OK;
  if (!L || !C || !U || !b || !x || !row_off || !order || !work || !counter)
    return PYRO_ERR_ARGUMENT;
  switch (nv) {
#define PYRO_BT_SEG(NV)                                                      \
  case NV:                                                                   \
    return launch_seg<NV>(L, C, U, b, x, row_off, order, nsys, work,         \
                          counter, status, ctas, stream);
    PYRO_BT_SEG(1) PYRO_BT_SEG(2) PYRO_BT_SEG(3) PYRO_BT_SEG(4)
    PYRO_BT_SEG(5) PYRO_BT_SEG(6) PYRO_BT_SEG(7) PYRO_BT_SEG(8)
    PYRO_BT_SEG(9) PYRO_BT_SEG(10) PYRO_BT_SEG(11) PYRO_BT_SEG(12)
    PYRO_BT_SEG(13) PYRO_BT_SEG(14) PYRO_BT_SEG(15) PYRO_BT_SEG(16)
#undef PYRO_BT_SEG
    default:
      return PYRO_ERR_ARGUMENT;
  }
}

// More right-hand sides after pyro_block_thomas_seg (whose two-ended
// factors the re-solve below cannot use): arguments as for
// pyro_block_thomas_resolve, nv <= 16.
PYRO_EXPORT int pyro_block_thomas_seg_resolve(
    const double* L, const double* U, const double* B, double* X,
    int nrhs, int64_t rhs_stride, const int64_t* row_off, const int* order,
    int nsys, int nv, const double* work, int* counter, int* status,
    cudaStream_t stream) {
  if (nsys < 0 || nv < 1 || nv > 16 || nrhs < 1 || nrhs > 4)
    return PYRO_ERR_ARGUMENT;
  if (nsys == 0) return PYRO_OK;
  if (!L || !U || !B || !X || !row_off || !order || !work || !counter)
    return PYRO_ERR_ARGUMENT;
  if (nrhs > 1 && rhs_stride < 1) return PYRO_ERR_ARGUMENT;
  switch (nv) {
#define PYRO_BT_SEGR(NV)                                                     \
  case NV:                                                                   \
    return launch_seg_resolve<NV>(L, U, B, X, nrhs, rhs_stride, row_off,     \
                                  order, nsys, work, counter, status,        \
                                  stream);
    PYRO_BT_SEGR(1) PYRO_BT_SEGR(2) PYRO_BT_SEGR(3) PYRO_BT_SEGR(4)
    PYRO_BT_SEGR(5) PYRO_BT_SEGR(6) PYRO_BT_SEGR(7) PYRO_BT_SEGR(8)
    PYRO_BT_SEGR(9) PYRO_BT_SEGR(10) PYRO_BT_SEGR(11) PYRO_BT_SEGR(12)
    PYRO_BT_SEGR(13) PYRO_BT_SEGR(14) PYRO_BT_SEGR(15) PYRO_BT_SEGR(16)
#undef PYRO_BT_SEGR
    default:
      return PYRO_ERR_ARGUMENT;
  }
}

// ------------------------------------------------------------------------
// Re-solve with kept factors.
//
// After pyro_block_thomas or pyro_block_thomas_small, `work` holds for
// every row the LU factors and pivots of C'_i (pyro_block_thomas_seg's
// two-ended factors have their own re-solve above).  More right-hand sides for
// the same L, C, U (the EOS-consistency adjoint solves share one operator,
// thermodynamic_consistency.py:105-307; a chord Newton iteration reuses its
// Jacobian) need only the vector recurrences:
//   forward:  b'_0 = b_0, b'_i = b_i - L_{i-1} t_{i-1}, t_i = C'_i^-1 b'_i
//   backward: x_{N-1} = t_{N-1}, x_i = C'_i^-1 (b'_i - U_i x_{i+1})
// -- 4 nv^2 FMAs per row and right-hand side instead of ~4.7 nv^3.  One
// warp per system, the lanes over matrix rows, the NRHS right-hand sides
// sharing every block element the lanes read (through L1).  A warp-wide
// FP64 instruction costs the FP64 pipe the same however few lanes it
// uses, so the nv diagonal reciprocals of a row's factors are formed by
// the lanes side by side once per row, not one per elimination step.
// b'_i is kept in x until the backward pass overwrites it.  Systems come
// from an atomic counter in the caller's order.

namespace {

constexpr int kResolveWarps = 4;

// y <- C'^-1 y for NRHS vectors y[q * 64 + i] (warp-private shared
// memory), factors A (nv x nv, row-major) and pivots from the workspace;
// rd: warp-private scratch for the diagonal reciprocals (64 doubles) and
// the pivots (64 ints after them).
template <int NRHS>
__device__ void warp_lu_solve(const double* __restrict__ A,
                              const double* __restrict__ pv, int nv,
                              double* y, double* rd, int lane) {
  int* ps = (int*)(rd + 64);
  for (int k = lane; k < nv; k += 32) {
    rd[k] = 1.0 / __ldg(A + k * nv + k);
    ps[k] = (int)__ldg(pv + k);
  }
  __syncwarp();
  if (lane == 0) {
    for (int k = 0; k < nv; ++k) {
      const int p = ps[k];
      if (p != k)
#pragma unroll
        for (int q = 0; q < NRHS; ++q) {
          const double t = y[q * 64 + k];
          y[q * 64 + k] = y[q * 64 + p];
          y[q * 64 + p] = t;
        }
    }
  }
  __syncwarp();
  // unit lower
  for (int k = 0; k < nv - 1; ++k) {
    double yk[NRHS];
#pragma unroll
    for (int q = 0; q < NRHS; ++q) yk[q] = y[q * 64 + k];
    for (int i = k + 1 + lane; i < nv; i += 32) {
      const double a = __ldg(A + i * nv + k);
#pragma unroll
      for (int q = 0; q < NRHS; ++q)
        y[q * 64 + i] = fma(-a, yk[q], y[q * 64 + i]);
    }
    __syncwarp();
  }
  // upper
  for (int k = nv - 1; k >= 0; --k) {
    double yk[NRHS];
    const double inv = rd[k];
#pragma unroll
    for (int q = 0; q < NRHS; ++q) yk[q] = y[q * 64 + k] * inv;
    __syncwarp();
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < NRHS; ++q) y[q * 64 + k] = yk[q];
    for (int i = lane; i < k; i += 32) {
      const double a = __ldg(A + i * nv + k);
#pragma unroll
      for (int q = 0; q < NRHS; ++q)
        y[q * 64 + i] = fma(-a, yk[q], y[q * 64 + i]);
    }
    __syncwarp();
  }
}

// y[q][j] -= sum_k M[j][k] z[q][k] for the warp's rows j.
template <int NRHS>
__device__ __forceinline__ void warp_matvec_sub(
    const double* __restrict__ M, const double* z, int nv, int lane,
    double* y) {
  for (int j = lane; j < nv; j += 32) {
    double acc[NRHS];
#pragma unroll
    for (int q = 0; q < NRHS; ++q) acc[q] = y[q * 64 + j];
    for (int k = 0; k < nv; ++k) {
      const double m = __ldg(M + j * nv + k);
#pragma unroll
      for (int q = 0; q < NRHS; ++q) acc[q] = fma(-m, z[q * 64 + k], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < NRHS; ++q) y[q * 64 + j] = acc[q];
  }
}

template <int NRHS>
__global__ void __launch_bounds__(32 * kResolveWarps)
    k_block_thomas_resolve(const double* __restrict__ Lm,
                           const double* __restrict__ Um,
                           const double* __restrict__ B,
                           double* __restrict__ X, int64_t rhs_stride,
                           const int64_t* __restrict__ row_off,
                           const int* __restrict__ order, int nsys, int nv,
                           const double* __restrict__ work,
                           int* __restrict__ counter,
                           int* __restrict__ status) {
  __shared__ double s_vec[kResolveWarps][2 * NRHS * 64 + 96];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double* y = s_vec[wid];            // current vector
  double* z = y + NRHS * 64;         // previous t_{i-1} / x_{i+1}
  double* rd = z + NRHS * 64;        // diagonal reciprocals, pivots
  const int64_t nn = (int64_t)nv * nv, wrow = nn + 2 * nv;
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(counter, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= nsys) break;
    const int s = order[q];
    const int64_t r0 = row_off[s];
    const int64_t n64 = row_off[s + 1] - r0;
    if (n64 <= 0) {  // an empty row range: skipped and flagged
      if (lane == 0 && status) atomicOr(status, 2);
      continue;
    }
    const int N = (int)n64;
    // forward
    for (int i = 0; i < N; ++i) {
      const int64_t row = r0 + i;
      for (int j = lane; j < nv; j += 32)
#pragma unroll
        for (int c = 0; c < NRHS; ++c)
          y[c * 64 + j] = __ldg(B + c * rhs_stride + row * nv + j);
      __syncwarp();
      if (i > 0) {
        warp_matvec_sub<NRHS>(Lm + (row - 1) * nn, z, nv, lane, y);
        __syncwarp();
      }
      // b'_i is kept in x for the backward pass
      for (int j = lane; j < nv; j += 32)
#pragma unroll
        for (int c = 0; c < NRHS; ++c)
          X[c * rhs_stride + row * nv + j] = y[c * 64 + j];
      const double* w = work + row * wrow;
      warp_lu_solve<NRHS>(w, w + nn + nv, nv, y, rd, lane);
      double* t = z;
      z = y;
      y = t;
      __syncwarp();
    }
    // z = t_{N-1} = x_{N-1}
    for (int j = lane; j < nv; j += 32)
#pragma unroll
      for (int c = 0; c < NRHS; ++c)
        X[c * rhs_stride + (r0 + N - 1) * nv + j] = z[c * 64 + j];
    __syncwarp();
    // backward
    for (int i = N - 2; i >= 0; --i) {
      const int64_t row = r0 + i;
      for (int j = lane; j < nv; j += 32)
#pragma unroll
        for (int c = 0; c < NRHS; ++c)
          y[c * 64 + j] = X[c * rhs_stride + row * nv + j];
      __syncwarp();
      warp_matvec_sub<NRHS>(Um + row * nn, z, nv, lane, y);
      __syncwarp();
      const double* w = work + row * wrow;
      warp_lu_solve<NRHS>(w, w + nn + nv, nv, y, rd, lane);
      for (int j = lane; j < nv; j += 32)
#pragma unroll
        for (int c = 0; c < NRHS; ++c)
          X[c * rhs_stride + row * nv + j] = y[c * 64 + j];
      double* t = z;
      z = y;
      y = t;
      __syncwarp();
    }
  }
}

template <int NRHS>
int launch_resolve(const double* L, const double* U, const double* B,
                   double* X, int64_t rhs_stride, const int64_t* row_off,
                   const int* order, int nsys, int nv, const double* work,
                   int* counter, int* status, cudaStream_t stream) {
  int blocks = (nsys + kResolveWarps - 1) / kResolveWarps;
  const int cap = pyro_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  k_block_thomas_resolve<NRHS><<<blocks, 32 * kResolveWarps, 0, stream>>>(
      L, U, B, X, rhs_stride, row_off, order, nsys, nv, work, counter,
      status);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

}  // namespace

// nrhs (1..4) right-hand sides B[c][rows][nv] (c-th at B + c * rhs_stride)
// -> X[c][rows][nv] for the systems whose factors a previous
// pyro_block_thomas / _small call with the same L, C, U left in
// `work`.  order, counter as for pyro_block_thomas (counter zeroed here);
// status (may be NULL): bit 1 for an empty row range; nv <= 64.  B and X
// must not overlap.  Asynchronous on `stream`.
PYRO_EXPORT int pyro_block_thomas_resolve(
    const double* L, const double* U, const double* B, double* X,
    int nrhs, int64_t rhs_stride, const int64_t* row_off, const int* order,
    int nsys, int nv, const double* work, int* counter, int* status,
    cudaStream_t stream) {
  if (nsys < 0 || nv < 1 || nv > 64 || nrhs < 1 || nrhs > 4)
    return PYRO_ERR_ARGUMENT;
  if (nsys == 0) return PYRO_OK;
  if (!L || !U || !B || !X || !row_off || !order || !work || !counter)
    return PYRO_ERR_ARGUMENT;
  if (nrhs > 1 && rhs_stride < 1) return PYRO_ERR_ARGUMENT;
  if (cudaMemsetAsync(counter, 0, sizeof(int), stream) != cudaSuccess)
    return PYRO_ERR_LAUNCH;
  switch (nrhs) {
    case 1:
      return launch_resolve<1>(L, U, B, X, rhs_stride, row_off, order, nsys,
                               nv, work, counter, status, stream);
    case 2:
      return launch_resolve<2>(L, U, B, X, rhs_stride, row_off, order, nsys,
                               nv, work, counter, status, stream);
    case 3:
      return launch_resolve<3>(L, U, B, X, rhs_stride, row_off, order, nsys,
                               nv, work, counter, status, stream);
    default:
      return launch_resolve<4>(L, U, B, X, rhs_stride, row_off, order, nsys,
                               nv, work, counter, status, stream);
  }
}

// ------------------------------------------------------------------------
// No-allocation variant.
//
// Some callers cannot allocate device memory at the point where they need a
// solve: host applications that hand all device memory to their own pool at
// start-up and forbid allocation inside a time step (for example a flow
// solver's implicit chemistry update), and real-time loops where the
// latency or a failure of an allocation in the middle of a step is not
// acceptable.  For them,
// pyro_block_thomas_noalloc takes the same inputs and outputs as
// pyro_block_thomas but keeps its scratch -- the per-row factor workspace
// and the work counter -- in the file-scope array below, so the
// call allocates nothing.
//
// Limits and sharing: the array holds PYRO_BT_STATIC_DOUBLES doubles
// (16 MiB), i.e. pyro_block_thomas_noalloc_max_rows(nv) packed rows
// (17,476 rows at nv = 10, 693 at nv = 54); every GPU that loads the
// library holds it until the process exits.  All calls share it and it
// keeps the last call's contents (the counter is cleared by every call;
// the workspace is written before it is read), so calls whose executions
// overlap on the GPU -- on different streams, or from different host
// threads -- race and must not be issued.  The first call on a device
// looks up the array's device address (cudaGetSymbolAddress, with that
// device current); make that first call before any stream capture.
// ------------------------------------------------------------------------

#include <mutex>

#define PYRO_BT_STATIC_DOUBLES (1 << 21)
#define PYRO_BT_MAX_DEVICES 64

// workspace, then 32 doubles (256 bytes) whose first int is the counter
static __device__ __align__(256) double
    pyro_bt_static_scratch[PYRO_BT_STATIC_DOUBLES + 32];

namespace {

std::mutex g_bt_static_mu;
double* g_bt_static_ptr[PYRO_BT_MAX_DEVICES] = {nullptr};

// Device address of the static scratch on the current device (looked up
// once per device).
int bt_static_scratch(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 ||
      dev >= PYRO_BT_MAX_DEVICES) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  std::lock_guard<std::mutex> lock(g_bt_static_mu);
  if (g_bt_static_ptr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, pyro_bt_static_scratch) != cudaSuccess ||
        p == nullptr) {
      (void)cudaGetLastError();
      return PYRO_ERR_LAUNCH;
    }
    g_bt_static_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_bt_static_ptr[dev];
  return PYRO_OK;
}

// k_block_thomas with a bound on the rows it may touch in `work`: a system
// whose rows fall outside [0, cap_rows) is skipped and flagged (status
// bit 1) instead of writing past the static scratch.
__global__ void k_block_thomas_capped(
    const double* __restrict__ Lm, const double* __restrict__ Cm,
    const double* __restrict__ Um, const double* __restrict__ B,
    double* __restrict__ X, const int64_t* __restrict__ row_off,
    const int* __restrict__ order, int nsys, int nv,
    double* __restrict__ work, int64_t cap_rows, int* __restrict__ counter,
    int* __restrict__ status) {
  extern __shared__ double smem[];
  __shared__ int s_sys;
  __shared__ int s_sing;
  for (;;) {
    if (threadIdx.x == 0) {
      s_sys = atomicAdd(counter, 1);
      s_sing = 0;
    }
    __syncthreads();
    const int q = s_sys;
    if (q >= nsys) break;
    const int s = order[q];
    const int64_t r0 = row_off[s];
    const int64_t r1 = row_off[s + 1];
    if (r0 < 0 || r1 <= r0 || r1 > cap_rows) {
      if (threadIdx.x == 0 && status) atomicOr(status, 2);
      __syncthreads();
      continue;
    }
    solve_system(Lm, Cm, Um, B, X, r0, (int)(r1 - r0), nv, work, smem,
                 &s_sing);
    if (threadIdx.x == 0 && s_sing && status) atomicOr(status, 1);
    __syncthreads();
  }
}

}  // namespace

// Rows of the static scratch for blocks of size nv (0 for nv out of range).
PYRO_EXPORT int64_t pyro_block_thomas_noalloc_max_rows(int nv) {
  if (nv < 1 || nv > 64) return 0;
  return (int64_t)PYRO_BT_STATIC_DOUBLES / ((int64_t)nv * nv + 2 * nv);
}

// pyro_block_thomas without a caller workspace or counter: scratch in the
// library's static device array (see above).  total_rows: row_off[nsys]
// (host value); more than pyro_block_thomas_noalloc_max_rows(nv) returns
// PYRO_ERR_CAPACITY before anything is launched.  status: as for
// pyro_block_thomas, plus bit 1 if a system's rows lie outside
// [0, total_rows].  Allocates nothing; asynchronous on `stream`.
PYRO_EXPORT int pyro_block_thomas_noalloc(
    const double* L, const double* C, const double* U, const double* b,
    double* x, const int64_t* row_off, const int* order, int nsys, int nv,
    int64_t total_rows, int* status, int threads, int ctas,
    cudaStream_t stream) {
  if (nsys < 0 || nv < 1 || nv > 64 || threads < 32 || threads > 1024 ||
      threads % 32 || total_rows < 0)
    return PYRO_ERR_ARGUMENT;
  if (total_rows > pyro_block_thomas_noalloc_max_rows(nv))
    return PYRO_ERR_CAPACITY;
  if (nsys == 0) return PYRO_OK;
  if (!L || !C || !U || !b || !x || !row_off || !order)
    return PYRO_ERR_ARGUMENT;
  double* scratch = nullptr;
  if (bt_static_scratch(&scratch) != PYRO_OK) return PYRO_ERR_LAUNCH;
  int* counter = reinterpret_cast<int*>(scratch + PYRO_BT_STATIC_DOUBLES);
  const size_t smem = (size_t)pyro_block_thomas_smem_bytes(nv);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute((const void*)k_block_thomas_capped,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  if (ctas <= 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, k_block_thomas_capped, threads, smem) != cudaSuccess ||
        per_sm < 1) {
      (void)cudaGetLastError();
      per_sm = 1;
    }
    ctas = per_sm * pyro_sm_count();
  }
  if (ctas > nsys) ctas = nsys;
  if (cudaMemsetAsync(counter, 0, sizeof(int), stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  k_block_thomas_capped<<<ctas, threads, smem, stream>>>(
      L, C, U, b, x, row_off, order, nsys, nv, scratch, total_rows, counter,
      status);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}
