/*
 * Batched block-Thomas solver (libpyro_block_thomas_<hash>.so).
 *
 * Replaces pyrometheus/flamelets/linear_solver.py:6-103
 * (block_thomas(lower, central, upper, rhs), one system per call, two
 * jax.lax.scan sweeps with jnp.linalg.solve) with one persistent launch over
 * many systems of uneven lengths.
 *
 * Packed layout: system s owns rows [row_off[s], row_off[s+1]) of
 * C[rows][nv][nv] (diagonal blocks), L and U (sub/super-diagonal blocks;
 * the last row of each system is ignored), b[rows][nv] and x[rows][nv].
 * All pointers are device pointers; row-major blocks; FP64.
 */
#ifndef PYRO_BLOCK_THOMAS_H
#define PYRO_BLOCK_THOMAS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* cudaStream_t;

/* Doubles of workspace pyro_block_thomas needs for `rows` packed rows
 * (per row: the LU factors of the modified diagonal block C'_i, b'_i and
 * the pivots, kept for the backward solves). */
int64_t pyro_block_thomas_work_doubles(int nv, int64_t rows);

/* Dynamic shared memory of one CTA for blocks of size nv. */
int64_t pyro_block_thomas_smem_bytes(int nv);

/* Solve nsys systems (1 <= nv <= 64).  order: permutation of 0..nsys-1
 * (longest first balances best); work: pyro_block_thomas_work_doubles
 * doubles; counter: device int (zeroed by the call); status: device int,
 * bit 0 set on a zero pivot (may be NULL); threads: CTA size (multiple of
 * 32); ctas: grid size (0 = all resident).  Asynchronous on `stream`;
 * returns 0 or a PyroStatus error. */
int pyro_block_thomas(const double* L, const double* C, const double* U,
                      const double* b, double* x, const int64_t* row_off,
                      const int* order, int nsys, int nv, double* work,
                      int* counter, int* status, int threads, int ctas,
                      cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PYRO_BLOCK_THOMAS_H */
