/*
 * Batched dense LU for many independent small FP64 systems
 * (libpyro_batched_lu_<hash>.so): the per-cell Newton matrices of the
 * implicit 0-D reactor integrator.
 *
 * Replaces the per-reactor dense Newton solve of the reference's implicit
 * reactor stepping, pyrometheus/examples/free_flame/time_integ.py:94
 * (jnp.linalg.solve(jac, -res): one LU factorisation and solve per call),
 * with one launch that factorises every selected cell's matrix and keeps
 * the factors, and a second entry point that solves with kept factors.
 *
 * All pointers are device pointers; matrices M[n][nv][nv] row-major;
 * 1 <= nv <= 64.  Every call is asynchronous on `stream` and allocates
 * nothing.
 */
#ifndef PYRO_BATCHED_LU_H
#define PYRO_BATCHED_LU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* cudaStream_t;

/* Factorise M_s in place (P M = L U, partial pivoting, unit-lower L below
 * the diagonal) for every s < n with mask[s] != 0 (mask may be NULL: all);
 * piv[s][k] = row swapped with k at step k.  status (device int, may be
 * NULL): bit 0 set if some matrix had a zero pivot column.  Returns 0 or
 * a PyroStatus code (1 argument, 2 launch). */
int pyro_batched_lu_factor(double* M, int* piv, const unsigned char* mask,
                           int n, int nv, int* status, cudaStream_t stream);

/* x_s = M_s^-1 b_s with the factors above, for every unmasked s; element i
 * of system s is b[s * b_ss + i * b_vs] (b_ss = nv, b_vs = 1 for [n][nv];
 * b_ss = 1, b_vs = n for variable-major [nv][n]); same for x.  x may alias
 * b with the same strides; masked-out x_s are left untouched. */
int pyro_batched_lu_solve(const double* LU, const int* piv,
                          const unsigned char* mask, const double* b,
                          int64_t b_ss, int64_t b_vs, double* x, int64_t x_ss,
                          int64_t x_vs, int n, int nv, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PYRO_BATCHED_LU_H */
