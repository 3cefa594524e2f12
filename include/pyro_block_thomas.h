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
 * Every system needs at least one row: a system whose row range is empty
 * (row_off[s+1] <= row_off[s]) is skipped, its x left untouched, and bit 1
 * of *status is set.  All pointers are device pointers; row-major blocks;
 * FP64.
 */
#ifndef PYRO_BLOCK_THOMAS_H
#define PYRO_BLOCK_THOMAS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* cudaStream_t;

/* Doubles of workspace the solvers need for `rows` packed rows
 * (rows = row_off[nsys]): per row the LU factors of the modified diagonal
 * block C'_i, b'_i and the pivots, kept for the backward solves and
 * pyro_block_thomas_resolve; for nv <= 16 then, after all rows of those,
 * S_i | t_i = C'_i^-1 (U_i | b'_i) of every row (nv x (nv + 1), written by
 * pyro_block_thomas_seg for its backward sweep). */
int64_t pyro_block_thomas_work_doubles(int nv, int64_t rows);

/* Dynamic shared memory of one CTA for blocks of size nv. */
int64_t pyro_block_thomas_smem_bytes(int nv);

/* Solve nsys systems (1 <= nv <= 64).  order: permutation of 0..nsys-1
 * (longest first balances best); work: pyro_block_thomas_work_doubles
 * doubles; counter: device int (zeroed by the call); status: device int,
 * bit 0 set on a zero pivot, bit 1 on an empty system (may be NULL);
 * threads: CTA size (multiple of 32); ctas: grid size (0 = all resident).
 * Asynchronous on `stream`; returns 0 or a PyroStatus error. */
int pyro_block_thomas(const double* L, const double* C, const double* U,
                      const double* b, double* x, const int64_t* row_off,
                      const int* order, int nsys, int nv, double* work,
                      int* counter, int* status, int threads, int ctas,
                      cudaStream_t stream);

/* pyro_block_thomas for blocks of size nv <= 16 with one thread per system
 * (the whole recurrence of a system runs in one thread, so every FP64
 * instruction of a warp does 32 useful operations).  Same arguments and
 * workspace as pyro_block_thomas without the counter and the grid size;
 * threads: systems per CTA, 32 or 64 (64 needs 3*nv*(nv+1)*8*64 bytes of
 * shared memory to fit in 227 KB).  Replaces the same reference function,
 * pyrometheus/flamelets/linear_solver.py:6-103. */
int pyro_block_thomas_small(const double* L, const double* C, const double* U,
                            const double* b, double* x,
                            const int64_t* row_off, const int* order,
                            int nsys, int nv, double* work, int* status,
                            int threads, cudaStream_t stream);

/* pyro_block_thomas for blocks of size nv <= 16 with 32 / nv systems per
 * warp (three at nv = 10), one lane per block row and the working rows in
 * registers: every lane of every FP64 instruction works, and nothing
 * synchronises beyond a warp.  Two-ended: each system is eliminated from
 * its first row down and from its last row up to its middle row m = N / 2
 * (two independent sweeps), the middle row is solved, and x follows
 * outwards, x_i = t_i - S_i x_{i+-1}.  A persistent grid whose lane
 * segments each take the next sweep of `order` when theirs is done; three
 * launches (sweeps, middle rows, sweeps back), the counter cleared before
 * each.  Pivoting is getrf's; the factors (of C'_i above the middle row,
 * of the upward sweep's modified blocks below it, of the middle row's
 * matrix at m) stay in the workspace for pyro_block_thomas_seg_resolve.
 * Same arguments as pyro_block_thomas without the CTA size (four warps
 * per CTA); ctas: forward grid size (0 = one or two warps per SM
 * partition by the batch size).  Replaces the same reference function,
 * pyrometheus/flamelets/linear_solver.py:6-103 (the same solution; the
 * reference sweeps top-down only). */
int pyro_block_thomas_seg(const double* L, const double* C, const double* U,
                          const double* b, double* x, const int64_t* row_off,
                          const int* order, int nsys, int nv, double* work,
                          int* counter, int* status, int ctas,
                          cudaStream_t stream);

/* More right-hand sides for systems already solved: after pyro_block_thomas
 * or pyro_block_thomas_small, `work` holds every row's LU factors and
 * pivots of C'_i; for the same L, C, U this solves nrhs (1..4) further
 * systems, B[c][rows][nv] -> X[c][rows][nv] (the c-th at offset
 * c * rhs_stride), with the vector recurrences only (4 nv^2 FMAs per row
 * and right-hand side).  The reference factorises again on every call to
 * block_thomas, pyrometheus/flamelets/linear_solver.py:6-103, including
 * the adjoint solves that share one operator in
 * pyrometheus/flamelets/thermodynamic_consistency.py:105-307.  order and
 * counter as for pyro_block_thomas; status (may be NULL): bit 1 on an empty
 * system; nv <= 64; B and X must not overlap. */
int pyro_block_thomas_resolve(const double* L, const double* U,
                              const double* B, double* X, int nrhs,
                              int64_t rhs_stride, const int64_t* row_off,
                              const int* order, int nsys, int nv,
                              const double* work, int* counter, int* status,
                              cudaStream_t stream);

/* pyro_block_thomas_resolve after pyro_block_thomas_seg: the same
 * arguments (nv <= 16), the vector recurrences of the two-ended sweeps
 * with its kept factors and S | t blocks. */
int pyro_block_thomas_seg_resolve(const double* L, const double* U,
                                  const double* B, double* X, int nrhs,
                                  int64_t rhs_stride, const int64_t* row_off,
                                  const int* order, int nsys, int nv,
                                  const double* work, int* counter,
                                  int* status, cudaStream_t stream);

/* No counterpart in the reference (its block_thomas allocates through JAX
 * on every call).  For callers that cannot allocate device memory when they
 * solve: host applications that hand all device memory to their own pool at
 * start-up and forbid allocation inside a time step (a flow solver's
 * implicit chemistry update), and real-time loops where the latency or a
 * failure of an allocation in the middle of a step is not acceptable.  Same
 * inputs and outputs as
 * pyro_block_thomas, but the per-row workspace and the work counter live in
 * a static device array of the library (16 MiB, held on every GPU that loads
 * the library until the process exits), so the call allocates nothing.
 * Limit: total_rows (= row_off[nsys], passed from the host) at most
 * pyro_block_thomas_noalloc_max_rows(nv) = 2^21 / (nv*nv + 2*nv) rows
 * (17,476 at nv = 10, 693 at nv = 54); larger requests return
 * PYRO_ERR_CAPACITY (5) before anything is launched.  status: bit 0 zero
 * pivot, bit 1 a system's rows outside [0, total_rows).  All calls share
 * the array and it keeps the last call's contents (the counter is cleared
 * by each call, the workspace is written before it is read): calls whose
 * executions overlap on the GPU race and must not be issued.  The first
 * call on a device looks up the array's address with that device current;
 * make that first call before any stream capture. */
int64_t pyro_block_thomas_noalloc_max_rows(int nv);
int pyro_block_thomas_noalloc(const double* L, const double* C,
                              const double* U, const double* b, double* x,
                              const int64_t* row_off, const int* order,
                              int nsys, int nv, int64_t total_rows,
                              int* status, int threads, int ctas,
                              cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PYRO_BLOCK_THOMAS_H */
