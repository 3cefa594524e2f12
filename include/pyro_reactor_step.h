/*
 * Per-cell reductions of the implicit 0-D reactor integrator
 * (libpyro_reactor_step_<hash>.so).
 *
 * The reference's implicit reactor step tests Newton convergence with
 * jnp.linalg.norm(dy) < tol for one reactor
 * (pyrometheus/examples/free_flame/time_integ.py:89-100); the batched
 * integrator here uses a weighted RMS norm per cell, summed in a fixed
 * order by one thread per cell so that a cell's step control does not
 * depend on the other cells of the batch.
 */
#ifndef PYRO_REACTOR_STEP_H
#define PYRO_REACTOR_STEP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* cudaStream_t;

/* out[i] = sqrt(sum_k (v[k*ldv + i] / w[k*ldw + i])^2 / nv), i < n, the
 * sum taken over k = 0 .. nv-1 in order.  Device pointers, FP64;
 * ldv, ldw >= n.  Returns 0 or a PyroStatus code (1 argument, 2 launch). */
int pyro_wrms_columns(const double* v, int64_t ldv, const double* w,
                      int64_t ldw, int nv, int64_t n, double* out,
                      cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PYRO_REACTOR_STEP_H */
