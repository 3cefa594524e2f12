// Per-cell reductions of the implicit 0-D reactor integrator (FP64,
// sm_103a).
//
// The integrator's step control needs, for every cell i, the weighted
// root-mean-square norm  sqrt(mean_k (v[k][i] / w[k][i])^2)  over the
// nv = S + 1 unknowns of the cell.  A library reduction over the unknown
// axis may split that sum across threads differently for different batch
// sizes, which would make a cell's rounding (and so its accepted steps)
// depend on what else is in the batch.  Here one thread owns one cell and
// adds its nv terms in a fixed order, so the result is a function of the
// cell's own data only.  Species-major layout ([nv][ld], unit stride along
// cells): a warp reads 32 consecutive cells of one row per load.
#include <cstdint>
#include <cuda_runtime.h>

#include "pyro_common.cuh"

namespace {

__global__ void k_wrms(const double* __restrict__ v, int64_t ldv,
                       const double* __restrict__ w, int64_t ldw, int nv,
                       int64_t n, double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < nv; ++k) {
      const double q = __ldg(v + k * ldv + i) / __ldg(w + k * ldw + i);
      acc = fma(q, q, acc);
    }
    out[i] = sqrt(acc / nv);
  }
}

}  // namespace

// out[i] = sqrt(sum_k (v[k*ldv + i] / w[k*ldw + i])^2 / nv) for i < n,
// summed over k in increasing order.  Asynchronous on `stream`.
PYRO_EXPORT int pyro_wrms_columns(const double* v, int64_t ldv,
                                  const double* w, int64_t ldw, int nv,
                                  int64_t n, double* out,
                                  cudaStream_t stream) {
  if (n < 0 || nv < 1 || ldv < n || ldw < n) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  if (!v || !w || !out) return PYRO_ERR_ARGUMENT;
  const int block = 256;
  k_wrms<<<pyro_grid(n, block, pyro_sm_count() * 16), block, 0, stream>>>(
      v, ldv, w, ldw, nv, n, out);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}
