// Evaluates pyro_exp / pyro_exp10 and CUDA's exp / exp10 on the same inputs,
// so tests can bound the table-driven exponential against CUDA's outputs.
#include <cstdint>
#include <cuda_runtime.h>

#include "pyro_common.cuh"
#include "pyro_math.cuh"

namespace {

__global__ void k_expcheck(const double* __restrict__ x, double* mine,
                           double* ref, int ten, int64_t n) {
  PYRO_EXP_PRELOAD();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    mine[i] = ten ? pyro_exp10(v) : pyro_exp(v);
    ref[i] = ten ? exp10(v) : exp(v);
  }
}

}  // namespace

// mine[i] = pyro_exp(x[i]) (pyro_exp10 when ten != 0), ref[i] = CUDA's
// exp (exp10).  Device pointers; asynchronous on stream.
PYRO_EXPORT int pyro_exp_check(const double* x, double* mine, double* ref,
                               int ten, int64_t n, cudaStream_t stream) {
  if (n < 0 || (n > 0 && (!x || !mine || !ref))) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  k_expcheck<<<pyro_grid(n, 256, pyro_sm_count() * 4), 256, 0, stream>>>(
      x, mine, ref, ten, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

namespace {

__global__ void k_logcheck(const double* __restrict__ x, double* mine,
                           double* ref, int ten, int64_t n) {
  PYRO_LOG_PRELOAD();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    mine[i] = ten ? pyro_log10(v) : pyro_log(v);
    ref[i] = ten ? log10(v) : log(v);
  }
}

}  // namespace

// mine[i] = pyro_log(x[i]) (pyro_log10 when ten != 0), ref[i] = CUDA's
// log (log10).  Device pointers; asynchronous on stream.
PYRO_EXPORT int pyro_log_check(const double* x, double* mine, double* ref,
                               int ten, int64_t n, cudaStream_t stream) {
  if (n < 0 || (n > 0 && (!x || !mine || !ref))) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  k_logcheck<<<pyro_grid(n, 256, pyro_sm_count() * 4), 256, 0, stream>>>(
      x, mine, ref, ten, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}

namespace {

__global__ void k_rcpcheck(const double* __restrict__ x, double* mine,
                           double* ref, int third, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    mine[i] = third ? pyro_rcp3(v) : pyro_rcp(v);
    ref[i] = 1.0 / v;
  }
}

}  // namespace

// mine[i] = pyro_rcp(x[i]) (third = 0) or pyro_rcp3(x[i]) (third = 1),
// ref[i] = CUDA's 1.0 / x[i].  Device pointers; asynchronous on stream.
PYRO_EXPORT int pyro_rcp_check(const double* x, double* mine, double* ref,
                               int third, int64_t n, cudaStream_t stream) {
  if (n < 0 || (n > 0 && (!x || !mine || !ref))) return PYRO_ERR_ARGUMENT;
  if (n == 0) return PYRO_OK;
  k_rcpcheck<<<pyro_grid(n, 256, pyro_sm_count() * 4), 256, 0, stream>>>(
      x, mine, ref, third, n);
  PYRO_CHECK_LAUNCH();
  return PYRO_OK;
}
