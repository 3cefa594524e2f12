// Shared device/host helpers for the generated per-mechanism kernels and the
// mechanism-independent kernels (block-Thomas, batched LU).
//
// Layout conventions (all FP64):
//   * per-species / per-reaction arrays are species-major: x[k * ld + i] for
//     state i, with ld >= n (unit stride along the state axis, so a warp's
//     32 consecutive states read one 256-byte row segment);
//   * per-state scalars take an element increment: inc = 1 for an array,
//     inc = 0 to broadcast a single device value to every state.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#ifndef PYRO_EXPORT
#define PYRO_EXPORT extern "C" __attribute__((visibility("default")))
#endif

// Status codes returned by every C-ABI entry point.
enum PyroStatus : int {
  PYRO_OK = 0,
  PYRO_ERR_ARGUMENT = 1,      // null pointer, negative size, ld < n, ...
  PYRO_ERR_LAUNCH = 2,        // a CUDA launch or runtime call failed
  PYRO_ERR_NOT_CONVERGED = 3, // some states' Newton iteration failed
  PYRO_ERR_UNSUPPORTED = 4,   // option not supported for this mechanism
  PYRO_ERR_CAPACITY = 5,      // request larger than a fixed static scratch
};

#define PYRO_CHECK_LAUNCH()                                   \
  do {                                                        \
    if (cudaPeekAtLastError() != cudaSuccess) {               \
      (void)cudaGetLastError();                               \
      return PYRO_ERR_LAUNCH;                                 \
    }                                                         \
  } while (0)

// Grid size for a 1-state-per-thread launch: enough blocks to cover n, capped
// at a whole number of waves (the kernels are grid-stride loops).
static inline int pyro_grid(int64_t n, int block, int max_blocks) {
  int64_t b = (n + block - 1) / block;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

// SM count of the current device (152 on GB300).
static inline int pyro_sm_count() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) ==
          cudaSuccess && sms > 0)
    return sms;
  return 152;
}

__device__ __forceinline__ double pyro_ld(const double* __restrict__ p,
                                          int64_t inc, int64_t i) {
  return __ldg(p + inc * i);
}

// 1/x by Newton-Raphson (Markstein, IBM J. Res. Dev. 34(1), 1990): the
// hardware approximation rcp.approx.ftz.f64 as the seed, then two steps of
// r <- r + r (1 - x r), each roughly doubling the correct bits; within an
// ulp of the correctly rounded reciprocal for normal x whose reciprocal is
// normal, and branch-free (so the scheduler can overlap it with
// independent work), unlike the IEEE division.  x = 0 or a subnormal x
// gives nan, not inf; callers use it on pivots they flag as singular when
// zero.
__device__ __forceinline__ double pyro_rcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

// 1/x with one third-order step instead of two Newton-Raphson steps: with
// the seed r = (1 - e) / x, 1/x = r (1 + e + e^2 + ...), so
// r (1 + (e + e^2)) leaves a relative error of order e^3 -- below double
// rounding for seeds good to 2^-18 -- in three FMAs instead of four (the
// same series Markstein's paper truncates after e).  Same special cases as
// pyro_rcp; checked against the IEEE division like it.
__device__ __forceinline__ double pyro_rcp3(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
}
