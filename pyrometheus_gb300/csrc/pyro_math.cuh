// Table-driven double-precision exponential for FP64-bound kernels.
//
// Method: P. T. P. Tang, "Table-driven implementation of the exponential
// function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989, with a
// larger table so the polynomial is short:
//
//   x = (2048 m + j) ln2/2048 + r,   |r| <= ln2/4096,
//   exp(x) = 2^m * 2^(j/2048) * exp(r),
//   exp(r) - 1 ~= r + r^2/2 + r^3/6   (truncation < 0.15 ulp at |r| max).
//
// k = round(x 2048/ln2) comes from adding 1.5 * 2^52 (its low word is k);
// r = x - k L with L = ln2/2048 rounded to double, one FMA.  L's rounding
// (|L - ln2/2048| < 2.7e-20) puts a relative error below |x| 8e-17 on the
// result: under the |x| 1.1e-16 that the rounding of x itself carries
// through exp, so the one-constant reduction loses nothing against the
// argument's own precision (a two-constant Cody-Waite split, PYRO_EXP_L1 /
// L2, would cost one more FMA per call).  The 2^(j/2048) values (correctly
// rounded, exp_table.cuh) are staged in shared memory once per block.
// Cost: 7 FP64 instructions per call (CUDA's exp costs about 20
// DFMA-equivalents on GB300's FP64 pipe).  |x| >= 708, inf and nan go to
// CUDA's exp, which handles overflow, gradual underflow and specials.
#pragma once

#include "exp_table.cuh"

__shared__ double pyro_exp_smem[PYRO_EXP_N];

// Every kernel that calls pyro_exp stages the table first.
#define PYRO_EXP_PRELOAD()                                              \
  do {                                                                  \
    for (int q_ = threadIdx.x; q_ < PYRO_EXP_N; q_ += blockDim.x)       \
      pyro_exp_smem[q_] = pyro_exp_table[q_];                           \
    __syncthreads();                                                    \
  } while (0)

// The table method alone, valid for |x| < 708 (no range check).
__device__ __forceinline__ double pyro_exp_core(double x) {
  const double s = fma(x, PYRO_EXP_INV_L, 0x1.8p52);
  const double kd = s - 0x1.8p52;
  const int k = __double2loint(s);
  const double r = fma(-kd, PYRO_EXP_L, x);
  const double p = fma(r * r, fma(r, 1.0 / 6.0, 0.5), r);
  const double t = pyro_exp_smem[k & (PYRO_EXP_N - 1)];
  const double v = fma(t, p, t);
  const unsigned m = (unsigned)(k >> 11);
  return __hiloint2double(__double2hiint(v) + (int)(m << 20),
                          __double2loint(v));
}

__device__ __forceinline__ double pyro_exp(double x) {
  const int hx = __double2hiint(x) & 0x7fffffff;
  if (hx >= 0x40862000) return exp(x);  // |x| >= 708, inf, nan
  return pyro_exp_core(x);
}

// 10^x as exp(x ln 10) (the reference evaluates 10**x with numpy's power).
__device__ __forceinline__ double pyro_exp10(double x) {
  return pyro_exp(x * 2.302585092994045684);
}

// Table-driven double-precision logarithm (the logarithm counterpart of the
// method above: P. T. P. Tang, "Table-driven implementation of the
// logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4),
// 1990), for the Troe blending of the straight-line rate kernels:
//
//   x = 2^m y, y in [1, 2);  F = 1 + j/128 nearest to y, f = y - F (exact),
//   |f| <= 1/256 + 2^-20,  u = f * (1/F),
//   ln x = m ln2 + ln F + ln(1 + u),
//   ln(1 + u) ~= u - u^2/2 + ... - u^6/6 + u^7/7  (truncation < 2e-18 u).
//
// 1/F and ln F (as hi + lo) are correctly rounded (log_table.cuh) and
// staged in shared memory; ln 2 is split so m * LN2_HI is exact.  About 14
// FP64 instructions per call.  Zero, negative, subnormal, infinite and nan
// arguments go to CUDA's log.
#include "log_table.cuh"

__shared__ double pyro_log_smem[3 * (PYRO_LOG_N + 1)];

// Every kernel that calls pyro_log / pyro_log10 stages the table first.
#define PYRO_LOG_PRELOAD()                                                 \
  do {                                                                     \
    for (int q_ = threadIdx.x; q_ < 3 * (PYRO_LOG_N + 1); q_ += blockDim.x) \
      pyro_log_smem[q_] = pyro_log_table[q_];                              \
    __syncthreads();                                                       \
  } while (0)

// shared memory the two tables take per block
#define PYRO_TABLES_SMEM \
  ((PYRO_EXP_N + 3 * (PYRO_LOG_N + 1)) * sizeof(double))

// kGlobal: read the table from global memory through L1 (kernels whose
// shared memory is spoken for) instead of the staged copy
template <bool kGlobal>
__device__ __forceinline__ double pyro_log_t(double x) {
  const int hx = __double2hiint(x);
  if (hx < 0x00100000 || hx >= 0x7ff00000) return log(x);
  const int mant = hx & 0x000fffff;
  const int m = (hx >> 20) - 1023;
  const double y = __hiloint2double(mant | 0x3ff00000, __double2loint(x));
  const int j = (mant + (1 << 12)) >> 13;  // nearest j/128, 0..128
  const double F = (double)(PYRO_LOG_N + j) * (1.0 / PYRO_LOG_N);
  const double f = y - F;
  double t0, t1, t2;
  if (kGlobal) {
    const double* t = pyro_log_table + 3 * j;
    t0 = __ldg(t);
    t1 = __ldg(t + 1);
    t2 = __ldg(t + 2);
  } else {
    const double* t = pyro_log_smem + 3 * j;
    t0 = t[0];
    t1 = t[1];
    t2 = t[2];
  }
  const double u = f * t0;
  // ln(1 + u) = u + u^2 (-1/2 + u (1/3 + u (-1/4 + u (1/5 + u (-1/6 +
  // u / 7)))))
  const double lp = fma(u * u, fma(u, fma(u, fma(u, fma(u, fma(u, 1.0 / 7.0,
                                                               -1.0 / 6.0),
                                                        1.0 / 5.0),
                                                 -1.0 / 4.0),
                                          1.0 / 3.0),
                                   -0.5),
                        u);
  const double md = (double)m;
  const double hi = fma(md, PYRO_LOG_LN2_HI, t1);
  const double lo = fma(md, PYRO_LOG_LN2_LO, t2) + lp;
  return hi + lo;
}

__device__ __forceinline__ double pyro_log(double x) {
  return pyro_log_t<false>(x);
}

// log10 with the table read from global memory (no staging)
__device__ __forceinline__ double pyro_log10_g(double x) {
  return pyro_log_t<true>(x) * PYRO_LOG_INV_LN10;
}

__device__ __forceinline__ double pyro_log10(double x) {
  return pyro_log(x) * PYRO_LOG_INV_LN10;
}

