// Live FP64 roofline denominators for the benchmark: DFMA throughput of the
// GPU, the FP64-pipe cost of CUDA's double-precision exp and log, and the
// FP64 tensor-core (mma.sync f64) rate that decides whether a small dense
// contraction here should use it instead of DFMA.
//
// Each kernel runs independent dependency chains per thread (enough ILP to
// cover latency) over a grid of several waves; the host times a launch with
// CUDA events.  Results are written through caller-provided device memory.
#include <cstdint>
#include <cuda_runtime.h>

#include "pyro_common.cuh"

namespace {

__global__ void k_dfma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b);
    x3 = fma(x3, a, b); x4 = fma(x4, a, b); x5 = fma(x5, a, b);
    x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] =
      x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_exp(double* out, int iters) {
  double x0 = -1.0 - threadIdx.x * 1e-6, x1 = x0 - 0.1, x2 = x0 - 0.2,
         x3 = x0 - 0.3, s = 0.0;
  for (int i = 0; i < iters; ++i) {
    s += exp(x0) + exp(x1) + exp(x2) + exp(x3);
    x0 -= 1e-7; x1 -= 1e-7; x2 -= 1e-7; x3 -= 1e-7;
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_log(double* out, int iters) {
  double x0 = 1.0 + threadIdx.x * 1e-6, x1 = x0 + 0.1, x2 = x0 + 0.2,
         x3 = x0 + 0.3, s = 0.0;
  for (int i = 0; i < iters; ++i) {
    s += log(x0) + log(x1) + log(x2) + log(x3);
    x0 += 1e-7; x1 += 1e-7; x2 += 1e-7; x3 += 1e-7;
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_rcp(double* out, int iters) {
  double x0 = 1.0 + threadIdx.x * 1e-6, x1 = x0 + 0.1, x2 = x0 + 0.2,
         x3 = x0 + 0.3, s = 0.0;
  for (int i = 0; i < iters; ++i) {
    s += 1.0 / x0 + 1.0 / x1 + 1.0 / x2 + 1.0 / x3;
    x0 += 1e-7; x1 += 1e-7; x2 += 1e-7; x3 += 1e-7;
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 tensor-core (DMMA) throughput: legacy warp-synchronous mma.sync with
// f64 operands (tcgen05 has no f64 kind).  Eight independent accumulator
// tiles per warp keep the pipe fed; the operands stay in registers, so the
// kernel measures the MMA issue rate alone.
__global__ void k_dmma_m8n8k4(double* out, int iters) {
  const double a = 1.0 + threadIdx.x * 1e-9, b = 1.0 - threadIdx.x * 1e-9;
  double d[8][2];
#pragma unroll
  for (int q = 0; q < 8; ++q) d[q][0] = d[q][1] = q * 1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 8; ++q)
      asm volatile(
          "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 "
          "{%0, %1}, {%2}, {%3}, {%0, %1};\n"
          : "+d"(d[q][0]), "+d"(d[q][1])
          : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) s += d[q][0] + d[q][1];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The sm_90+ shape m16n8k16: A 16x16 (8 doubles per lane), B 16x8 (4),
// C/D 16x8 (4); four independent accumulator tiles per warp.
__global__ void k_dmma_m16n8k16(double* out, int iters) {
  double a[8], b[4], d[4][4];
#pragma unroll
  for (int q = 0; q < 8; ++q) a[q] = 1.0 + (threadIdx.x + q) * 1e-9;
#pragma unroll
  for (int q = 0; q < 4; ++q) b[q] = 1.0 - (threadIdx.x + q) * 1e-9;
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int r = 0; r < 4; ++r) d[q][r] = (q + r) * 1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 "
          "{%0, %1, %2, %3}, {%4, %5, %6, %7, %8, %9, %10, %11}, "
          "{%12, %13, %14, %15}, {%0, %1, %2, %3};\n"
          : "+d"(d[q][0]), "+d"(d[q][1]), "+d"(d[q][2]), "+d"(d[q][3])
          : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]),
            "d"(a[5]), "d"(a[6]), "d"(a[7]), "d"(b[0]), "d"(b[1]),
            "d"(b[2]), "d"(b[3]));
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) s += d[q][0] + d[q][1] + d[q][2] + d[q][3];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

// *result = double-precision reciprocals (1.0 / x, IEEE-rounded) per second.
// scratch: pyro_peaks_scratch_doubles() doubles.  Synchronous.
PYRO_EXPORT int pyro_measure_fp64_rcp(double* scratch, double* result,
                                      int repeats) {
  if (!scratch || !result || repeats < 1) return PYRO_ERR_ARGUMENT;
  const int blocks = pyro_sm_count() * 8, threads = 256, iters = 256;
  const double n = (double)blocks * threads;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return PYRO_ERR_LAUNCH;
  if (cudaEventCreate(&e1) != cudaSuccess) return PYRO_ERR_LAUNCH;
  double best = 0.0;
  for (int r = 0; r < repeats + 1; ++r) {
    float ms = 0.f;
    cudaEventRecord(e0);
    k_rcp<<<blocks, threads>>>(scratch, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (r && ms > 0) best = fmax(best, 4.0 * iters * n / (ms * 1e-3));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) return PYRO_ERR_LAUNCH;
  *result = best;
  return PYRO_OK;
}

// Number of doubles the scratch buffer of pyro_measure_fp64 must hold.
PYRO_EXPORT int64_t pyro_peaks_scratch_doubles() {
  return (int64_t)pyro_sm_count() * 8 * 256;
}

// results[0] = DFMA FLOP/s (2 per FMA), results[1] = exp(double)/s,
// results[2] = log(double)/s.  scratch: pyro_peaks_scratch_doubles()
// doubles of device memory.  Synchronous.
PYRO_EXPORT int pyro_measure_fp64(double* scratch, double* results,
                                  int repeats) {
  if (!scratch || !results || repeats < 1) return PYRO_ERR_ARGUMENT;
  const int blocks = pyro_sm_count() * 8, threads = 256;
  const double n = (double)blocks * threads;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return PYRO_ERR_LAUNCH;
  if (cudaEventCreate(&e1) != cudaSuccess) return PYRO_ERR_LAUNCH;
  double best[3] = {0.0, 0.0, 0.0};
  const int it_fma = 4096, it_exp = 256, it_log = 256;
  for (int r = 0; r < repeats + 1; ++r) {
    float ms = 0.f;
    cudaEventRecord(e0);
    k_dfma<<<blocks, threads>>>(scratch, it_fma, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (r && ms > 0) best[0] = fmax(best[0], 16.0 * it_fma * n / (ms * 1e-3));
    cudaEventRecord(e0);
    k_exp<<<blocks, threads>>>(scratch, it_exp);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (r && ms > 0) best[1] = fmax(best[1], 4.0 * it_exp * n / (ms * 1e-3));
    cudaEventRecord(e0);
    k_log<<<blocks, threads>>>(scratch, it_log);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (r && ms > 0) best[2] = fmax(best[2], 4.0 * it_log * n / (ms * 1e-3));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) return PYRO_ERR_LAUNCH;
  for (int q = 0; q < 3; ++q) results[q] = best[q];
  return PYRO_OK;
}

// results[0] = FP64 FLOP/s of mma.sync m8n8k4 (512 flops per warp-wide
// MMA), results[1] = the same for m16n8k16 (4,096 flops per MMA).
// scratch: pyro_peaks_scratch_doubles() doubles.  Synchronous.
PYRO_EXPORT int pyro_measure_dmma(double* scratch, double* results,
                                  int repeats) {
  if (!scratch || !results || repeats < 1) return PYRO_ERR_ARGUMENT;
  const int blocks = pyro_sm_count() * 8, threads = 256;
  const double warps = (double)blocks * threads / 32;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return PYRO_ERR_LAUNCH;
  if (cudaEventCreate(&e1) != cudaSuccess) return PYRO_ERR_LAUNCH;
  double best[2] = {0.0, 0.0};
  const int it_s = 1024, it_l = 128;
  for (int r = 0; r < repeats + 1; ++r) {
    float ms = 0.f;
    cudaEventRecord(e0);
    k_dmma_m8n8k4<<<blocks, threads>>>(scratch, it_s);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (r && ms > 0)
      best[0] = fmax(best[0], 8.0 * it_s * 512.0 * warps / (ms * 1e-3));
    cudaEventRecord(e0);
    k_dmma_m16n8k16<<<blocks, threads>>>(scratch, it_l);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (r && ms > 0)
      best[1] = fmax(best[1], 4.0 * it_l * 4096.0 * warps / (ms * 1e-3));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) return PYRO_ERR_LAUNCH;
  results[0] = best[0];
  results[1] = best[1];
  return PYRO_OK;
}
