// Host-side runtime helpers of the package (no kernels): strided
// host<->device copies used to stream species-major state columns in chunks.
#include <cstdint>
#include <cuda_runtime.h>

#include "pyro_common.cuh"

// Copies `height` rows of `width_bytes` bytes between pitched buffers
// (host or device, unified addressing) asynchronously on `stream`; one DMA
// for a [rows, columns-slice] block of a species-major array.
PYRO_EXPORT int pyro_memcpy2d_async(void* dst, int64_t dpitch_bytes,
                                    const void* src, int64_t spitch_bytes,
                                    int64_t width_bytes, int64_t height,
                                    cudaStream_t stream) {
  if (width_bytes < 0 || height < 0 || dpitch_bytes < width_bytes ||
      spitch_bytes < width_bytes)
    return PYRO_ERR_ARGUMENT;
  if (width_bytes == 0 || height == 0) return PYRO_OK;
  if (!dst || !src) return PYRO_ERR_ARGUMENT;
  if (cudaMemcpy2DAsync(dst, (size_t)dpitch_bytes, src, (size_t)spitch_bytes,
                        (size_t)width_bytes, (size_t)height, cudaMemcpyDefault,
                        stream) != cudaSuccess) {
    (void)cudaGetLastError();
    return PYRO_ERR_LAUNCH;
  }
  return PYRO_OK;
}
