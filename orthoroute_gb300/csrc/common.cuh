// Shared helpers for the GB300 PathFinder kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/orthoroute_gb300.h"

#define OGR_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return OGR_ERR_CUDA;              \
  } while (0)

#define OGR_LAUNCH_CHECK() OGR_CUDA_TRY(cudaGetLastError())

static inline cudaStream_t ogr_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

static inline int ogr_blocks(int64_t n, int threads, int cap = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

// Non-negative doubles order like their bit patterns as unsigned integers.
__device__ __forceinline__ unsigned long long ogr_dbits(double d) {
  return (unsigned long long)__double_as_longlong(d);
}
