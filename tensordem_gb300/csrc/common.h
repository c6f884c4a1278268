// Shared helpers of the tdem CUDA translation units: error plumbing and
// deterministic block reductions.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/tdem.h"

namespace tdem {

// Records `msg` in `err` and returns `code` (used by every C-ABI function).
inline int fail(std::string* err, int code, const std::string& msg) {
  if (err) *err = msg;
  return code;
}

#define TDEM_CUDA_TRY(err_str, expr)                                                   \
  do {                                                                                 \
    cudaError_t e_ = (expr);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      return ::tdem::fail((err_str), TDEM_ERR_CUDA,                                    \
                          std::string(#expr) + ": " + cudaGetErrorString(e_));         \
    }                                                                                  \
  } while (0)

// Block-wide sum of K doubles per thread into `out` (valid in thread 0 only).
// The combination order is fixed by thread index, so the result is
// bit-reproducible run to run. `scratch` must hold K * (blockDim.x / 32)
// doubles. Ends with a __syncthreads so scratch may be reused at once.
template <int K>
__device__ inline void block_sum_f64(double (&v)[K], double* scratch, double (&out)[K]) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double x = v[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if (lane == 0) scratch[k * nwarp + warp] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = scratch[k * nwarp];
      for (int w = 1; w < nwarp; ++w) s += scratch[k * nwarp + w];
      out[k] = s;
    }
  }
  __syncthreads();
}

// Block-wide minimum of one double (valid in thread 0 only).
__device__ inline double block_min_f64(double x, double* scratch) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) x = fmin(x, __shfl_down_sync(0xffffffffu, x, off));
  if (lane == 0) scratch[warp] = x;
  __syncthreads();
  double m = scratch[0];
  if (threadIdx.x == 0)
    for (int w = 1; w < nwarp; ++w) m = fmin(m, scratch[w]);
  __syncthreads();
  return m;
}

}  // namespace tdem
