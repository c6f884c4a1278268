// Shared helpers of the tdem CUDA translation units: error plumbing and
// deterministic block reductions.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/tdem.h"

namespace tdem {

// Records `msg` in `err` and returns `code` (used by every C-ABI function).
inline int fail(std::string* err, int code, const std::string& msg) {
  if (err) *err = msg;
  return code;
}

// Host memcpy split over up to 8 threads for large copies (the staging of
// host arrays through pinned buffers is bound by one core's copy rate).
inline void parallel_copy(void* dst, const void* src, size_t bytes) {
  constexpr size_t kChunk = size_t(4) << 20;
  const size_t parts = std::min<size_t>(8, bytes / kChunk);
  if (parts < 2) {
    std::memcpy(dst, src, bytes);
    return;
  }
  const size_t step = (bytes / parts + 63) & ~size_t(63);
  std::vector<std::thread> workers;
  for (size_t k = 1; k < parts; ++k) {
    const size_t a = k * step;
    if (a >= bytes) break;
    workers.emplace_back([=] {
      std::memcpy(static_cast<char*>(dst) + a, static_cast<const char*>(src) + a, std::min(step, bytes - a));
    });
  }
  std::memcpy(dst, src, std::min(step, bytes));
  for (auto& w : workers) w.join();
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
