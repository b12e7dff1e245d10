// Launch-shape helpers shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

namespace fcg {

constexpr int kTPB = 256;  // threads per block of the streaming and gather kernels

// Grid for a grid-stride loop over `count` items: enough blocks to fill every SM
// (the caller passes the device's SM count) and never more than the items need.
inline int grid_for(long long count, int num_sms, int blocks_per_sm = 8) {
  long long need = (count + kTPB - 1) / kTPB;
  long long cap = (long long)num_sms * blocks_per_sm;
  return (int)std::max(1LL, std::min(need, cap));
}

#define FCG_GRID_STRIDE(i, count)                                                       \
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (count);     \
       i += (long long)gridDim.x * blockDim.x)

}  // namespace fcg
