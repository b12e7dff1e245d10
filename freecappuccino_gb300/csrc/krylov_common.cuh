// Device helpers shared by the solver translation units: deterministic grid-wide sums
// and the sliced-ELL row product.
#pragma once

#include <cuda_runtime.h>

#include "fcg_internal.h"
#include "launch.h"

namespace fcg {

constexpr int kWarps = kTPB / 32;

// ---------------------------------------------------------------------------
// Deterministic reductions
// ---------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (*sh)[kWarps]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][w] = v[k];
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = lane < kWarps ? sh[k][lane] : 0.0;
#pragma unroll
    for (int o = kWarps / 2; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < NV; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  __syncthreads();
}

// Stores this block's sums; returns true in the last block to arrive, whose thread 0
// then holds the grid-wide sums in v (partials added in block-index order).
template <int NV>
__device__ __forceinline__ bool reduce_commit(double (&v)[NV], double *partials, unsigned int *ticket) {
  __shared__ double sh[NV][kWarps];
  __shared__ bool am_last;
  block_sum<NV>(v, sh);
  const int G = gridDim.x;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * G + blockIdx.x] = v[k];
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    am_last = (t == (unsigned int)G - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) s[k] = 0.0;
  for (int i = threadIdx.x; i < G; i += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] += __ldcg(&partials[k * G + i]);
  block_sum<NV>(s, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = s[k];
    *ticket = 0u;
  }
  return true;
}

// Row sum of A x for lane `lane` of slice `slice` (one warp per slice).  Uniform
// slices read one shared offset per slot (a broadcast load) instead of 32 columns.
// V is the value type, X the vector type; the sum is accumulated in V*X's type.
template <class V, class X>
__device__ __forceinline__ decltype(V(0) * X(0)) sell_row(const SellView &s, int n,
                                                         const V *__restrict__ val,
                                                         const X *__restrict__ x, int slice,
                                                         int lane) {
  using A = decltype(V(0) * X(0));
  const long long base = __ldg(&s.ptr[slice]) + lane;
  const int w = __ldg(&s.width[slice]), op = __ldg(&s.offp[slice]);
  A acc = 0;
  const int kind = __ldg(&s.kind[slice]);
  if (sizeof(V) == 4 && kind == 0 && w <= 8) {
    // all loads of the row issue before the first multiply-add
    const int row = slice * 32 + lane;
    V v[8];
    X xv[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (j < w) {
        int c = row + __ldg(&s.off[op + j]);
        c = c < 0 ? 0 : (c >= n ? n - 1 : c);
        v[j] = __ldg(&val[base + (long long)j * 32]);
        xv[j] = __ldg(&x[c]);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (j < w) acc += (A)v[j] * (A)xv[j];
  } else if (kind == 0) {
    const int row = slice * 32 + lane;
    for (int j = 0; j < w; ++j) {
      int c = row + __ldg(&s.off[op + j]);
      c = c < 0 ? 0 : (c >= n ? n - 1 : c);
      acc += (A)__ldg(&val[base + (long long)j * 32]) * (A)__ldg(&x[c]);
    }
  } else {
#pragma unroll 4
    for (int j = 0; j < w; ++j)
      acc += (A)__ldg(&val[base + (long long)j * 32]) *
             (A)__ldg(&x[__ldg(&s.off[op + 32 * j + lane])]);
  }
  return acc;
}

#define FCG_SLICE_LOOP(slice, lane, s)                                                      \
  const int lane = threadIdx.x & 31;                                                       \
  for (int slice = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);        \
       slice < (s).nslices; slice += (int)(((long long)gridDim.x * blockDim.x) >> 5))


}  // namespace fcg
