// The per-warp 16-cell tile of one message-passing layer of the learned preconditioner,
// shared by every form of the layer kernel (learned.cu: the sliced gather form and the
// split form; learned_hex.cu: the plane-staged form for lexicographic hex meshes), so
// that all of them round identically.
//
// A warp holds 16 cells as BF16 rows [h; m] (64 values, padded to kTileStride) in
// shared memory.  The 64 -> 32 product runs as 4 k-steps x 4 n-blocks of
// mma.sync.m16n8k16 (BF16 operands, FP32 accumulation), W_l staged in shared memory with
// the same padding.  The epilogue adds the bias, applies the ReLU and the skip
// connection, h' = h + relu(W [h; m] + b), and writes h' over the h half of the tile.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace fcg {
namespace lp {

constexpr int kTileC = 32;                 // channels
constexpr int kTileStride = 2 * kTileC + 8;  // padded BF16 row of the [h; m] tile and of W_l

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Four 8x8 BF16 matrices from shared memory, one 16-byte row address per lane (lanes
// 8m..8m+7 give the rows of matrix m); register m of each lane gets the lane's pair
// (row lane/4, columns 2(lane%4), +1) of matrix m: the mma.m16n8k16 fragment layout.
__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const __nv_bfloat16 *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"((unsigned)__cvta_generic_to_shared(p)));
}

// acc[0..7] = fma(v, 8 BF16 values packed in q, acc): one neighbour's term of m = Ahat h
// for eight channels.  The explicit fused multiply-add fixes the rounding for every
// kernel form.
__device__ __forceinline__ void fma8(float (&acc)[8], float v, const uint4 &q) {
  const __nv_bfloat162 *e = reinterpret_cast<const __nv_bfloat162 *>(&q);
  const float2 vv = make_float2(v, v);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    // packed FP32 FMA: each half is fma(v, h, acc), rounded to nearest
    const float2 r =
        __ffma2_rn(vv, __bfloat1622float2(e[c]), make_float2(acc[2 * c], acc[2 * c + 1]));
    acc[2 * c] = r.x;
    acc[2 * c + 1] = r.y;
  }
}

// The network's output before its scaling, w_out . h + b_out, over one BF16 row of
// kTileC channels held in v, in channel order (w = [w_out, b_out]).
__device__ __forceinline__ float out_dot_vals(const uint4 (&v)[4], const float *w) {
  float acc = w[kTileC];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v[q]);
#pragma unroll
    for (int c = 0; c < 8; ++c) acc += w[q * 8 + c] * bf(e[c]);
  }
  return acc;
}

// out_dot_vals of a row in shared memory (16-byte aligned).
__device__ __forceinline__ float out_dot_row(const __nv_bfloat16 *row, const float *w) {
  uint4 v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = reinterpret_cast<const uint4 *>(row)[q];
  return out_dot_vals(v, w);
}

// Stores row `row` of the warp's tile: own = the cell's h (8 channels at qc), acc = its
// m (FP32 sums, rounded to BF16 here).
__device__ __forceinline__ void tile_put_row(__nv_bfloat16 *tw, int row, int qc, const uint4 &own,
                                             const float (&acc)[8], __nv_bfloat16 (&mb)[8]) {
  __nv_bfloat16 *p = tw + row * kTileStride;
  *reinterpret_cast<uint4 *>(p + qc) = own;
#pragma unroll
  for (int c = 0; c < 8; ++c) mb[c] = __float2bfloat16(acc[c]);
  *reinterpret_cast<uint4 *>(p + kTileC + qc) = *reinterpret_cast<const uint4 *>(mb);
}

// The product and epilogue of one tile (every lane of the warp; the tile complete).
// zout(row, col, z0, z1) receives the pre-activations of channels col, col+1 of tile row
// `row` (training); pass a no-op otherwise.
template <class ZOut>
__device__ __forceinline__ void tile_dense(__nv_bfloat16 *tw, const __nv_bfloat16 *wsm,
                                           const float *bsm, int lane, ZOut zout) {
  constexpr int TS = kTileStride;
  const int g = lane >> 2, tg = lane & 3;
  float d[4][4];
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) d[nt][q] = 0.f;
  // fragment rows by ldmatrix: A, matrices (rows 0-7 | 8-15) x (k 0-7 | 8-15) of the
  // k-step; B, for two n-blocks at a time, (n-block) x (k 0-7 | 8-15) of W_l's rows
  const int mi = lane >> 3, mr = lane & 7;
  const __nv_bfloat16 *pa = tw + (mr + 8 * (mi & 1)) * TS + 8 * (mi >> 1);
  const __nv_bfloat16 *pb = wsm + (8 * (mi >> 1) + mr) * TS + 8 * (mi & 1);
#pragma unroll
  for (int kb = 0; kb < 4; ++kb) {
    unsigned a[4], b[4];
    ldsm_x4(a, pa + kb * 16);
    ldsm_x4(b, pb + kb * 16);
    mma_bf16(d[0], a, b[0], b[1]);
    mma_bf16(d[1], a, b[2], b[3]);
    ldsm_x4(b, pb + 16 * TS + kb * 16);
    mma_bf16(d[2], a, b[0], b[1]);
    mma_bf16(d[3], a, b[2], b[3]);
  }
  __syncwarp();  // every lane has its fragments: the h part of the tile may change
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int rr = g + 8 * hh, col = nt * 8 + tg * 2;
      const float z0 = d[nt][2 * hh] + bsm[col], z1 = d[nt][2 * hh + 1] + bsm[col + 1];
      __nv_bfloat162 *hp = reinterpret_cast<__nv_bfloat162 *>(tw + rr * TS + col);
      const __nv_bfloat162 hold = *hp;
      __nv_bfloat162 o;
      o.x = __float2bfloat16(bf(hold.x) + fmaxf(z0, 0.f));
      o.y = __float2bfloat16(bf(hold.y) + fmaxf(z1, 0.f));
      *hp = o;
      zout(rr, col, z0, z1);
    }
  }
  __syncwarp();
}

struct NoZ {
  __device__ __forceinline__ void operator()(int, int, float, float) const {}
};

}  // namespace lp
}  // namespace fcg
