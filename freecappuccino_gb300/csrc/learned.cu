// Learned preconditioner and flexible CG (no counterpart in the reference; it builds on
// the DPCG of dpcg.f90, which stays the fallback and the check on the result).
//
// The network maps the residual of the Jacobi-scaled pressure system,
// r^ = D^-1/2 r with Ahat = D^-1/2 A D^-1/2, to an approximation of its error
// e^ = Ahat^-1 r^.  Width C = 32, L = 6 layers, F = 6 inputs per cell:
//   f  = [r^/rms(r^), log(a_PP / vol^1/3) - log 6, log(vol n / sum vol),
//         sum|S_x| / (2 vol^2/3) - 1, same for y and z]
//   h0 = relu(W_in f + b_in)
//   h_l = h_{l-1} + relu(W_l [h_{l-1}; Ahat h_{l-1}] + b_l)        (W_l: 32 x 64)
//   z  = r^ + rms(r^) (w_out . h_L + b_out)
// The skip r^ is the Jacobi preconditioner of dpcg.f90 in the scaled system; the output
// layer starts at zero, so the untrained network is exactly that preconditioner.
// Activations are stored in BF16.  The 64 -> 32 products of the layers run on tensor
// cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation; weights staged in shared
// memory); the aggregation Ahat h gathers BF16 neighbour activations through the FP32
// scaled matrix of the sliced layout the solvers use.  Training minimises, on
// (residual, error) pairs, the error of z in the residual norm,
// |Ahat z - r^|^2 / |r^|^2 = |Ahat (z - e^)|^2 / |Ahat e^|^2 (default), or in the energy
// norm (z - e^).Ahat (z - e^) / e^.Ahat e^.  Measured on jittered 64^3 and 128^3
// pressure systems, the energy-norm loss drives the network towards corrections of the
// smooth error that six hops cannot represent and the flexible CG stalls, while the
// residual-norm loss (the sparse-approximate-inverse criterion) gives 3.4-4.5x fewer
// iterations than Jacobi.  It keeps FP32 master weights: the forward pass saves its
// pre-activations, the backward pass runs in FP32
// (the BF16 roundings pass gradients through unchanged), weight gradients are summed per
// block and then over blocks in index order (deterministic), and Adam updates the
// weights and refreshes their BF16 copies.
//
// Flexible CG (Notay, SIAM J. Sci. Comput. 22 (2000) 1444, truncated to the last m
// directions, m <= 8): z = N(r), p = z - sum_j (z.q_j / p_j.q_j) p_j, q = Ahat p,
// alpha = p.r / p.q.  Keeping several directions makes the iteration robust to the
// network being a nonlinear preconditioner.  It runs in FP32 on the scaled system with reliable updates in
// FP64 (true residual su - A x recomputed, correction folded into the FP64 solution,
// also at least every `ru_every` iterations) and the reference's L1 stop test on the
// true residual.  When the true residual has not fallen by `stall_factor` within
// `stall_window` iterations, or a value turns non-finite, the solve continues with
// the FP64 DPCG from the current solution for the remaining sweeps.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "coarse.h"
#include "fcg_internal.h"
#include "krylov_common.cuh"
#include "launch.h"
#include "lp_hex.h"
#include "lp_tile.cuh"

namespace fcg {
namespace lp {

constexpr int C = 32, L = 6, F = 6;
constexpr int kLayerParams = 2 * C * C + C;  // W_l (32 x 64, row-major [out][in]) + b_l
constexpr int oWin = 0, oBin = C * F, oLayer0 = C * F + C;
constexpr int oWout = oLayer0 + L * kLayerParams, oBout = oWout + C;
constexpr int P = oBout + 1;
static_assert(P == FCG_LP_PARAMS, "parameter count must match the header");
static_assert(oBin == oWin + C * F && oLayer0 == oBin + C, "parameter layout");
constexpr int kBwdTile = 64;            // cells per shared-memory tile of the layer backward
static_assert(kTileC == C && kTileStride == 2 * C + 8, "tile layout of lp_tile.cuh");
constexpr int kRed = 8;                 // reduction tickets
constexpr int kMaxDir = 8;              // most previous directions the FCG keeps

// Device scalars of one learned FCG solve.
struct LScal {
  double res0, resl, small, resmax;
  double rr, maxr, l1ratio, delta;
  double pqs[kMaxDir];  // p_j . Ahat p_j of the stored directions (ring slots)
  double bets[kMaxDir]; // z . q_j / p_j . q_j of the current iteration
  double alf;
  double chk_l1, stall_factor;
  double l2r, l2b;
  int iter, nsw, done, converged, status, ru, nupdates, last_ru;
  int chk_iter, stall_window, ru_every;
  int mdir, nwin, head;  // directions kept, directions stored, slot of the next one
  unsigned int ticket[kRed];
  unsigned int body_count;
};

}  // namespace lp
}  // namespace fcg

using fcg::DBuf;

struct fcg_learned {
  int device = 0;
  int num_sms = 0;
  std::string err;
  DBuf params, adam_m, adam_v, grad, wbf;  // FP32 master weights, Adam moments, gradient, BF16 W_l
  long long step = 0;
  // workspaces (sized for the largest mesh seen)
  size_t ncap = 0;
  bool train_cap = false;
  DBuf feat, hbuf, mbuf, zbuf, dh, dh2, dm, y, dvec, part, red, scal;
  // which context, mesh and matrix the features belong to
  unsigned long long fuid = 0;
  unsigned fgen = 0;
  const void *fmat = nullptr;
  // recorded at the end of every call that queues work; calls for another context and
  // host reads of the weights wait for it (the context's stream may be gone by then)
  cudaEvent_t ev_last = nullptr;
  bool ev_pending = false;
  unsigned long long last_uid = 0;
  // flexible CG
  DBuf fvec;
  fcg::lp::LScal *S = nullptr, *hS = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  std::vector<const void *> graph_key;
  cudaStream_t cap = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int mdir = 8, ru_every = 50, stall_window = 400;
  int loss_kind = 1;  // 0 energy norm, 1 residual norm
  double stall_factor = 0.5, delta = 0.1;
  // coarse-grid correction of the flexible CG (coarse.cu, aggregation.cpp)
  fcg::ml::Options mlo;
  std::vector<fcg::ml::Hierarchy *> mlc;  // one per context, least recently used first
  // plane-staged layer (learned_hex.cu) for the context and mesh it was detected on,
  // and the stencil value planes of the matrix loaded last
  fcg::lphex::HexGrid hex;
  unsigned long long hex_uid = 0;
  unsigned hex_gen = 0;
  DBuf hexval;
};

namespace fcg {
namespace {

using lp::C;
using lp::F;
using lp::L;
using lp::LScal;
using lp::P;

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ bool stopped(const int *done) { return done && __ldcg(done) != 0; }

// ---------------------------------------------------------------------------
// Features
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTPB, 8)
    k_lp_volsum(int n, const double *__restrict__ vol, double *partials, unsigned *ticket,
                double *out) {
  double v[1] = {0.0};
  FCG_GRID_STRIDE(i, n) v[0] += vol[i];
  if (reduce_commit<1>(v, partials, ticket) && threadIdx.x == 0) out[0] = v[0];
}

__global__ void k_lp_features(MeshView m, const double *__restrict__ s64,
                              const double *__restrict__ vsum, float *__restrict__ feat) {
  const double vmean = vsum[0] / m.n;
  FCG_GRID_STRIDE(i, m.n) {
    const double v = m.vol[i], d = 1.0 / (s64[i] * s64[i]);
    const double h = (double)cbrtf((float)v);  // the features are FP32
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int e = m.cf_ptr[i]; e < m.cf_ptr[i + 1]; ++e) {
      const int ent = m.cf_ent[e], f = (ent > 0 ? ent : -ent) - 1;
      ax += fabs(m.arx[f]);
      ay += fabs(m.ary[f]);
      az += fabs(m.arz[f]);
    }
    for (int e = m.cb_ptr[i]; e < m.cb_ptr[i + 1]; ++e) {
      const int f = m.cb_face[e];
      ax += fabs(m.arx[f]);
      ay += fabs(m.ary[f]);
      az += fabs(m.arz[f]);
    }
    const double a2 = 2.0 * h * h;
    const long long nn = m.n;  // feature-major: feature k of cell i at k * n + i
    feat[i] = 0.f;
    feat[nn + i] = logf((float)(d / h)) - 1.7917595f;  // log 6
    feat[2 * nn + i] = logf((float)(v / vmean));
    feat[3 * nn + i] = (float)(ax / a2 - 1.0);
    feat[4 * nn + i] = (float)(ay / a2 - 1.0);
    feat[5 * nn + i] = (float)(az / a2 - 1.0);
  }
}

// ---------------------------------------------------------------------------
// Forward
// ---------------------------------------------------------------------------
// rms of r (FP32 squares, FP64 sums); 1 for a zero vector.
__global__ void __launch_bounds__(kTPB, 8)
    k_lp_rms(int n, const float *__restrict__ x, double *partials, unsigned *ticket,
             float *__restrict__ out, const int *done) {
  if (stopped(done)) return;
  float t = 0.f;
  FCG_GRID_STRIDE(i, n) t += x[i] * x[i];
  double v[1] = {(double)t};
  if (reduce_commit<1>(v, partials, ticket) && threadIdx.x == 0)
    out[0] = v[0] > 0 ? (float)sqrt(v[0] / n) : 1.0f;
}

// f0 = r / rms (stored as feature 0); h0 = relu(W_in f + b_in) in BF16; z0
// (pre-activation) when training.  Features are feature-major (k * n + i).  One thread
// per cell, the weights broadcast from shared memory; each warp stages its 32 x 32 BF16
// output tile in shared memory (rows padded to 80 bytes, so the 16-byte writes of eight
// lanes fall in distinct banks) and stores it as 2 KB of contiguous 16-byte writes.
constexpr int kEmbRow = 40;  // BF16 elements per staged row (32 + 8 padding)

// Four blocks per SM (at most 64 registers): with two, the six feature loads of a cell
// were not hidden.
__global__ void __launch_bounds__(kTPB, 4)
    k_lp_embed(int n, const float *__restrict__ r, const float *__restrict__ rms,
               float *__restrict__ feat, const float *__restrict__ prm,
               __nv_bfloat16 *__restrict__ h0, float *__restrict__ z0, const int *done) {
  if (stopped(done)) return;
  // weights of output channels 2p and 2p+1 side by side: w2[p * F + k], biases after them
  __shared__ float2 w2[C / 2 * F + C / 2];
  __shared__ __align__(16) __nv_bfloat16 tile[kTPB / 32][32 * kEmbRow];
  for (int t = threadIdx.x; t < C / 2 * F; t += blockDim.x) {
    const int pr = t / F, k = t % F;
    w2[t] = make_float2(prm[lp::oWin + 2 * pr * F + k], prm[lp::oWin + (2 * pr + 1) * F + k]);
  }
  for (int pr = threadIdx.x; pr < C / 2; pr += blockDim.x)
    w2[C / 2 * F + pr] = make_float2(prm[lp::oWin + C * F + 2 * pr], prm[lp::oWin + C * F + 2 * pr + 1]);
  __syncthreads();
  const float inv = 1.0f / rms[0];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __nv_bfloat16 *my = tile[warp];
  const long long nwarps = (long long)gridDim.x * (kTPB / 32);
  for (long long base = ((long long)blockIdx.x * (kTPB / 32) + warp) * 32; base < n;
       base += nwarps * 32) {
    const long long i = base + lane;
    if (i < n) {
      float f[F];
      f[0] = r[i] * inv;
      feat[i] = f[0];
#pragma unroll
      for (int k = 1; k < F; ++k) f[k] = feat[k * (long long)n + i];
#pragma unroll
      for (int g = 0; g < C / 8; ++g) {
        __align__(16) __nv_bfloat16 hv[8];
#pragma unroll
        for (int o = 0; o < 4; ++o) {  // channels 2p, 2p+1: z = fma(w, f, z) for k in order
          const int pr = g * 4 + o;
          float2 z = w2[C / 2 * F + pr];
#pragma unroll
          for (int k = 0; k < F; ++k) z = __ffma2_rn(w2[pr * F + k], make_float2(f[k], f[k]), z);
          if (z0) {
            z0[i * C + 2 * pr] = z.x;
            z0[i * C + 2 * pr + 1] = z.y;
          }
          hv[2 * o] = __float2bfloat16(fmaxf(z.x, 0.f));
          hv[2 * o + 1] = __float2bfloat16(fmaxf(z.y, 0.f));
        }
        *reinterpret_cast<uint4 *>(my + lane * kEmbRow + g * 8) =
            *reinterpret_cast<const uint4 *>(hv);
      }
    }
    __syncwarp();
    // 32 rows x 64 bytes = 128 chunks of 16 bytes, four per lane
    const long long rows = n - base < 32 ? n - base : 32;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = lane + 32 * j, row = c >> 2, part = c & 3;
      if (row < rows)
        *reinterpret_cast<uint4 *>(h0 + (base + row) * C + part * 8) =
            *reinterpret_cast<const uint4 *>(my + row * kEmbRow + part * 8);
    }
    __syncwarp();
  }
}

using lp::fma8;

// One message-passing layer.  Tiles are dealt to warps grid-stride, so all blocks work
// on one narrow band of the mesh at a time and the rows at +-N^2 that a tile gathers were
// loaded moments before by other blocks (L2 hits); a contiguous run of tiles per block
// measured 14% slower at 256^3.  A warp owns 16 cells (one tile) at a time and takes them
// in two rounds of 8: four lanes per cell, eight channels per lane, sum
// m = Ahat h over the cell's sliced row -- for uniform slices the column offsets,
// values and neighbour activations of four slots are loaded before any is used -- and
// write the [h; m] row (64 BF16) into the warp's shared tile.  4 k-steps x 4 n-blocks of
// mma.sync give the 16 x 32 pre-activation; the epilogue adds the bias, applies the ReLU
// and the skip connection, puts h' back into the tile, and the tile leaves in 16-byte
// stores (16 consecutive cells = 1 KB contiguous).  Rows of the tile and of W_l are
// padded to 72 elements so that the fragment loads of the 8 row groups fall in distinct
// banks.
__global__ void __launch_bounds__(kTPB, 4)
    k_lp_layer(SellView s, int n, const float *__restrict__ aval,
               const __nv_bfloat16 *__restrict__ hin, __nv_bfloat16 *__restrict__ hout,
               const __nv_bfloat16 *__restrict__ wl, const float *__restrict__ bl,
               float *__restrict__ mout, float *__restrict__ zout, const int *done) {
  if (stopped(done)) return;
  constexpr int TS = lp::kTileStride;
  __shared__ __align__(16) __nv_bfloat16 wsm[C * TS];
  __shared__ float bsm[C];
  __shared__ __align__(16) __nv_bfloat16 tile[kTPB / 32][16 * TS];
  for (int t = threadIdx.x; t < C * 2 * C; t += blockDim.x)
    wsm[(t / (2 * C)) * TS + t % (2 * C)] = wl[t];
  if (threadIdx.x < C) bsm[threadIdx.x] = bl[threadIdx.x];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qc = 8 * (lane & 3);
  __nv_bfloat16 *tw = tile[warp];
  const int ntiles = (n + 15) / 16;
  const int nwarps = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  for (int tt = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5); tt < ntiles;
       tt += nwarps) {
#pragma unroll 1
    for (int rd = 0; rd < 2; ++rd) {
      const int rloc = rd * 8 + (lane >> 2);
      const int r = tt * 16 + rloc;
      float acc[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] = 0.f;
      uint4 own = make_uint4(0, 0, 0, 0);
      if (r < n) {
        const int slice = r >> 5, ln = r & 31;
        const long long base = __ldg(&s.ptr[slice]) + ln;
        const int w = __ldg(&s.width[slice]), op = __ldg(&s.offp[slice]);
        const __nv_bfloat16 *hq = hin + qc;
        if (__ldg(&s.kind[slice]) == 0 && w <= 8) {
#pragma unroll
          for (int j0 = 0; j0 < 8; j0 += 4) {
            float v[4];
            uint4 hv[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              if (j0 + j < w) {
                int col = r + __ldg(&s.off[op + j0 + j]);
                col = col < 0 ? 0 : (col >= n ? n - 1 : col);
                v[j] = __ldg(&aval[base + (long long)(j0 + j) * 32]);
                hv[j] = __ldg(reinterpret_cast<const uint4 *>(hq + (long long)col * C));
              }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
              if (j0 + j < w) fma8(acc, v[j], hv[j]);
          }
        } else {
          const bool uni = __ldg(&s.kind[slice]) == 0;
          for (int j = 0; j < w; ++j) {
            int col = uni ? r + __ldg(&s.off[op + j]) : __ldg(&s.off[op + 32 * j + ln]);
            col = col < 0 ? 0 : (col >= n ? n - 1 : col);
            fma8(acc, __ldg(&aval[base + (long long)j * 32]),
                 __ldg(reinterpret_cast<const uint4 *>(hq + (long long)col * C)));
          }
        }
        own = __ldg(reinterpret_cast<const uint4 *>(hq + (long long)r * C));
      }
      __align__(16) __nv_bfloat16 mb[8];
      lp::tile_put_row(tw, rloc, qc, own, acc, mb);
      if (mout && r < n) {
        float4 *mo = reinterpret_cast<float4 *>(mout + (long long)r * C + qc);
        mo[0] = make_float4(bf(mb[0]), bf(mb[1]), bf(mb[2]), bf(mb[3]));
        mo[1] = make_float4(bf(mb[4]), bf(mb[5]), bf(mb[6]), bf(mb[7]));
      }
    }
    __syncwarp();
    lp::tile_dense(tw, wsm, bsm, lane, [&](int rr, int col, float z0, float z1) {
      const int cell = tt * 16 + rr;
      if (zout && cell < n)
        *reinterpret_cast<float2 *>(zout + (long long)cell * C + col) = make_float2(z0, z1);
    });
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int idx = lane + 32 * k, rr = idx >> 2, part = idx & 3;
      const int cell = tt * 16 + rr;
      if (cell < n)
        *reinterpret_cast<uint4 *>(hout + (long long)cell * C + 8 * part) =
            *reinterpret_cast<const uint4 *>(tw + rr * TS + 8 * part);
    }
    __syncwarp();
  }
}

// The same layer as two streaming kernels (k_lp_agg, k_lp_dense), bit-identical to
// k_lp_layer: the aggregation writes m = Ahat h rounded to BF16, four threads per cell
// and eight channels per thread with all neighbour loads of a row in flight at full
// occupancy; the dense kernel streams the [h; m] rows of a 16-cell tile into the warp's
// shared tile and runs the same mma.sync product and epilogue.
__global__ void __launch_bounds__(kTPB)
    k_lp_agg(SellView s, int n, const float *__restrict__ aval,
             const __nv_bfloat16 *__restrict__ hin, __nv_bfloat16 *__restrict__ mout,
             const int *done) {
  if (stopped(done)) return;
  FCG_GRID_STRIDE(t, 4LL * n) {
    const int r = (int)(t >> 2), qc = 8 * (int)(t & 3);
    const int slice = r >> 5, ln = r & 31;
    const long long base = __ldg(&s.ptr[slice]) + ln;
    const int w = __ldg(&s.width[slice]), op = __ldg(&s.offp[slice]);
    const __nv_bfloat16 *hq = hin + qc;
    float acc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = 0.f;
    if (__ldg(&s.kind[slice]) == 0 && w <= 8) {
      float v[8];
      uint4 hv[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (j < w) {
          int col = r + __ldg(&s.off[op + j]);
          col = col < 0 ? 0 : (col >= n ? n - 1 : col);
          v[j] = __ldg(&aval[base + (long long)j * 32]);
          hv[j] = __ldg(reinterpret_cast<const uint4 *>(hq + (long long)col * C));
        }
      }
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (j < w) fma8(acc, v[j], hv[j]);
    } else {
      const bool uni = __ldg(&s.kind[slice]) == 0;
      for (int j = 0; j < w; ++j) {
        int col = uni ? r + __ldg(&s.off[op + j]) : __ldg(&s.off[op + 32 * j + ln]);
        col = col < 0 ? 0 : (col >= n ? n - 1 : col);
        fma8(acc, __ldg(&aval[base + (long long)j * 32]),
             __ldg(reinterpret_cast<const uint4 *>(hq + (long long)col * C)));
      }
    }
    __align__(16) __nv_bfloat16 mb[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) mb[c] = __float2bfloat16(acc[c]);
    *reinterpret_cast<uint4 *>(mout + (long long)r * C + qc) = *reinterpret_cast<const uint4 *>(mb);
  }
}

__global__ void __launch_bounds__(kTPB, 4)
    k_lp_dense(int n, const __nv_bfloat16 *__restrict__ hin,
               const __nv_bfloat16 *__restrict__ min_, __nv_bfloat16 *__restrict__ hout,
               const __nv_bfloat16 *__restrict__ wl, const float *__restrict__ bl,
               const int *done) {
  if (stopped(done)) return;
  constexpr int TS = lp::kTileStride;
  __shared__ __align__(16) __nv_bfloat16 wsm[C * TS];
  __shared__ float bsm[C];
  __shared__ __align__(16) __nv_bfloat16 tile[kTPB / 32][16 * TS];
  for (int t = threadIdx.x; t < C * 2 * C; t += blockDim.x)
    wsm[(t / (2 * C)) * TS + t % (2 * C)] = wl[t];
  if (threadIdx.x < C) bsm[threadIdx.x] = bl[threadIdx.x];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __nv_bfloat16 *tw = tile[warp];
  const int ntiles = (n + 15) / 16;
  const int nwarps = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  for (int tt = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5); tt < ntiles;
       tt += nwarps) {
    // 16 rows x (4 uint4 of h + 4 uint4 of m): 128 copies, 4 per lane
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int idx = lane + 32 * k, rr = idx >> 3, part = idx & 7;
      const int cell = tt * 16 + rr;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (cell < n) {
        const __nv_bfloat16 *src = part < 4 ? hin + (long long)cell * C + 8 * part
                                            : min_ + (long long)cell * C + 8 * (part - 4);
        v = __ldg(reinterpret_cast<const uint4 *>(src));
      }
      *reinterpret_cast<uint4 *>(tw + rr * TS + 8 * part) = v;
    }
    __syncwarp();
    lp::tile_dense(tw, wsm, bsm, lane, lp::NoZ());
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int idx = lane + 32 * k, rr = idx >> 2, part = idx & 3;
      const int cell = tt * 16 + rr;
      if (cell < n)
        *reinterpret_cast<uint4 *>(hout + (long long)cell * C + 8 * part) =
            *reinterpret_cast<const uint4 *>(tw + rr * TS + 8 * part);
    }
    __syncwarp();
  }
}

__device__ __forceinline__ float out_dot(const __nv_bfloat16 *__restrict__ h, long long i,
                                         const float *w) {
  const uint4 *hp = reinterpret_cast<const uint4 *>(h + i * C);
  uint4 v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = __ldg(hp + q);
  return lp::out_dot_vals(v, w);
}

// Output with the Jacobi skip: y = r/rms + w_out . h_L + b_out (the normalised output),
// z = r + rms (w_out . h_L + b_out).  With e given (training), d = y - e/rms.
__global__ void __launch_bounds__(kTPB)
    k_lp_out(int n, const __nv_bfloat16 *__restrict__ h, const float *__restrict__ prm,
             const float *__restrict__ rms, const float *__restrict__ r,
             const float *__restrict__ e, float *__restrict__ y, float *__restrict__ d,
             float *__restrict__ z) {
  __shared__ float w[C + 1];
  if (threadIdx.x <= C) w[threadIdx.x] = prm[lp::oWout + threadIdx.x];
  __syncthreads();
  const float sc = rms[0], inv = 1.0f / sc;
  FCG_GRID_STRIDE(i, n) {
    const float acc = out_dot(h, i, w);
    const float yi = r[i] * inv + acc;
    if (y) y[i] = yi;
    if (d) d[i] = yi - e[i] * inv;
    if (z) z[i] = r[i] + sc * acc;
  }
}

// ---------------------------------------------------------------------------
// Loss, backward, Adam
// ---------------------------------------------------------------------------
// Loss of the normalised output, d = y - e/rms, t = e/rms (Ahat d = Ahat y - r/rms):
//   kind 0 (energy norm):   loss = d.Ahat d / t.Ahat t,         d loss/dy = 2 Ahat d / t.Ahat t
//   kind 1 (residual norm): loss = |Ahat d|^2 / |Ahat t|^2,      d loss/dy = 2 Ahat Ahat d / |Ahat t|^2
// sums[0], sums[1] = numerator, denominator; ad = Ahat d.
__global__ void __launch_bounds__(kTPB, 6)
    k_lp_aloss(SellView s, int n, const float *__restrict__ val, const float *__restrict__ d,
               const float *__restrict__ e, const float *__restrict__ rms,
               float *__restrict__ ad, double *partials, unsigned *ticket,
               float *__restrict__ sums, int kind) {
  const float inv = 1.0f / rms[0];
  float a = 0.f, b = 0.f;
  FCG_SLICE_LOOP(slice, lane, s) {
    const float adv = sell_row(s, n, val, d, slice, lane);
    const float atv = sell_row(s, n, val, e, slice, lane) * inv;
    const int row = slice * 32 + lane;
    if (row < n) {
      ad[row] = adv;
      if (kind == 0) {
        a += d[row] * adv;
        b += (e[row] * inv) * atv;
      } else {
        a += adv * adv;
        b += atv * atv;
      }
    }
  }
  double v[2] = {(double)a, (double)b};
  if (reduce_commit<2>(v, partials, ticket) && threadIdx.x == 0) {
    sums[0] = (float)v[0];
    sums[1] = (float)v[1];
  }
}

// y = Ahat x in FP32 (the second product of the residual-norm loss)
__global__ void __launch_bounds__(kTPB, 6)
    k_lp_spmv32(SellView s, int n, const float *__restrict__ val, const float *__restrict__ x,
                float *__restrict__ y) {
  FCG_SLICE_LOOP(slice, lane, s) {
    const float v = sell_row(s, n, val, x, slice, lane);
    const int row = slice * 32 + lane;
    if (row < n) y[row] = v;
  }
}

// d = y_c - e/rms (the cycle loss's output error)
__global__ void __launch_bounds__(kTPB)
    k_lp_cycle_d(int n, const float *__restrict__ yc, const float *__restrict__ e,
                 const float *__restrict__ rms, float *__restrict__ d) {
  const float inv = 1.0f / rms[0];
  FCG_GRID_STRIDE(i, n) d[i] = yc[i] - e[i] * inv;
}

// g = u - g (the cycle loss's gradient, in place)
__global__ void __launch_bounds__(kTPB)
    k_lp_cycle_g(int n, const float *__restrict__ u, float *__restrict__ g) {
  FCG_GRID_STRIDE(i, n) g[i] = u[i] - g[i];
}

// dy = 2 g / sums[1] (g = Ahat d or Ahat Ahat d); dh_L = dy w_out; per-block sums of
// dy h_L and dy.
__global__ void __launch_bounds__(kTPB)
    k_lp_out_bwd(int n, const float *__restrict__ ad, const float *__restrict__ sums,
                 const __nv_bfloat16 *__restrict__ h, const float *__restrict__ prm,
                 float *__restrict__ dh, float *__restrict__ part /* [G][C+1] */) {
  __shared__ float acc[kTPB / 32][C + 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float k2 = 2.0f / fmaxf(sums[1], 1e-30f);
  const float wl = prm[lp::oWout + lane];
  float gw = 0.f, gb = 0.f;
  for (long long i = (long long)blockIdx.x * (kTPB / 32) + warp; i < n;
       i += (long long)gridDim.x * (kTPB / 32)) {
    const float dy = k2 * ad[i];
    dh[i * C + lane] = dy * wl;
    gw += dy * bf(h[i * C + lane]);
    gb += dy;
  }
  acc[warp][lane] = gw;
  if (lane == 0) acc[warp][C] = gb;
  __syncthreads();
  if (threadIdx.x <= C) {
    float sacc = 0.f;
    for (int w = 0; w < kTPB / 32; ++w) sacc += acc[w][threadIdx.x];
    part[(long long)blockIdx.x * (C + 1) + threadIdx.x] = sacc;
  }
}

// Layer backward, per cell (FP32): dz = dh * [z > 0]; [dh_x; dm] = W_l^T dz;
// dh_prev = dh + dh_x (skip connection), dm kept for the aggregation.  Per-block sums of
// dz [h; m]^T and dz give the gradient of W_l and b_l.  Block b owns a contiguous run of
// cells, staged 64 at a time in shared memory.
__global__ void __launch_bounds__(kTPB, 2)
    k_lp_layer_bwd(int n, const float *__restrict__ dh, const float *__restrict__ z,
                   const __nv_bfloat16 *__restrict__ hin, const float *__restrict__ m,
                   const float *__restrict__ prm_l, float *__restrict__ dh_prev,
                   float *__restrict__ dm, float *__restrict__ part /* [G][kLayerParams] */) {
  __shared__ float W[C * 2 * C];
  __shared__ float dzs[lp::kBwdTile][C + 1];
  __shared__ float xs[lp::kBwdTile][2 * C];
  for (int t = threadIdx.x; t < C * 2 * C; t += blockDim.x) W[t] = prm_l[t];
  float gw[8], gbias = 0.f;  // thread t: weights t + 256 q, bias t (t < 32)
#pragma unroll
  for (int q = 0; q < 8; ++q) gw[q] = 0.f;
  __syncthreads();
  const long long per = ((long long)n + gridDim.x - 1) / gridDim.x;
  const long long c0 = (long long)blockIdx.x * per, c1 = min((long long)n, c0 + per);
  for (long long base = c0; base < c1; base += lp::kBwdTile) {
    const int cnt = (int)min((long long)lp::kBwdTile, c1 - base);
    for (int t = threadIdx.x; t < cnt * C; t += blockDim.x) {
      const int cl = t / C, ch = t % C;
      const long long o = (base + cl) * C + ch;
      dzs[cl][ch] = z[o] > 0.f ? dh[o] : 0.f;
      xs[cl][ch] = bf(hin[o]);
      xs[cl][C + ch] = m[o];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < cnt * C; t += blockDim.x) {
      const int cl = t / C, k = t % C;
      float gh = 0.f, gm = 0.f;
#pragma unroll 8
      for (int o = 0; o < C; ++o) {
        const float dz = dzs[cl][o];
        gh += W[o * 2 * C + k] * dz;
        gm += W[o * 2 * C + C + k] * dz;
      }
      const long long oo = (base + cl) * C + k;
      dh_prev[oo] = dh[oo] + gh;
      dm[oo] = gm;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int idx = threadIdx.x + q * kTPB;
      const int o = idx / (2 * C), k = idx % (2 * C);
      float sacc = 0.f;
      for (int cl = 0; cl < cnt; ++cl) sacc += dzs[cl][o] * xs[cl][k];
      gw[q] += sacc;
    }
    if (threadIdx.x < C)
      for (int cl = 0; cl < cnt; ++cl) gbias += dzs[cl][threadIdx.x];
    __syncthreads();
  }
  float *pb = part + (long long)blockIdx.x * lp::kLayerParams;
#pragma unroll
  for (int q = 0; q < 8; ++q) pb[threadIdx.x + q * kTPB] = gw[q];
  if (threadIdx.x < C) pb[2 * C * C + threadIdx.x] = gbias;
}

// dh_prev += Ahat dm (Ahat of the pressure system is symmetric); a warp per cell, a
// lane per channel.
__global__ void __launch_bounds__(kTPB)
    k_lp_agg_bwd(SellView s, int n, const float *__restrict__ aval,
                 const float *__restrict__ dm, float *__restrict__ dh_prev) {
  const int lane = threadIdx.x & 31;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((long long)gridDim.x * blockDim.x) >> 5) {
    const int slice = (int)(r >> 5), ln = (int)(r & 31);
    const long long base = __ldg(&s.ptr[slice]) + ln;
    const int w = __ldg(&s.width[slice]), op = __ldg(&s.offp[slice]);
    const bool uni = __ldg(&s.kind[slice]) == 0;
    float acc = 0.f;
    for (int j = 0; j < w; ++j) {
      long long col = uni ? r + __ldg(&s.off[op + j]) : __ldg(&s.off[op + 32 * j + ln]);
      col = col < 0 ? 0 : (col >= n ? n - 1 : col);
      acc += __ldg(&aval[base + (long long)j * 32]) * dm[col * C + lane];
    }
    dh_prev[r * C + lane] += acc;
  }
}

// Embedding backward: dz0 = dh0 * [z0 > 0]; per-block sums of dz0 f^T and dz0.
__global__ void __launch_bounds__(kTPB)
    k_lp_embed_bwd(int n, const float *__restrict__ dh, const float *__restrict__ z0,
                   const float *__restrict__ feat, float *__restrict__ part /* [G][C*F+C] */) {
  __shared__ float acc[kTPB / 32][C * F + C];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;  // lane = output channel
  float g[F + 1];
#pragma unroll
  for (int k = 0; k <= F; ++k) g[k] = 0.f;
  for (long long i = (long long)blockIdx.x * (kTPB / 32) + warp; i < n;
       i += (long long)gridDim.x * (kTPB / 32)) {
    const long long o = i * C + lane;
    const float dz = z0[o] > 0.f ? dh[o] : 0.f;
#pragma unroll
    for (int k = 0; k < F; ++k) g[k] += dz * feat[k * (long long)n + i];
    g[F] += dz;
  }
#pragma unroll
  for (int k = 0; k < F; ++k) acc[warp][lane * F + k] = g[k];
  acc[warp][C * F + lane] = g[F];
  __syncthreads();
  for (int t = threadIdx.x; t < C * F + C; t += blockDim.x) {
    float sacc = 0.f;
    for (int w = 0; w < kTPB / 32; ++w) sacc += acc[w][t];
    part[(long long)blockIdx.x * (C * F + C) + t] = sacc;
  }
}

// grad[t] = sum over blocks, in block order, of part[b][t]
__global__ void k_lp_sum_parts(const float *__restrict__ part, int nblocks, int width,
                               float *__restrict__ grad) {
  FCG_GRID_STRIDE(t, width) {
    double sacc = 0.0;
    for (int b = 0; b < nblocks; ++b) sacc += part[(long long)b * width + t];
    grad[t] = (float)sacc;
  }
}

// Adam (Kingma & Ba, ICLR 2015) with bias correction.
__global__ void k_lp_adam(float *__restrict__ prm, float *__restrict__ m, float *__restrict__ v,
                          const float *__restrict__ g, float lr, float c1, float c2) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  FCG_GRID_STRIDE(i, P) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    prm[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_lp_to_bf16(const float *__restrict__ prm, __nv_bfloat16 *__restrict__ wbf) {
  FCG_GRID_STRIDE(t, (long long)L * 2 * C * C) {
    const int l = (int)(t / (2 * C * C)), k = (int)(t % (2 * C * C));
    wbf[t] = __float2bfloat16(prm[lp::oLayer0 + l * lp::kLayerParams + k]);
  }
}

// ---------------------------------------------------------------------------
// Flexible CG kernels (scaled system in FP32, reliable updates in FP64)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool fdone(const LScal *S) { return __ldcg(&S->done) != 0; }

// res = su - A x (FP64), res0 = sum |res|, r = D^-1/2 res (FP32), y = 0
__global__ void __launch_bounds__(kTPB, 8)
    k_f_init(SellView s, int n, const double *__restrict__ val, const double *__restrict__ su,
             const double *__restrict__ x, double *__restrict__ res,
             const double *__restrict__ s64, float *__restrict__ r32, float *__restrict__ y32,
             LScal *S, double *partials) {
  double l1 = 0.0;
  float t = 0.f;
  FCG_SLICE_LOOP(slice, lane, s) {
    const int r = slice * 32 + lane;
    const double ax = sell_row(s, n, val, x, slice, lane);
    if (r < n) {
      const double rr = su[r] - ax;
      res[r] = rr;
      l1 += fabs(rr);
      const float r3 = (float)(s64[r] * rr);
      r32[r] = r3;
      y32[r] = 0.f;
      t += r3 * r3;
    }
  }
  double v[2] = {l1, (double)t};
  if (reduce_commit<2>(v, partials, &S->ticket[0]) && threadIdx.x == 0) {
    S->res0 = v[0];
    S->resl = v[0];
    S->rr = v[1];
    S->maxr = sqrt(v[1]);
    S->l1ratio = v[1] > 0 ? v[0] / sqrt(v[1]) : 0.0;
    S->chk_l1 = v[0];
    S->nwin = 0;
    S->head = 0;
    if (!isfinite(v[0])) S->status = FCG_ERR_NONFINITE;
    if (S->nsw <= 0 || v[0] == 0.0 || S->status) S->done = 1;
    if (v[0] == 0.0) S->converged = 1;
  }
}

// z = r + rms (w_out . h_L + b_out) and z . q_j for the stored directions j, which give
// beta_j = z . q_j / p_j . q_j (truncated flexible CG, Notay 2000, eq. 2.7)
__global__ void __launch_bounds__(kTPB, 4)
    k_f_out(int n, const __nv_bfloat16 *__restrict__ h, const float *__restrict__ prm,
            const float *__restrict__ rms, const float *__restrict__ r, float *__restrict__ z,
            const float *__restrict__ qring, long long stride, LScal *S, double *partials,
            int dots) {
  if (fdone(S)) return;
  __shared__ float w[C + 1];
  if (threadIdx.x <= C) w[threadIdx.x] = prm[lp::oWout + threadIdx.x];
  __syncthreads();
  const float sc = rms[0];
  if (!dots) {  // z only: a coarse-grid correction follows, then k_f_zdots
    FCG_GRID_STRIDE(i, n) z[i] = r[i] + sc * out_dot(h, i, w);
    return;
  }
  const int nwin = __ldcg(&S->nwin);
  float t[lp::kMaxDir];
#pragma unroll
  for (int j = 0; j < lp::kMaxDir; ++j) t[j] = 0.f;
  FCG_GRID_STRIDE(i, n) {
    const float zi = r[i] + sc * out_dot(h, i, w);
    z[i] = zi;
#pragma unroll
    for (int j = 0; j < lp::kMaxDir; ++j)
      if (j < nwin) t[j] += zi * qring[j * stride + i];
  }
  double v[lp::kMaxDir];
#pragma unroll
  for (int j = 0; j < lp::kMaxDir; ++j) v[j] = (double)t[j];
  if (reduce_commit<lp::kMaxDir>(v, partials, &S->ticket[1]) && threadIdx.x == 0) {
    for (int j = 0; j < lp::kMaxDir; ++j) {
      S->bets[j] = j < nwin ? v[j] / S->pqs[j] : 0.0;
      if (!isfinite(S->bets[j])) {
        S->status = FCG_ERR_NONFINITE;
        S->done = 1;
      }
    }
  }
}

// beta_j = z . q_j / p_j . q_j of the stored directions (after a coarse-grid correction)
__global__ void __launch_bounds__(kTPB, 4)
    k_f_zdots(int n, const float *__restrict__ z, const float *__restrict__ qring,
              long long stride, LScal *S, double *partials) {
  if (fdone(S)) return;
  const int nwin = __ldcg(&S->nwin);
  float t[lp::kMaxDir];
#pragma unroll
  for (int j = 0; j < lp::kMaxDir; ++j) t[j] = 0.f;
  FCG_GRID_STRIDE(i, n) {
    const float zi = z[i];
#pragma unroll
    for (int j = 0; j < lp::kMaxDir; ++j)
      if (j < nwin) t[j] += zi * qring[j * stride + i];
  }
  double v[lp::kMaxDir];
#pragma unroll
  for (int j = 0; j < lp::kMaxDir; ++j) v[j] = (double)t[j];
  if (reduce_commit<lp::kMaxDir>(v, partials, &S->ticket[1]) && threadIdx.x == 0) {
    for (int j = 0; j < lp::kMaxDir; ++j) {
      S->bets[j] = j < nwin ? v[j] / S->pqs[j] : 0.0;
      if (!isfinite(S->bets[j])) {
        S->status = FCG_ERR_NONFINITE;
        S->done = 1;
      }
    }
  }
}

// p_head = z - sum_j beta_j p_j (the slot written may be the oldest one read: each
// element reads all slots before it is written)
__global__ void __launch_bounds__(kTPB, 8)
    k_f_p(int n, const float *__restrict__ z, float *__restrict__ pring, long long stride,
          const LScal *S) {
  if (fdone(S)) return;
  const int nwin = __ldcg(&S->nwin), head = __ldcg(&S->head);
  float b[lp::kMaxDir];
#pragma unroll
  for (int j = 0; j < lp::kMaxDir; ++j) b[j] = (float)__ldcg(&S->bets[j]);
  float *ph = pring + head * stride;
  FCG_GRID_STRIDE(i, n) {
    float acc = z[i];
#pragma unroll
    for (int j = 0; j < lp::kMaxDir; ++j)
      if (j < nwin) acc -= b[j] * pring[j * stride + i];
    ph[i] = acc;
  }
}

// q_head = Ahat p_head; alpha = p.r / p.q; the new direction joins the window
__global__ void __launch_bounds__(kTPB, 6)
    k_f_spmv(SellView s, int n, const float *__restrict__ val, const float *__restrict__ pring,
             float *__restrict__ qring, long long stride, const float *__restrict__ r, LScal *S,
             double *partials) {
  if (fdone(S)) return;
  const int head = __ldcg(&S->head);
  const float *p = pring + head * stride;
  float *q = qring + head * stride;
  float tq = 0.f, tr = 0.f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int per = (s.nslices + gridDim.x - 1) / gridDim.x;
  const int sbeg = blockIdx.x * per, send = min(s.nslices, sbeg + per);
  for (int slice = sbeg + warp; slice < send; slice += kTPB / 32) {
    const float qv = sell_row(s, n, val, p, slice, lane);
    const int row = slice * 32 + lane;
    if (row < n) {
      q[row] = qv;
      const float pv = p[row];
      tq += pv * qv;
      tr += pv * r[row];
    }
  }
  double v[2] = {(double)tq, (double)tr};
  if (reduce_commit<2>(v, partials, &S->ticket[2]) && threadIdx.x == 0) {
    S->pqs[head] = v[0];
    S->alf = v[1] / v[0];
    S->head = (head + 1) % S->mdir;
    S->nwin = min(S->nwin + 1, S->mdir);
    if (!isfinite(S->alf) || !(v[0] > 0.0)) {
      S->status = FCG_ERR_NONFINITE;
      S->done = 1;
    }
  }
}

__device__ __noinline__ void f_decide(LScal *S, double rrn) {
  const int it = S->iter + 1;
  S->iter = it;
  const double nr = sqrt(rrn);
  const double pred = S->l1ratio * nr;
  const bool ru = nr < S->delta * S->maxr || pred < 0.9 * S->resmax * (S->res0 + S->small) ||
                  it - S->last_ru >= S->ru_every || it >= S->nsw || !isfinite(rrn);
  S->rr = rrn;
  S->ru = ru ? 1 : 0;
}

// y += alpha p, r -= alpha q (the direction just added); ||r||^2 decides on a reliable
// update (arms the IF node)
__global__ void __launch_bounds__(kTPB, 8)
    k_f_update(int n, float *__restrict__ y, float *__restrict__ r,
               const float *__restrict__ pring, const float *__restrict__ qring,
               long long stride, LScal *S, double *partials, cudaGraphConditionalHandle hif,
               int use_cond) {
  if (fdone(S)) {
    if (use_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(hif, 0u);
    return;
  }
  const int m = __ldcg(&S->mdir), slot = (__ldcg(&S->head) + m - 1) % m;
  const float *p = pring + slot * stride, *q = qring + slot * stride;
  const float alf = (float)__ldcg(&S->alf);
  float t = 0.f;
  FCG_GRID_STRIDE(i, n) {
    y[i] = y[i] + alf * p[i];
    const float rv = r[i] - alf * q[i];
    r[i] = rv;
    t += rv * rv;
  }
  double v[1] = {(double)t};
  if (reduce_commit<1>(v, partials, &S->ticket[3]) && threadIdx.x == 0) {
    f_decide(S, v[0]);
    if (use_cond) cudaGraphSetConditional(hif, S->ru ? 1u : 0u);
  }
}

// reliable update, part 1: x += D^-1/2 y (FP64), y = 0
__global__ void __launch_bounds__(kTPB, 8)
    k_f_ru1(int n, double *__restrict__ x, float *__restrict__ y, const double *__restrict__ s64,
            const LScal *S) {
  if (fdone(S) || !__ldcg(&S->ru)) return;
  FCG_GRID_STRIDE(i, n) {
    x[i] = x[i] + s64[i] * (double)y[i];
    y[i] = 0.f;
  }
}

__device__ __noinline__ void f_after_update(LScal *S, double l1, double rrn) {
  S->resl = l1;
  S->nupdates++;
  S->last_ru = S->iter;
  const double rsm = l1 / (S->res0 + S->small);
  if (rsm < S->resmax) S->converged = 1;
  if (!isfinite(l1) || !isfinite(rrn)) S->status = FCG_ERR_NONFINITE;
  if (l1 <= S->stall_factor * S->chk_l1) {
    S->chk_l1 = l1;
    S->chk_iter = S->iter;
  } else if (S->iter - S->chk_iter >= S->stall_window) {
    S->status = FCG_ERR_STALL;
  }
  if (S->converged || S->iter >= S->nsw || S->status) {
    S->done = 1;
    return;
  }
  S->rr = rrn;
  S->maxr = sqrt(rrn);
  S->l1ratio = rrn > 0 ? l1 / sqrt(rrn) : 0.0;
  S->ru = 0;
}

// reliable update, part 2: res = su - A x (FP64), its L1, r = D^-1/2 res
__global__ void __launch_bounds__(kTPB, 8)
    k_f_ru2(SellView s, int n, const double *__restrict__ val, const double *__restrict__ su,
            const double *__restrict__ x, double *__restrict__ res,
            const double *__restrict__ s64, float *__restrict__ r32, LScal *S,
            double *partials) {
  if (fdone(S) || !__ldcg(&S->ru)) return;
  double l1 = 0.0;
  float t = 0.f;
  FCG_SLICE_LOOP(slice, lane, s) {
    const int r = slice * 32 + lane;
    const double ax = sell_row(s, n, val, x, slice, lane);
    if (r < n) {
      const double rr = su[r] - ax;
      res[r] = rr;
      l1 += fabs(rr);
      const float r3 = (float)(s64[r] * rr);
      r32[r] = r3;
      t += r3 * r3;
    }
  }
  double v[2] = {l1, (double)t};
  if (reduce_commit<2>(v, partials, &S->ticket[4]) && threadIdx.x == 0)
    f_after_update(S, v[0], v[1]);
}

// closes the loop body: bound on the number of bodies, stop when done
__global__ void k_f_close(LScal *S, cudaGraphConditionalHandle h, int use_cond) {
  if (threadIdx.x != 0) return;
  const unsigned c = atomicAdd(&S->body_count, 1u) + 1u;
  if (c > (unsigned)S->nsw + 2u && !S->done) {
    S->status = FCG_ERR_TIMEOUT;
    S->done = 1;
  }
  if (use_cond && S->done) cudaGraphSetConditional(h, 0u);
}

// ||su - A x||^2 and ||su||^2 in FP64
__global__ void __launch_bounds__(kTPB, 8)
    k_f_final(SellView s, int n, const double *__restrict__ val, const double *__restrict__ su,
              const double *__restrict__ x, LScal *S, double *partials) {
  double v[2] = {0.0, 0.0};
  FCG_SLICE_LOOP(slice, lane, s) {
    const int r = slice * 32 + lane;
    const double ax = sell_row(s, n, val, x, slice, lane);
    if (r < n) {
      const double rr = su[r] - ax;
      v[0] += rr * rr;
      v[1] += su[r] * su[r];
    }
  }
  if (reduce_commit<2>(v, partials, &S->ticket[5]) && threadIdx.x == 0) {
    S->l2r = v[0];
    S->l2b = v[1];
  }
}

}  // namespace
}  // namespace fcg

using namespace fcg;

namespace {

constexpr int kMaxBlocks = 1024;  // upper bound of the blocks of any reduction grid here

// Deterministic initialisation: U(-1, 1)/sqrt(fan_in) from a counter hash of the seed;
// the residual layers start at a tenth of that scale, the output layer at zero.
std::vector<float> init_params(unsigned long long seed) {
  std::vector<float> p(lp::P, 0.f);
  auto u = [&](long long i) {
    unsigned long long z =
        seed * 0x9E3779B97F4A7C15ULL + (unsigned long long)i * 0xD1B54A32D192ED03ULL;
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ULL;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  for (int t = 0; t < lp::C * lp::F; ++t)
    p[lp::oWin + t] = (float)(u(t) / std::sqrt((double)lp::F));
  for (int l = 0; l < lp::L; ++l)
    for (int t = 0; t < 2 * lp::C * lp::C; ++t)
      p[lp::oLayer0 + l * lp::kLayerParams + t] =
          (float)(0.1 * u(1000 + l * 4096 + t) / std::sqrt(2.0 * lp::C));
  // w_out and b_out start at 0: the untrained network is the Jacobi preconditioner
  return p;
}

int lp_fail(fcg_learned *Lp, int status, const std::string &msg) {
  if (Lp) Lp->err = msg;
  return status;
}

int lp_cuda(fcg_learned *Lp, cudaError_t e, const char *where) {
  return lp_fail(Lp, FCG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define LP_TRY(Lp, expr)                                    \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) return lp_cuda((Lp), _e, #expr); \
  } while (0)

int reduction_grid(const fcg_context *c) { return std::min(kMaxBlocks, c->num_sms * 4); }

// Workspaces for meshes of up to n cells (training adds the saved tensors).
int ensure_workspace(fcg_learned *Lp, fcg_context *c, bool train) {
  const size_t n = (size_t)c->n;
  if (n > Lp->ncap) {
    Lp->ncap = n;
    Lp->train_cap = false;
    LP_TRY(Lp, Lp->feat.ensure(sizeof(float) * n * lp::F));
    LP_TRY(Lp, Lp->y.ensure(sizeof(float) * n));
    LP_TRY(Lp, Lp->hbuf.ensure(sizeof(__nv_bfloat16) * 3 * n * lp::C));  // h ping-pong + m
    Lp->fuid = 0;  // features must be recomputed into the new buffer
  }
  if (train && !Lp->train_cap) {
    const size_t nc = Lp->ncap * lp::C;
    LP_TRY(Lp, Lp->hbuf.ensure(sizeof(__nv_bfloat16) * (lp::L + 1) * nc));
    LP_TRY(Lp, Lp->mbuf.ensure(sizeof(float) * lp::L * nc));
    LP_TRY(Lp, Lp->zbuf.ensure(sizeof(float) * (lp::L + 1) * nc));
    LP_TRY(Lp, Lp->dh.ensure(sizeof(float) * nc));
    LP_TRY(Lp, Lp->dh2.ensure(sizeof(float) * nc));
    LP_TRY(Lp, Lp->dm.ensure(sizeof(float) * nc));
    LP_TRY(Lp, Lp->dvec.ensure(sizeof(float) * 6 * Lp->ncap));
    Lp->train_cap = true;
  }
  return FCG_OK;
}

// Waits for the work the handle queued last (on any context's stream).
int wait_last(fcg_learned *Lp) {
  if (Lp->ev_pending) LP_TRY(Lp, cudaEventSynchronize(Lp->ev_last));
  Lp->ev_pending = false;
  return FCG_OK;
}

// Orders this call after work the handle queued on another context's stream.
int switch_stream(fcg_learned *Lp, fcg_context *c) {
  if (Lp->last_uid != c->uid) {
    int rc = wait_last(Lp);
    if (rc) return rc;
  }
  Lp->last_uid = c->uid;
  return FCG_OK;
}

int mark_done(fcg_learned *Lp, fcg_context *c) {
  LP_TRY(Lp, cudaEventRecord(Lp->ev_last, c->stream));
  Lp->ev_pending = true;
  return FCG_OK;
}

int check_ctx(fcg_learned *Lp, fcg_context *c) {
  if (!Lp || !c) return FCG_ERR_ARG;
  if (!c->bound) return lp_fail(Lp, FCG_ERR_STATE, "context has no mesh (fcg_bind_mesh)");
  if (c->mv.noc)
    return lp_fail(Lp, FCG_ERR_UNSUPPORTED,
                   "the learned preconditioner does not take O-C grid cuts (noc > 0)");
  if (c->device != Lp->device)
    return lp_fail(Lp, FCG_ERR_ARG, "context and learned preconditioner on different devices");
  LP_TRY(Lp, cudaSetDevice(c->device));
  return switch_stream(Lp, c);
}

bool features_current(const fcg_learned *Lp, const fcg_context *c) {
  return Lp->fuid == c->uid && Lp->fgen == c->bind_gen && Lp->fmat == (const void *)scaled32(c) &&
         scaled32(c) != nullptr;
}

// Device int of the scal buffer that a plane-staged layer outside a solve reports a wait
// timeout to.
constexpr int kHexStatus = 41;

// The plane-staged layer serves inference on lexicographic hex meshes; FCG_LP_LAYER=gather
// (or =split) keeps the sliced gather form everywhere.
bool hex_allowed() {
  const char *e = std::getenv("FCG_LP_LAYER");
  return !(e && (std::strcmp(e, "gather") == 0 || std::strcmp(e, "split") == 0));
}

bool hex_on(const fcg_learned *Lp, const fcg_context *c) {
  return Lp->hex.ok && Lp->hex_uid == c->uid && Lp->hex_gen == c->bind_gen && hex_allowed();
}

// Detects the block structure of c's mesh once per bound mesh, then writes the stencil
// value planes of the scaled matrix loaded last.
int hex_prepare(fcg_learned *Lp, fcg_context *c) {
  if (Lp->hex_uid != c->uid || Lp->hex_gen != c->bind_gen) {
    fcg::lphex::HexGrid g;
    int rc = fcg::lphex::detect(c, &g);
    if (rc) return lp_fail(Lp, rc, fcg_last_error(c));
    if (g.ok) {
      const size_t bytes = sizeof(float) * fcg::lphex::value_count(g);
      LP_TRY(Lp, Lp->hexval.ensure(bytes));
      LP_TRY(Lp, cudaMemsetAsync(Lp->hexval.p, 0, bytes, c->stream));  // padding columns
    }
    Lp->hex = g;
    Lp->hex_uid = c->uid;
    Lp->hex_gen = c->bind_gen;
  }
  if (Lp->hex.ok)
    LP_TRY(Lp, fcg::lphex::values(c, Lp->hex, scaled32(c), Lp->hexval.as<float>(), c->stream));
  return FCG_OK;
}

// Reads and clears the timeout status of the plane-staged layer (calls outside a solve).
int hex_status(fcg_learned *Lp, fcg_context *c) {
  int st = 0;
  LP_TRY(Lp, cudaMemcpyAsync(&st, Lp->scal.as<int>() + kHexStatus, sizeof st,
                             cudaMemcpyDeviceToHost, c->stream));
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  if (st == 0) return FCG_OK;
  LP_TRY(Lp, cudaMemsetAsync(Lp->scal.as<int>() + kHexStatus, 0, sizeof(int), c->stream));
  return lp_fail(Lp, st, "plane-staged layer: a copy wait gave up");
}

// Features of the context's mesh and of the scaled matrix loaded into it.
int compute_features(fcg_learned *Lp, fcg_context *c) {
  int rc = ensure_workspace(Lp, c, false);
  if (rc) return rc;
  const int G = reduction_grid(c);
  double *red = Lp->red.as<double>();
  k_lp_volsum<<<G, kTPB, 0, c->stream>>>(c->n, c->mv.vol, red, Lp->scal.as<unsigned>() + 16,
                                         red + lp::kMaxDir * kMaxBlocks);
  k_lp_features<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(
      c->mv, scale64(c), red + lp::kMaxDir * kMaxBlocks, Lp->feat.as<float>());
  LP_TRY(Lp, cudaGetLastError());
  if ((rc = hex_prepare(Lp, c))) return rc;
  Lp->fuid = c->uid;
  Lp->fgen = c->bind_gen;
  Lp->fmat = scaled32(c);
  return FCG_OK;
}

// Inference runs each layer as the one-kernel form k_lp_layer; FCG_LP_LAYER=split selects
// k_lp_agg + k_lp_dense (same bits; measured 2.0 ms against 1.44 ms per layer at 256^3).
bool layer_split() {
  const char *e = std::getenv("FCG_LP_LAYER");
  return e && std::strcmp(e, "split") == 0;
}

// Forward pass on r (device, FP32) up to h_L.  Training keeps h_0..h_L, m_1..m_L and the
// pre-activations; inference ping-pongs two activation buffers.  `done` (device flag or
// NULL) turns the launches into no-ops; `status` (device int or NULL) receives a wait
// timeout of the plane-staged layer.  Inference on a lexicographic hex mesh runs that
// layer (learned_hex.cu, the same bits as k_lp_layer).
// The forward pass of the network on r.  With `out` given (inference), the plane-staged
// form writes the output z of lphex::OutFuse from its last layer and sets *fused; the
// caller runs the output kernel itself when *fused stays false.
void enqueue_forward(fcg_learned *Lp, fcg_context *c, cudaStream_t st, const float *r, bool train,
                     const int *done, unsigned *rms_ticket, int *status,
                     const fcg::lphex::OutFuse *out = nullptr, bool *fused = nullptr) {
  if (fused) *fused = false;
  const int n = c->n;
  float *rms = Lp->scal.as<float>();
  const float *prm = Lp->params.as<float>();
  __nv_bfloat16 *H = Lp->hbuf.as<__nv_bfloat16>();
  const size_t hs = (size_t)n * lp::C;
  k_lp_rms<<<reduction_grid(c), kTPB, 0, st>>>(n, r, Lp->red.as<double>(), rms_ticket, rms, done);
  k_lp_embed<<<grid_for(n, c->num_sms, 8), kTPB, 0, st>>>(
      n, r, rms, Lp->feat.as<float>(), prm, H, train ? Lp->zbuf.as<float>() : nullptr, done);
  const float *aval = scaled32(c);
  const __nv_bfloat16 *wbf = Lp->wbf.as<__nv_bfloat16>();
  const int ntiles = (n + 15) / 16;
  const int lg = std::max(1, std::min((ntiles + 7) / 8, c->num_sms * 4));
  const bool split = !train && layer_split();
  for (int l = 0; l < lp::L; ++l) {
    const __nv_bfloat16 *hin = train ? H + l * hs : H + (l % 2) * hs;
    __nv_bfloat16 *hout = train ? H + (l + 1) * hs : H + ((l + 1) % 2) * hs;
    const __nv_bfloat16 *wl = wbf + (size_t)l * 2 * lp::C * lp::C;
    const float *bl = prm + lp::oLayer0 + l * lp::kLayerParams + 2 * lp::C * lp::C;
    if (split) {
      k_lp_agg<<<grid_for(4LL * n, c->num_sms, 8), kTPB, 0, st>>>(c->sv, n, aval, hin, H + 2 * hs,
                                                                 done);
      k_lp_dense<<<lg, kTPB, 0, st>>>(n, hin, H + 2 * hs, hout, wl, bl, done);
    } else if (!train && hex_on(Lp, c) &&
               fcg::lphex::layer(Lp->hex, c->num_sms, hin, hout, Lp->hexval.as<float>(), wl, bl,
                                 done, status, st, l + 1 == lp::L ? out : nullptr,
                                 l + 1 == lp::L ? fused : nullptr) == cudaSuccess) {
      // plane-staged form launched
    } else {
      k_lp_layer<<<lg, kTPB, 0, st>>>(c->sv, n, aval, hin, hout, wl, bl,
                                      train ? Lp->mbuf.as<float>() + l * hs : nullptr,
                                      train ? Lp->zbuf.as<float>() + (l + 1) * hs : nullptr, done);
    }
  }
}

const __nv_bfloat16 *last_activation(fcg_learned *Lp, fcg_context *c, bool train) {
  const size_t hs = (size_t)c->n * lp::C;
  __nv_bfloat16 *H = Lp->hbuf.as<__nv_bfloat16>();
  return train ? H + (size_t)lp::L * hs : H + (lp::L % 2) * hs;
}

// Hierarchies of the coarse-grid correction, one per context (the handle may train on
// several), at most kMlCache (16), least recently used first.
constexpr size_t kMlCache = 16;

fcg::ml::Hierarchy *ml_for(const fcg_learned *Lp, const fcg_context *c) {
  for (fcg::ml::Hierarchy *h : Lp->mlc)
    if (h->built_for(c, Lp->mlo)) return h;
  return nullptr;
}

// The correction is active for this context (options on, hierarchy built).
bool ml_on(const fcg_learned *Lp, const fcg_context *c) {
  return Lp->mlo.enabled && ml_for(Lp, c) != nullptr;
}

// Builds the aggregation hierarchy for c's mesh from the loaded matrix when the handle
// has none for it (once per mesh and options), then recomputes the level matrices from
// the loaded matrix (every call).
int ml_prepare(fcg_learned *Lp, fcg_context *c) {
  if (!Lp->mlo.enabled) return FCG_OK;
  fcg::ml::Hierarchy *H = ml_for(Lp, c);
  if (!H) {
    for (fcg::ml::Hierarchy *h : Lp->mlc)
      if (h->uid == c->uid) H = h;  // same context, rebound or other options: rebuild
    if (!H && Lp->mlc.size() >= kMlCache) H = Lp->mlc.front();
    if (!H) {
      H = new fcg::ml::Hierarchy();
      Lp->mlc.push_back(H);
    }
    std::string err;
    int rc = fcg::ml::build(*H, c, Lp->mlo, err);
    if (rc) return lp_fail(Lp, rc, err);
  }
  auto it = std::find(Lp->mlc.begin(), Lp->mlc.end(), H);
  Lp->mlc.erase(it);
  Lp->mlc.push_back(H);
  if (fcg::ml::values(*H, c, c->stream))
    return lp_cuda(Lp, cudaGetLastError(), "coarse level values");
  return FCG_OK;
}

// Loss and gradient of one (r, e) pair (device, FP32) into Lp->grad; sums at scal[2..3].
int loss_grad(fcg_learned *Lp, fcg_context *c, const float *r, const float *e) {
  int rc = ensure_workspace(Lp, c, true);
  if (rc) return rc;
  if (Lp->loss_kind == FCG_LP_LOSS_CYCLE) {
    if (!Lp->mlo.enabled)
      return lp_fail(Lp, FCG_ERR_STATE, "the cycle loss needs the coarse-grid correction on");
    if ((rc = ml_prepare(Lp, c))) return rc;
  }
  const int n = c->n;
  cudaStream_t st = c->stream;
  unsigned *tk = Lp->scal.as<unsigned>() + 16;
  enqueue_forward(Lp, c, st, r, true, nullptr, tk + 1, nullptr);
  float *rms = Lp->scal.as<float>();
  float *sums = rms + 2;
  const float *prm = Lp->params.as<float>();
  const int G = reduction_grid(c);
  float *dvec = Lp->dvec.as<float>(), *advec = dvec + Lp->ncap, *aadvec = advec + Lp->ncap;
  k_lp_out<<<grid_for(n, c->num_sms), kTPB, 0, st>>>(n, last_activation(Lp, c, true), prm, rms, r,
                                                     e, Lp->y.as<float>(), dvec, nullptr);
  const float *gy = advec;
  if (Lp->loss_kind == FCG_LP_LOSS_CYCLE) {
    // y_c = y + alpha P V P^T (r/rms - Ahat y), d = y_c - e/rms; loss d.Ahat d / t.Ahat t
    // (energy norm, t = e/rms); d loss / dy = E^T (2 Ahat d / t.Ahat t) with
    // E = I - alpha P V P^T Ahat: for the symmetric V that is u - Ahat (alpha P V P^T u),
    // u = Ahat d (the factor 2 / t.Ahat t is applied by k_lp_out_bwd)
    fcg::ml::Hierarchy *H = ml_for(Lp, c);
    float *yc = aadvec + Lp->ncap, *w = yc + Lp->ncap, *tmp = w + Lp->ncap;
    LP_TRY(Lp, cudaMemcpyAsync(yc, Lp->y.p, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
    fcg::ml::enqueue_correction(*H, c, Lp->mlo, st, Lp->feat.as<float>(), yc, nullptr);
    k_lp_cycle_d<<<grid_for(n, c->num_sms), kTPB, 0, st>>>(n, yc, e, rms, dvec);
    k_lp_aloss<<<G, kTPB, 0, st>>>(c->sv, n, scaled32(c), dvec, e, rms, advec,
                                   Lp->red.as<double>(), tk + 2, sums, 0);
    LP_TRY(Lp, cudaMemsetAsync(w, 0, sizeof(float) * n, st));
    fcg::ml::enqueue_correction(*H, c, Lp->mlo, st, advec, w, nullptr);
    k_lp_spmv32<<<G, kTPB, 0, st>>>(c->sv, n, scaled32(c), w, tmp);
    k_lp_cycle_g<<<grid_for(n, c->num_sms), kTPB, 0, st>>>(n, advec, tmp);
    gy = tmp;
  } else {
    k_lp_aloss<<<G, kTPB, 0, st>>>(c->sv, n, scaled32(c), dvec, e, rms, advec,
                                   Lp->red.as<double>(), tk + 2, sums, Lp->loss_kind);
    if (Lp->loss_kind == FCG_LP_LOSS_RESIDUAL) {
      k_lp_spmv32<<<G, kTPB, 0, st>>>(c->sv, n, scaled32(c), advec, aadvec);
      gy = aadvec;
    }
  }
  const int GB = c->num_sms * 2;  // blocks of the weight-gradient kernels
  float *part = Lp->part.as<float>();
  float *grad = Lp->grad.as<float>();
  const size_t hs = (size_t)n * lp::C;
  const __nv_bfloat16 *H = Lp->hbuf.as<__nv_bfloat16>();
  float *dh = Lp->dh.as<float>(), *dh2 = Lp->dh2.as<float>();
  k_lp_out_bwd<<<GB, kTPB, 0, st>>>(n, gy, sums, H + (size_t)lp::L * hs, prm, dh, part);
  k_lp_sum_parts<<<1, kTPB, 0, st>>>(part, GB, lp::C + 1, grad + lp::oWout);
  for (int l = lp::L - 1; l >= 0; --l) {
    k_lp_layer_bwd<<<GB, kTPB, 0, st>>>(n, dh, Lp->zbuf.as<float>() + (l + 1) * hs, H + l * hs,
                                        Lp->mbuf.as<float>() + l * hs,
                                        prm + lp::oLayer0 + l * lp::kLayerParams, dh2,
                                        Lp->dm.as<float>(), part);
    k_lp_sum_parts<<<grid_for(lp::kLayerParams, c->num_sms), kTPB, 0, st>>>(
        part, GB, lp::kLayerParams, grad + lp::oLayer0 + l * lp::kLayerParams);
    k_lp_agg_bwd<<<grid_for((long long)n * 32, c->num_sms), kTPB, 0, st>>>(
        c->sv, n, scaled32(c), Lp->dm.as<float>(), dh2);
    std::swap(dh, dh2);
  }
  k_lp_embed_bwd<<<GB, kTPB, 0, st>>>(n, dh, Lp->zbuf.as<float>(), Lp->feat.as<float>(), part);
  k_lp_sum_parts<<<1, kTPB, 0, st>>>(part, GB, lp::C * lp::F + lp::C, grad + lp::oWin);
  LP_TRY(Lp, cudaGetLastError());
  return FCG_OK;
}

int read_loss(fcg_learned *Lp, fcg_context *c, float *loss) {
  if (!loss) return FCG_OK;
  float h[2];
  LP_TRY(Lp, cudaMemcpyAsync(h, Lp->scal.as<float>() + 2, sizeof h, cudaMemcpyDeviceToHost,
                             c->stream));
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  *loss = h[1] > 0 ? h[0] / h[1] : h[0];
  return FCG_OK;
}

// Stages a host or device FP32 vector of the context's size (staging slots 4..5).
int stage_f32(fcg_learned *Lp, fcg_context *c, const float *user, int slot, bool copy_in,
              float **dev, bool *host) {
  void *d = nullptr;
  int rc = stage_in(c, user, sizeof(float) * c->n, slot, copy_in, &d, host);
  if (rc) return lp_fail(Lp, rc, fcg_last_error(c));
  *dev = (float *)d;
  return FCG_OK;
}

int matrix_ready(fcg_learned *Lp, fcg_context *c) {
  if (!features_current(Lp, c))
    return lp_fail(Lp, FCG_ERR_STATE,
                   "no scaled matrix for this context: call fcg_lp_set_matrix first");
  return FCG_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int fcg_lp_destroy(fcg_learned *Lp);

extern "C" int fcg_lp_create(int device, unsigned long long seed, fcg_learned **out) {
  if (!out) return FCG_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return FCG_ERR_CUDA;
  }
  fcg_learned *Lp = new fcg_learned();
  Lp->device = device;
  auto fail = [&](int rc) {
    cudaGetLastError();
    fcg_lp_destroy(Lp);
    return rc;
  };
  if (cudaDeviceGetAttribute(&Lp->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return fail(FCG_ERR_CUDA);
  const size_t pb = sizeof(float) * lp::P;
  if (Lp->params.ensure(pb) || Lp->adam_m.ensure(pb) || Lp->adam_v.ensure(pb) ||
      Lp->grad.ensure(pb) || Lp->wbf.ensure(sizeof(__nv_bfloat16) * lp::L * 2 * lp::C * lp::C) ||
      Lp->part.ensure(sizeof(float) * (size_t)Lp->num_sms * 2 * lp::kLayerParams) ||
      Lp->red.ensure(sizeof(double) * (lp::kMaxDir * kMaxBlocks + 8)) ||
      Lp->scal.ensure(sizeof(float) * 64) || cudaMalloc(&Lp->S, sizeof(lp::LScal)) ||
      cudaMallocHost(&Lp->hS, sizeof(lp::LScal)) ||
      cudaStreamCreateWithFlags(&Lp->cap, cudaStreamNonBlocking) ||
      cudaEventCreate(&Lp->ev0) || cudaEventCreate(&Lp->ev1) ||
      cudaEventCreateWithFlags(&Lp->ev_last, cudaEventDisableTiming))
    return fail(FCG_ERR_NOMEM);
  std::vector<float> p = init_params(seed);
  if (cudaMemcpy(Lp->params.p, p.data(), pb, cudaMemcpyHostToDevice) ||
      cudaMemset(Lp->adam_m.p, 0, pb) || cudaMemset(Lp->adam_v.p, 0, pb) ||
      cudaMemset(Lp->scal.p, 0, sizeof(float) * 64) || cudaMemset(Lp->S, 0, sizeof(lp::LScal)))
    return fail(FCG_ERR_CUDA);
  k_lp_to_bf16<<<64, kTPB>>>(Lp->params.as<float>(), Lp->wbf.as<__nv_bfloat16>());
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(FCG_ERR_CUDA);
  *out = Lp;
  return FCG_OK;
}

extern "C" int fcg_lp_destroy(fcg_learned *Lp) {
  if (!Lp) return FCG_OK;
  cudaSetDevice(Lp->device);
  if (Lp->ev_pending) cudaEventSynchronize(Lp->ev_last);
  if (Lp->ev_last) cudaEventDestroy(Lp->ev_last);
  if (Lp->exec) cudaGraphExecDestroy(Lp->exec);
  if (Lp->graph) cudaGraphDestroy(Lp->graph);
  if (Lp->cap) cudaStreamDestroy(Lp->cap);
  if (Lp->ev0) cudaEventDestroy(Lp->ev0);
  if (Lp->ev1) cudaEventDestroy(Lp->ev1);
  if (Lp->S) cudaFree(Lp->S);
  if (Lp->hS) cudaFreeHost(Lp->hS);
  DBuf *bufs[] = {&Lp->params, &Lp->adam_m, &Lp->adam_v, &Lp->grad, &Lp->wbf, &Lp->feat,
                  &Lp->hbuf,   &Lp->mbuf,   &Lp->zbuf,   &Lp->dh,   &Lp->dh2, &Lp->dm,
                  &Lp->y,      &Lp->dvec,   &Lp->part,   &Lp->red,  &Lp->scal, &Lp->fvec};
  for (DBuf *b : bufs) b->release();
  for (fcg::ml::Hierarchy *h : Lp->mlc) {
    h->release();
    delete h;
  }
  delete Lp;
  return FCG_OK;
}

extern "C" const char *fcg_lp_last_error(const fcg_learned *Lp) {
  return Lp ? Lp->err.c_str() : "NULL learned preconditioner";
}

extern "C" int fcg_lp_get_weights(fcg_learned *Lp, float *out, int count) {
  if (!Lp || !out || count != lp::P) return FCG_ERR_ARG;
  LP_TRY(Lp, cudaSetDevice(Lp->device));
  if (int rc = wait_last(Lp)) return rc;
  LP_TRY(Lp, cudaMemcpy(out, Lp->params.p, sizeof(float) * lp::P, cudaMemcpyDefault));
  return FCG_OK;
}

// Sets the weights (FP32, FCG_LP_PARAMS values) and clears the Adam state.
extern "C" int fcg_lp_set_weights(fcg_learned *Lp, const float *w, int count) {
  if (!Lp || !w || count != lp::P) return FCG_ERR_ARG;
  if (!is_device_pointer(w))
    for (int i = 0; i < count; ++i)
      if (!std::isfinite(w[i])) return lp_fail(Lp, FCG_ERR_NONFINITE, "non-finite weight");
  LP_TRY(Lp, cudaSetDevice(Lp->device));
  if (int rc = wait_last(Lp)) return rc;
  const size_t pb = sizeof(float) * lp::P;
  LP_TRY(Lp, cudaMemcpy(Lp->params.p, w, pb, cudaMemcpyDefault));
  LP_TRY(Lp, cudaMemset(Lp->adam_m.p, 0, pb));
  LP_TRY(Lp, cudaMemset(Lp->adam_v.p, 0, pb));
  Lp->step = 0;
  k_lp_to_bf16<<<64, kTPB>>>(Lp->params.as<float>(), Lp->wbf.as<__nv_bfloat16>());
  LP_TRY(Lp, cudaDeviceSynchronize());
  return FCG_OK;
}

// Checkpoint: "FCGLP001", int32 width, layers, features, parameter count, int64 Adam
// step, then the parameters, Adam m and Adam v as FP32 (host byte order).
extern "C" int fcg_lp_save(fcg_learned *Lp, const char *path) {
  if (!Lp || !path) return FCG_ERR_ARG;
  std::vector<float> buf(3 * (size_t)lp::P);
  LP_TRY(Lp, cudaSetDevice(Lp->device));
  if (int rc = wait_last(Lp)) return rc;
  const size_t pb = sizeof(float) * lp::P;
  LP_TRY(Lp, cudaMemcpy(buf.data(), Lp->params.p, pb, cudaMemcpyDeviceToHost));
  LP_TRY(Lp, cudaMemcpy(buf.data() + lp::P, Lp->adam_m.p, pb, cudaMemcpyDeviceToHost));
  LP_TRY(Lp, cudaMemcpy(buf.data() + 2 * lp::P, Lp->adam_v.p, pb, cudaMemcpyDeviceToHost));
  FILE *f = std::fopen(path, "wb");
  if (!f) return lp_fail(Lp, FCG_ERR_ARG, std::string("cannot write ") + path);
  const int hdr[4] = {lp::C, lp::L, lp::F, lp::P};
  const long long step = Lp->step;
  bool ok = std::fwrite("FCGLP001", 1, 8, f) == 8 && std::fwrite(hdr, sizeof hdr, 1, f) == 1 &&
            std::fwrite(&step, sizeof step, 1, f) == 1 &&
            std::fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? FCG_OK : lp_fail(Lp, FCG_ERR_ARG, std::string("short write to ") + path);
}

extern "C" int fcg_lp_load(fcg_learned *Lp, const char *path) {
  if (!Lp || !path) return FCG_ERR_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return lp_fail(Lp, FCG_ERR_ARG, std::string("cannot read ") + path);
  char magic[8];
  int hdr[4];
  long long step = 0;
  std::vector<float> buf(3 * (size_t)lp::P);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "FCGLP001", 8) == 0 &&
            std::fread(hdr, sizeof hdr, 1, f) == 1 && hdr[0] == lp::C && hdr[1] == lp::L &&
            hdr[2] == lp::F && hdr[3] == lp::P && std::fread(&step, sizeof step, 1, f) == 1 &&
            std::fread(buf.data(), sizeof(float), buf.size(), f) == buf.size();
  std::fclose(f);
  if (!ok) return lp_fail(Lp, FCG_ERR_ARG, std::string("not a matching checkpoint: ") + path);
  for (float v : buf)
    if (!std::isfinite(v)) return lp_fail(Lp, FCG_ERR_NONFINITE, "non-finite value in checkpoint");
  LP_TRY(Lp, cudaSetDevice(Lp->device));
  if (int rc = wait_last(Lp)) return rc;
  const size_t pb = sizeof(float) * lp::P;
  LP_TRY(Lp, cudaMemcpy(Lp->params.p, buf.data(), pb, cudaMemcpyHostToDevice));
  LP_TRY(Lp, cudaMemcpy(Lp->adam_m.p, buf.data() + lp::P, pb, cudaMemcpyHostToDevice));
  LP_TRY(Lp, cudaMemcpy(Lp->adam_v.p, buf.data() + 2 * lp::P, pb, cudaMemcpyHostToDevice));
  Lp->step = step;
  k_lp_to_bf16<<<64, kTPB>>>(Lp->params.as<float>(), Lp->wbf.as<__nv_bfloat16>());
  LP_TRY(Lp, cudaDeviceSynchronize());
  return FCG_OK;
}

// Loads CSR values a (host or device) into the context's solver state, builds the FP32
// scaled matrix and the per-cell features.
extern "C" int fcg_lp_set_matrix(fcg_learned *Lp, fcg_context *c, const double *a) {
  int rc = check_ctx(Lp, c);
  if (rc) return rc;
  if (!a) return lp_fail(Lp, FCG_ERR_ARG, "NULL a");
  void *da;
  bool ha;
  if ((rc = stage_in(c, a, sizeof(double) * c->nnz, 0, true, &da, &ha)))
    return lp_fail(Lp, rc, fcg_last_error(c));
  if ((rc = prepare_scaled32(c, (const double *)da))) return lp_fail(Lp, rc, fcg_last_error(c));
  if ((rc = compute_features(Lp, c))) return rc;
  return mark_done(Lp, c);
}

extern "C" int fcg_lp_features(fcg_learned *Lp, fcg_context *c, float *out) {
  int rc = check_ctx(Lp, c);
  if (rc) return rc;
  if (!out) return FCG_ERR_ARG;
  if ((rc = matrix_ready(Lp, c))) return rc;
  LP_TRY(Lp, cudaMemcpyAsync(out, Lp->feat.p, sizeof(float) * lp::F * c->n, cudaMemcpyDefault,
                             c->stream));
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

// z = N(r) for the scaled system of the matrix last set (FP32 vectors, host or device).
extern "C" int fcg_lp_apply(fcg_learned *Lp, fcg_context *c, const float *r, float *z) {
  int rc = check_ctx(Lp, c);
  if (rc) return rc;
  if (!r || !z) return lp_fail(Lp, FCG_ERR_ARG, "NULL r or z");
  if ((rc = matrix_ready(Lp, c)) || (rc = ensure_workspace(Lp, c, false))) return rc;
  float *dr, *dz;
  bool hr, hz;
  if ((rc = stage_f32(Lp, c, r, 4, true, &dr, &hr))) return rc;
  if ((rc = stage_f32(Lp, c, z, 5, false, &dz, &hz))) return rc;
  enqueue_forward(Lp, c, c->stream, dr, false, nullptr, Lp->scal.as<unsigned>() + 17,
                  Lp->scal.as<int>() + kHexStatus);
  k_lp_out<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(
      c->n, last_activation(Lp, c, false), Lp->params.as<float>(), Lp->scal.as<float>(), dr,
      nullptr, nullptr, nullptr, dz);
  LP_TRY(Lp, cudaGetLastError());
  if ((rc = stage_out(c, z, dz, sizeof(float) * c->n, hz)))
    return lp_fail(Lp, rc, fcg_last_error(c));
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  if ((rc = hex_status(Lp, c))) return rc;
  return mark_done(Lp, c);
}

// Diagnostics: mean milliseconds of each kernel of one forward pass on r (host or
// device), CUDA events around every launch: 0 k_lp_rms, 1 k_lp_embed, 2..7 k_lp_layer
// (layers 1..6), 8 k_lp_out.
extern "C" int fcg_lp_profile(fcg_learned *Lp, fcg_context *c, const float *r, int reps,
                              double *ms, int max_units, int *units) {
  int rc = check_ctx(Lp, c);
  if (rc) return rc;
  if (!r || reps < 1 || !ms) return lp_fail(Lp, FCG_ERR_ARG, "NULL r/ms or reps < 1");
  if ((rc = matrix_ready(Lp, c)) || (rc = ensure_workspace(Lp, c, false))) return rc;
  float *dr;
  bool hr;
  if ((rc = stage_f32(Lp, c, r, 4, true, &dr, &hr))) return rc;
  constexpr int U = 3 + lp::L;
  cudaEvent_t ev[U + 1];
  for (auto &e : ev) LP_TRY(Lp, cudaEventCreate(&e));
  double acc[U] = {0};
  const int n = c->n;
  cudaStream_t st = c->stream;
  const size_t hs = (size_t)n * lp::C;
  __nv_bfloat16 *H = Lp->hbuf.as<__nv_bfloat16>();
  float *rms = Lp->scal.as<float>();
  const float *prm = Lp->params.as<float>();
  const int ntiles = (n + 15) / 16;
  const int lg = std::max(1, std::min((ntiles + 7) / 8, c->num_sms * 4));
  for (int it = 0; it <= reps; ++it) {  // the first pass warms up
    LP_TRY(Lp, cudaEventRecord(ev[0], st));
    k_lp_rms<<<reduction_grid(c), kTPB, 0, st>>>(n, dr, Lp->red.as<double>(),
                                                 Lp->scal.as<unsigned>() + 17, rms, nullptr);
    LP_TRY(Lp, cudaEventRecord(ev[1], st));
    k_lp_embed<<<grid_for(n, c->num_sms, 8), kTPB, 0, st>>>(n, dr, rms, Lp->feat.as<float>(),
                                                                 prm, H, nullptr, nullptr);
    LP_TRY(Lp, cudaEventRecord(ev[2], st));
    for (int l = 0; l < lp::L; ++l) {
      const __nv_bfloat16 *wl = Lp->wbf.as<__nv_bfloat16>() + (size_t)l * 2 * lp::C * lp::C;
      const float *bl = prm + lp::oLayer0 + l * lp::kLayerParams + 2 * lp::C * lp::C;
      if (layer_split()) {
        k_lp_agg<<<grid_for(4LL * n, c->num_sms, 8), kTPB, 0, st>>>(
            c->sv, n, scaled32(c), H + (l % 2) * hs, H + 2 * hs, nullptr);
        k_lp_dense<<<lg, kTPB, 0, st>>>(n, H + (l % 2) * hs, H + 2 * hs, H + ((l + 1) % 2) * hs,
                                        wl, bl, nullptr);
      } else if (hex_on(Lp, c) &&
                 fcg::lphex::layer(Lp->hex, c->num_sms, H + (l % 2) * hs,
                                   H + ((l + 1) % 2) * hs, Lp->hexval.as<float>(), wl, bl,
                                   nullptr, Lp->scal.as<int>() + kHexStatus, st) == cudaSuccess) {
        // plane-staged form launched
      } else {
        k_lp_layer<<<lg, kTPB, 0, st>>>(c->sv, n, scaled32(c), H + (l % 2) * hs,
                                        H + ((l + 1) % 2) * hs, wl, bl, nullptr, nullptr, nullptr);
      }
      LP_TRY(Lp, cudaEventRecord(ev[3 + l], st));
    }
    k_lp_out<<<grid_for(n, c->num_sms), kTPB, 0, st>>>(n, H + (lp::L % 2) * hs, prm, rms, dr,
                                                       nullptr, Lp->y.as<float>(), nullptr,
                                                       nullptr);
    LP_TRY(Lp, cudaEventRecord(ev[U], st));
    LP_TRY(Lp, cudaGetLastError());
    LP_TRY(Lp, cudaEventSynchronize(ev[U]));
    if (it == 0) continue;
    for (int u = 0; u < U; ++u) {
      float t = 0.f;
      LP_TRY(Lp, cudaEventElapsedTime(&t, ev[u], ev[u + 1]));
      acc[u] += t;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if ((rc = hex_status(Lp, c))) return rc;
  const int nu = std::min(U, max_units);
  for (int u = 0; u < nu; ++u) ms[u] = acc[u] / reps;
  if (units) *units = U;
  return mark_done(Lp, c);
}

extern "C" int fcg_lp_layer_form(fcg_learned *Lp, fcg_context *c, int *form, int *dims) {
  int rc = check_ctx(Lp, c);
  if (rc) return rc;
  if (!form) return lp_fail(Lp, FCG_ERR_ARG, "NULL form");
  if ((rc = matrix_ready(Lp, c))) return rc;
  const bool on = hex_on(Lp, c);
  *form = on ? FCG_LP_LAYER_PLANES : FCG_LP_LAYER_GATHER;
  if (dims) {
    dims[0] = on ? Lp->hex.nx : 0;
    dims[1] = on ? Lp->hex.ny : 0;
    dims[2] = on ? Lp->hex.nz : 0;
  }
  return FCG_OK;
}

// loss = ||N(r) - e||^2 / ||e||^2 and its gradient with respect to the FP32 weights.
extern "C" int fcg_lp_loss_grad(fcg_learned *Lp, fcg_context *c, const float *r, const float *e,
                                float *loss, float *grad) {
  int rc = check_ctx(Lp, c);
  if (rc) return rc;
  if (!r || !e) return lp_fail(Lp, FCG_ERR_ARG, "NULL r or e");
  if ((rc = matrix_ready(Lp, c))) return rc;
  float *dr, *de;
  bool hr, he;
  if ((rc = stage_f32(Lp, c, r, 4, true, &dr, &hr))) return rc;
  if ((rc = stage_f32(Lp, c, e, 5, true, &de, &he))) return rc;
  if ((rc = loss_grad(Lp, c, dr, de))) return rc;
  if (grad)
    LP_TRY(Lp, cudaMemcpyAsync(grad, Lp->grad.p, sizeof(float) * lp::P, cudaMemcpyDefault,
                               c->stream));
  if ((rc = read_loss(Lp, c, loss))) return rc;
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  return mark_done(Lp, c);
}

// One Adam step on the pair (r, e); loss (before the step) returned when loss != NULL.
extern "C" int fcg_lp_train_step(fcg_learned *Lp, fcg_context *c, const float *r, const float *e,
                                 float lr, float *loss) {
  int rc = check_ctx(Lp, c);
  if (rc) return rc;
  if (!r || !e || !(lr > 0.f)) return lp_fail(Lp, FCG_ERR_ARG, "NULL r/e or lr <= 0");
  if ((rc = matrix_ready(Lp, c))) return rc;
  float *dr, *de;
  bool hr, he;
  if ((rc = stage_f32(Lp, c, r, 4, true, &dr, &hr))) return rc;
  if ((rc = stage_f32(Lp, c, e, 5, true, &de, &he))) return rc;
  if ((rc = loss_grad(Lp, c, dr, de))) return rc;
  Lp->step++;
  const float c1 = 1.f - std::pow(0.9f, (float)Lp->step);
  const float c2 = 1.f - std::pow(0.999f, (float)Lp->step);
  k_lp_adam<<<grid_for(lp::P, c->num_sms), kTPB, 0, c->stream>>>(
      Lp->params.as<float>(), Lp->adam_m.as<float>(), Lp->adam_v.as<float>(),
      Lp->grad.as<float>(), lr, c1, c2);
  k_lp_to_bf16<<<64, kTPB, 0, c->stream>>>(Lp->params.as<float>(), Lp->wbf.as<__nv_bfloat16>());
  LP_TRY(Lp, cudaGetLastError());
  if ((rc = mark_done(Lp, c))) return rc;
  return read_loss(Lp, c, loss);
}

extern "C" int fcg_lp_set_loss(fcg_learned *Lp, int kind) {
  if (!Lp || kind < FCG_LP_LOSS_ENERGY || kind > FCG_LP_LOSS_CYCLE) return FCG_ERR_ARG;
  Lp->loss_kind = kind;
  return FCG_OK;
}

// Iterations and FP64 residual replacements of the last fcg_fcg_learned call (the
// reliable-update branch of the CUDA graph runs two kernels per replacement).
extern "C" int fcg_lp_last_solve_stats(const fcg_learned *Lp, int *iters, int *updates) {
  if (!Lp || !Lp->hS) return FCG_ERR_ARG;
  if (iters) *iters = Lp->hS->iter;
  if (updates) *updates = Lp->hS->nupdates;
  return FCG_OK;
}

extern "C" int fcg_lp_set_fcg_options(fcg_learned *Lp, int directions, int ru_every,
                                      int stall_window, double stall_factor) {
  if (!Lp || directions < 1 || directions > lp::kMaxDir || ru_every < 1 || stall_window < 1 ||
      !(stall_factor > 0.0) || !(stall_factor <= 1.0))
    return FCG_ERR_ARG;
  Lp->mdir = directions;
  Lp->ru_every = ru_every;
  Lp->stall_window = stall_window;
  Lp->stall_factor = stall_factor;
  return FCG_OK;
}

namespace {

struct FcgVecs {
  double *x, *res, *su;
  float *y, *r, *z, *p, *q;  // p, q: rings of kMaxDir vectors, `stride` apart
  long long stride;
};

size_t fcg_bytes(int n) {
  const size_t n8 = ((size_t)n + 63) & ~(size_t)63;
  return 3 * n8 * sizeof(double) + (3 + 2 * lp::kMaxDir) * n8 * sizeof(float);
}

FcgVecs fcg_vectors(fcg_learned *Lp, int n) {
  const size_t n8 = ((size_t)n + 63) & ~(size_t)63;
  double *d = Lp->fvec.as<double>();
  float *f = (float *)(d + 3 * n8);
  return {d,      d + n8,          d + 2 * n8, f, f + n8, f + 2 * n8, f + 3 * n8,
          f + (3 + lp::kMaxDir) * n8, (long long)n8};
}

// z = M(r): the network (or Jacobi sweeps) followed by the coarse-grid correction.  In
// the flexible CG (S given) the output kernel honours S->done and leaves the dot
// products to k_f_zdots.
void enqueue_preconditioner(fcg_learned *Lp, fcg_context *c, cudaStream_t st, const float *r,
                            float *z, const int *done, unsigned *rms_ticket, lp::LScal *S) {
  const int n = c->n;
  if (Lp->mlo.smoother == FCG_LP_SMOOTH_JACOBI) {
    fcg::ml::enqueue_jacobi_cycle(*ml_for(Lp, c), c, Lp->mlo, st, r, z, done);
    return;
  }
  // in the flexible CG the plane-staged last layer writes z itself (the same bits as
  // k_f_out on h_L, which is then not stored)
  const fcg::lphex::OutFuse of{r, Lp->scal.as<float>(), Lp->params.as<float>() + lp::oWout, z};
  bool fused = false;
  enqueue_forward(Lp, c, st, r, false, done, rms_ticket,
                  S ? &S->status : Lp->scal.as<int>() + kHexStatus, S ? &of : nullptr, &fused);
  if (S && !fused)
    k_f_out<<<reduction_grid(c), kTPB, 0, st>>>(n, last_activation(Lp, c, false),
                                                Lp->params.as<float>(), Lp->scal.as<float>(), r,
                                                z, nullptr, 0, S, nullptr, 0);
  else if (!S)
    k_lp_out<<<grid_for(n, c->num_sms), kTPB, 0, st>>>(n, last_activation(Lp, c, false),
                                                       Lp->params.as<float>(),
                                                       Lp->scal.as<float>(), r, nullptr, nullptr,
                                                       nullptr, z);
  fcg::ml::enqueue_correction(*ml_for(Lp, c), c, Lp->mlo, st, r, z, done);
}

void enqueue_body_head(fcg_learned *Lp, fcg_context *c, cudaStream_t st, const FcgVecs &v,
                       cudaGraphConditionalHandle hif, int use_cond) {
  const int n = c->n;
  const int G = reduction_grid(c);
  double *red = Lp->red.as<double>();
  const int *done = &Lp->S->done;
  if (!ml_on(Lp, c)) {
    enqueue_forward(Lp, c, st, v.r, false, done, &Lp->S->ticket[6], &Lp->S->status);
    k_f_out<<<G, kTPB, 0, st>>>(n, last_activation(Lp, c, false), Lp->params.as<float>(),
                                Lp->scal.as<float>(), v.r, v.z, v.q, v.stride, Lp->S, red, 1);
  } else {
    enqueue_preconditioner(Lp, c, st, v.r, v.z, done, &Lp->S->ticket[6], Lp->S);
    k_f_zdots<<<G, kTPB, 0, st>>>(n, v.z, v.q, v.stride, Lp->S, red);
  }
  k_f_p<<<grid_for(n, c->num_sms), kTPB, 0, st>>>(n, v.z, v.p, v.stride, Lp->S);
  k_f_spmv<<<G, kTPB, 0, st>>>(c->sv, n, scaled32(c), v.p, v.q, v.stride, v.r, Lp->S, red);
  k_f_update<<<G, kTPB, 0, st>>>(n, v.y, v.r, v.p, v.q, v.stride, Lp->S, red, hif, use_cond);
}

void enqueue_ru(fcg_learned *Lp, fcg_context *c, cudaStream_t st, const FcgVecs &v) {
  const int n = c->n;
  k_f_ru1<<<grid_for(n, c->num_sms), kTPB, 0, st>>>(n, v.x, v.y, scale64(c), Lp->S);
  k_f_ru2<<<reduction_grid(c), kTPB, 0, st>>>(c->sv, n, sliced64(c), v.su, v.x, v.res, scale64(c),
                                              v.r, Lp->S, Lp->red.as<double>());
}

int build_fcg_graph(fcg_learned *Lp, fcg_context *c, const FcgVecs &v) {
  std::vector<const void *> key = {(const void *)(uintptr_t)c->uid,
                                   (const void *)(uintptr_t)c->bind_gen,
                                   scaled32(c), scale64(c),
                                   sliced64(c), Lp->fvec.p,
                                   Lp->hbuf.p,  Lp->feat.p,
                                   c->stream,   (const void *)(uintptr_t)c->n,
                                   (const void *)(uintptr_t)ml_on(Lp, c),
                                   (const void *)ml_for(Lp, c),
                                   (const void *)(uintptr_t)(ml_for(Lp, c) ? ml_for(Lp, c)->build_id : 0),
                                   (const void *)(uintptr_t)Lp->mlo.smoother,
                                   (const void *)(uintptr_t)Lp->mlo.sweeps,
                                   (const void *)(uintptr_t)(Lp->mlo.alpha * 1e6),
                                   (const void *)(uintptr_t)(Lp->mlo.omega * 1e6),
                                   (const void *)(uintptr_t)Lp->mlo.smoothed,
                                   (const void *)(uintptr_t)hex_on(Lp, c), Lp->hexval.p};
  if (Lp->exec && key == Lp->graph_key) return FCG_OK;
  if (Lp->exec) cudaGraphExecDestroy(Lp->exec);
  if (Lp->graph) cudaGraphDestroy(Lp->graph);
  Lp->exec = nullptr;
  Lp->graph = nullptr;
  cudaGraph_t g;
  LP_TRY(Lp, cudaGraphCreate(&g, 0));
  auto fail = [&](cudaError_t e, const char *what) {
    cudaGraphDestroy(g);
    return lp_cuda(Lp, e, what);
  };
  cudaGraphConditionalHandle h, hif;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (e) return fail(e, "conditional handle");
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t loop;
  if ((e = cudaGraphAddNode(&loop, g, nullptr, nullptr, 0, &np))) return fail(e, "WHILE node");
  cudaGraph_t body = np.conditional.phGraph_out[0];
  if ((e = cudaGraphConditionalHandleCreate(&hif, body, 0, cudaGraphCondAssignDefault)))
    return fail(e, "IF handle");
  if ((e = cudaStreamBeginCaptureToGraph(Lp->cap, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal)))
    return fail(e, "capture");
  enqueue_body_head(Lp, c, Lp->cap, v, hif, 1);
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  cudaGraph_t captured = nullptr;
  if ((e = cudaStreamGetCaptureInfo(Lp->cap, &cs, nullptr, nullptr, &deps, nullptr, &nd))) {
    cudaStreamEndCapture(Lp->cap, &captured);
    return fail(e, "capture info");
  }
  cudaGraphNodeParams ip = {cudaGraphNodeTypeConditional};
  ip.conditional.handle = hif;
  ip.conditional.type = cudaGraphCondTypeIf;
  ip.conditional.size = 1;
  cudaGraphNode_t ifnode;
  if ((e = cudaGraphAddNode(&ifnode, body, deps, nullptr, nd, &ip)) ||
      (e = cudaStreamUpdateCaptureDependencies(Lp->cap, &ifnode, nullptr, 1,
                                               cudaStreamSetCaptureDependencies))) {
    cudaStreamEndCapture(Lp->cap, &captured);
    return fail(e, "IF node");
  }
  k_f_close<<<1, 32, 0, Lp->cap>>>(Lp->S, h, 1);
  if ((e = cudaStreamEndCapture(Lp->cap, &captured))) return fail(e, "end of capture");
  if ((e = cudaStreamBeginCaptureToGraph(Lp->cap, ip.conditional.phGraph_out[0], nullptr, nullptr,
                                         0, cudaStreamCaptureModeThreadLocal)))
    return fail(e, "capture of the reliable update");
  enqueue_ru(Lp, c, Lp->cap, v);
  if ((e = cudaStreamEndCapture(Lp->cap, &captured))) return fail(e, "end of capture");
  if ((e = cudaGraphInstantiate(&Lp->exec, g, 0))) return fail(e, "cudaGraphInstantiate (FCG)");
  Lp->graph = g;
  Lp->graph_key = key;
  return FCG_OK;
}

bool graphs_off() {
  const char *e = std::getenv("FCG_NO_GRAPH");
  return e && e[0] == '1';
}

}  // namespace

// Learned-preconditioned flexible CG on A fi = su (the argument meaning of fcg_dpcg).
// rep->iters counts FCG iterations plus the DPCG sweeps of a fallback; *fcg_iters (if
// not NULL) the FCG iterations alone, *fallback (if not NULL) 1 when DPCG finished it.
extern "C" int fcg_fcg_learned(fcg_context *c, fcg_learned *Lp, const double *a,
                               const double *su, double *fi, double *res, double sor, int nsw,
                               double *resor, fcg_solve_report *rep, int *fcg_iters,
                               int *fallback) {
  if (!c || !Lp) return FCG_ERR_ARG;
  int rc = check_ctx(Lp, c);
  if (rc) return set_error(c, rc, Lp->err);
  if (!a || !su || !fi) return set_error(c, FCG_ERR_ARG, "NULL a, su or fi");
  if (nsw < 0) return set_error(c, FCG_ERR_ARG, "nsw must be >= 0");
  const int n = c->n;
  const size_t n1 = sizeof(double) * n;
  void *da, *dsu, *dfi;
  bool ha, hsu, hfi;
  if ((rc = stage_in(c, a, sizeof(double) * c->nnz, 0, true, &da, &ha))) return rc;
  if ((rc = stage_in(c, su, n1, 1, true, &dsu, &hsu))) return rc;
  if ((rc = stage_in(c, fi, n1, 2, true, &dfi, &hfi))) return rc;
  FCG_CUDA_TRY(c, cudaEventRecord(Lp->ev0, c->stream));
  if ((rc = prepare_scaled32(c, (const double *)da))) return rc;
  if ((rc = compute_features(Lp, c))) return set_error(c, rc, Lp->err);
  if ((rc = ensure_workspace(Lp, c, false))) return set_error(c, rc, Lp->err);
  if ((rc = ml_prepare(Lp, c))) return set_error(c, rc, Lp->err);
  const size_t n8 = ((size_t)n + 63) & ~(size_t)63;
  (void)n8;
  FCG_CUDA_TRY(c, Lp->fvec.ensure(fcg_bytes(n)));
  const FcgVecs v = fcg_vectors(Lp, n);
  FCG_CUDA_TRY(c, cudaMemcpyAsync(v.su, dsu, n1, cudaMemcpyDeviceToDevice, c->stream));
  FCG_CUDA_TRY(c, cudaMemcpyAsync(v.x, dfi, n1, cudaMemcpyDeviceToDevice, c->stream));
  lp::LScal init;
  std::memset(&init, 0, sizeof init);
  init.small = (double)1e-20f;  // parameters::small (modules_allocatable.f90:27)
  init.resmax = sor;
  init.delta = Lp->delta;
  init.nsw = nsw;
  init.ru_every = Lp->ru_every;
  init.stall_window = Lp->stall_window;
  init.stall_factor = Lp->stall_factor;
  init.mdir = Lp->mdir;
  *Lp->hS = init;
  FCG_CUDA_TRY(c, cudaMemcpyAsync(Lp->S, Lp->hS, sizeof(lp::LScal), cudaMemcpyHostToDevice,
                                  c->stream));
  const int G = reduction_grid(c);
  k_f_init<<<G, kTPB, 0, c->stream>>>(c->sv, n, sliced64(c), v.su, v.x, v.res, scale64(c), v.r,
                                      v.y, Lp->S, Lp->red.as<double>());
  FCG_CHECK_LAUNCH(c, "k_f_init");
  if (!graphs_off()) {
    if ((rc = build_fcg_graph(Lp, c, v))) return set_error(c, rc, Lp->err);
    FCG_CUDA_TRY(c, cudaGraphLaunch(Lp->exec, c->stream));
  } else {
    // host-driven loop (for profilers that do not follow conditional graph nodes)
    for (int it = 0; it <= nsw + 1; it += 8) {
      for (int j = 0; j < 8; ++j) {
        enqueue_body_head(Lp, c, c->stream, v, 0, 0);
        enqueue_ru(Lp, c, c->stream, v);
        k_f_close<<<1, 32, 0, c->stream>>>(Lp->S, 0, 0);
      }
      FCG_CHECK_LAUNCH(c, "FCG iterations");
      FCG_CUDA_TRY(c, cudaMemcpyAsync(Lp->hS, Lp->S, sizeof(lp::LScal), cudaMemcpyDeviceToHost,
                                      c->stream));
      FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      if (Lp->hS->done) break;
    }
  }
  FCG_CUDA_TRY(c, cudaMemcpyAsync(Lp->hS, Lp->S, sizeof(lp::LScal), cudaMemcpyDeviceToHost,
                                  c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const lp::LScal S = *Lp->hS;
  int total = S.iter, used_fallback = 0;
  const double res0 = S.res0;
  double resl = S.resl;
  bool converged = S.converged != 0;
  int status = 0;
  if (!converged && S.status != FCG_ERR_TIMEOUT && nsw - S.iter > 0 && S.res0 > 0) {
    // FP64 DPCG from the current solution, to the same absolute target
    fcg_solve_report r2;
    double resor2 = 0.0;
    const double sor2 = S.resl > 0 ? sor * (S.res0 + init.small) / S.resl : sor;
    rc = fcg_dpcg(c, (const double *)da, v.su, v.x, v.res, sor2, nsw - S.iter, &resor2, &r2);
    if (rc) return rc;
    used_fallback = 1;
    total += r2.iters;
    resl = r2.resl;
    converged = resl / (res0 + init.small) < sor;
  } else if (S.status && !converged) {
    status = S.status;
  }
  k_f_final<<<G, kTPB, 0, c->stream>>>(c->sv, n, sliced64(c), v.su, v.x, Lp->S,
                                       Lp->red.as<double>());
  FCG_CHECK_LAUNCH(c, "k_f_final");
  FCG_CUDA_TRY(c, cudaEventRecord(Lp->ev1, c->stream));
  FCG_CUDA_TRY(c, cudaMemcpyAsync(dfi, v.x, n1, cudaMemcpyDeviceToDevice, c->stream));
  if ((rc = stage_out(c, fi, dfi, n1, hfi))) return rc;
  if (res) {
    void *dres;
    bool hres;
    if ((rc = stage_in(c, res, n1, 3, false, &dres, &hres))) return rc;
    FCG_CUDA_TRY(c, cudaMemcpyAsync(dres, v.res, n1, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = stage_out(c, res, dres, n1, hres))) return rc;
  }
  FCG_CUDA_TRY(c, cudaMemcpyAsync(Lp->hS, Lp->S, sizeof(lp::LScal), cudaMemcpyDeviceToHost,
                                  c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if ((rc = mark_done(Lp, c))) return set_error(c, rc, Lp->err);
  if (resor && total > 0) *resor = res0;
  if (fcg_iters) *fcg_iters = S.iter;
  if (fallback) *fallback = used_fallback;
  if (rep) {
    rep->res0 = res0;
    rep->resl = resl;
    rep->iters = total;
    rep->converged = converged ? 1 : 0;
    rep->l2_rel = Lp->hS->l2b > 0 ? std::sqrt(Lp->hS->l2r / Lp->hS->l2b) : std::sqrt(Lp->hS->l2r);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, Lp->ev0, Lp->ev1);
    rep->seconds = ms * 1e-3;
  }
  if (status)
    return set_error(c, status, status == FCG_ERR_TIMEOUT ? "FCG loop exceeded nsw + 2 bodies"
                                                          : "non-finite value in the FCG");
  return FCG_OK;
}

// ---------------------------------------------------------------------------
// Coarse-grid correction: options, hierarchy, standalone application
// ---------------------------------------------------------------------------
extern "C" int fcg_lp_set_multilevel(fcg_learned *Lp, const fcg_lp_multilevel *o) {
  if (!Lp || !o) return FCG_ERR_ARG;
  if ((o->enabled != 0 && o->enabled != 1) ||
      (o->smoother != FCG_LP_SMOOTH_NETWORK && o->smoother != FCG_LP_SMOOTH_JACOBI) ||
      o->sweeps < 1 || o->sweeps > 8 || o->max_levels < 2 || o->max_levels > FCG_LP_MAX_LEVELS ||
      o->dense_max < 1 || o->dense_max > 160 || !(o->alpha > 0.0 && o->alpha < 4.0) ||
      !(o->omega > 0.0 && o->omega < 2.0) || (o->smoothed != 0 && o->smoothed != 1))
    return lp_fail(Lp, FCG_ERR_ARG, "multilevel option out of range");
  Lp->mlo.enabled = o->enabled;
  Lp->mlo.smoother = o->smoother;
  Lp->mlo.sweeps = o->sweeps;
  Lp->mlo.max_levels = o->max_levels;
  Lp->mlo.dense_max = o->dense_max;
  Lp->mlo.alpha = o->alpha;
  Lp->mlo.omega = o->omega;
  Lp->mlo.smoothed = o->smoothed;
  return FCG_OK;
}

extern "C" int fcg_lp_get_multilevel(const fcg_learned *Lp, fcg_lp_multilevel *o) {
  if (!Lp || !o) return FCG_ERR_ARG;
  o->enabled = Lp->mlo.enabled;
  o->smoother = Lp->mlo.smoother;
  o->sweeps = Lp->mlo.sweeps;
  o->max_levels = Lp->mlo.max_levels;
  o->dense_max = Lp->mlo.dense_max;
  o->alpha = Lp->mlo.alpha;
  o->omega = Lp->mlo.omega;
  o->smoothed = Lp->mlo.smoothed;
  return FCG_OK;
}

namespace {
int ml_ready(fcg_learned *Lp, fcg_context *c) {
  int rc = check_ctx(Lp, c);
  if (rc) return rc;
  if ((rc = matrix_ready(Lp, c))) return rc;
  if (!Lp->mlo.enabled) return lp_fail(Lp, FCG_ERR_STATE, "the coarse-grid correction is off");
  return ml_prepare(Lp, c);
}
}  // namespace

extern "C" int fcg_lp_hierarchy_info(fcg_learned *Lp, fcg_context *c, int *levels, int *cells,
                                     long long *entries, double *setup_seconds) {
  int rc = ml_ready(Lp, c);
  if (rc) return rc;
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  const fcg::ml::Hierarchy &H = *ml_for(Lp, c);
  const int nl = (int)H.lv.size() + 1;
  if (levels) *levels = nl;
  for (int l = 0; l < nl; ++l) {
    if (cells) cells[l] = l == 0 ? c->n : H.lv[l - 1].n;
    if (entries) entries[l] = l == 0 ? c->nnz : H.lv[l - 1].nnz;
  }
  if (setup_seconds) *setup_seconds = H.setup_seconds;
  return mark_done(Lp, c);
}

extern "C" int fcg_lp_hierarchy_built_on(fcg_learned *Lp, fcg_context *c, int *on_device) {
  if (!on_device) return FCG_ERR_ARG;
  int rc = ml_ready(Lp, c);
  if (rc) return rc;
  *on_device = ml_for(Lp, c)->built_on_device ? 1 : 0;
  return mark_done(Lp, c);
}

extern "C" int fcg_lp_hierarchy_level(fcg_learned *Lp, fcg_context *c, int level, int *agg,
                                      int *mptr, int *mem, int *ptr, int *col, float *val) {
  int rc = ml_ready(Lp, c);
  if (rc) return rc;
  const fcg::ml::Hierarchy &H = *ml_for(Lp, c);
  if (level < 1 || level > (int)H.lv.size())
    return lp_fail(Lp, FCG_ERR_ARG, "no such coarse level");
  const fcg::ml::DevLevel &L = H.lv[level - 1];
  const int np = level == 1 ? c->n : H.lv[level - 2].n;
  auto get = [&](void *dst, const void *src, size_t b) {
    return dst ? cudaMemcpyAsync(dst, src, b, cudaMemcpyDefault, c->stream) : cudaSuccess;
  };
  LP_TRY(Lp, get(agg, L.agg, sizeof(int) * np));
  LP_TRY(Lp, get(mptr, L.mptr, sizeof(int) * (L.n + 1)));
  LP_TRY(Lp, get(mem, L.mem, sizeof(int) * np));
  LP_TRY(Lp, get(ptr, L.ptr, sizeof(int) * (L.n + 1)));
  LP_TRY(Lp, get(col, L.col, sizeof(int) * L.nnz));
  LP_TRY(Lp, get(val, L.a32, sizeof(float) * L.nnz));
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  return mark_done(Lp, c);
}

// z = M(r), the preconditioner of fcg_fcg_learned (FP32 vectors, host or device).
extern "C" int fcg_lp_precondition(fcg_learned *Lp, fcg_context *c, const float *r, float *z) {
  int rc = ml_ready(Lp, c);
  if (rc) return rc;
  if (!r || !z) return lp_fail(Lp, FCG_ERR_ARG, "NULL r or z");
  if ((rc = ensure_workspace(Lp, c, false))) return rc;
  float *dr, *dz;
  bool hr, hz;
  if ((rc = stage_f32(Lp, c, r, 4, true, &dr, &hr))) return rc;
  if ((rc = stage_f32(Lp, c, z, 5, false, &dz, &hz))) return rc;
  enqueue_preconditioner(Lp, c, c->stream, dr, dz, nullptr, Lp->scal.as<unsigned>() + 17, nullptr);
  LP_TRY(Lp, cudaGetLastError());
  if ((rc = stage_out(c, z, dz, sizeof(float) * c->n, hz)))
    return lp_fail(Lp, rc, fcg_last_error(c));
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  if ((rc = hex_status(Lp, c))) return rc;
  return mark_done(Lp, c);
}

// out = z + alpha P V(P^T (r - Ahat z)), the coarse-grid correction alone.
extern "C" int fcg_lp_coarse_correct(fcg_learned *Lp, fcg_context *c, const float *r,
                                     const float *z, float *out) {
  int rc = ml_ready(Lp, c);
  if (rc) return rc;
  if (!r || !z || !out) return lp_fail(Lp, FCG_ERR_ARG, "NULL r, z or out");
  float *dr, *dz, *dout;
  bool hr, hz, ho;
  if ((rc = stage_f32(Lp, c, r, 4, true, &dr, &hr))) return rc;
  if ((rc = stage_f32(Lp, c, z, 5, true, &dz, &hz))) return rc;
  if ((rc = stage_f32(Lp, c, out, 6, false, &dout, &ho))) return rc;
  LP_TRY(Lp, cudaMemcpyAsync(dout, dz, sizeof(float) * c->n, cudaMemcpyDeviceToDevice, c->stream));
  fcg::ml::enqueue_correction(*ml_for(Lp, c), c, Lp->mlo, c->stream, dr, dout, nullptr);
  LP_TRY(Lp, cudaGetLastError());
  if ((rc = stage_out(c, out, dout, sizeof(float) * c->n, ho)))
    return lp_fail(Lp, rc, fcg_last_error(c));
  LP_TRY(Lp, cudaStreamSynchronize(c->stream));
  return mark_done(Lp, c);
}
