// Coarse-grid correction of the learned FCG (a V-cycle over the aggregation hierarchy
// of aggregation.cpp), device side.
//
// The flexible CG of learned.cu preconditions with z = N(r), the network, and then
//   z += P V(P^T (r - Ahat z)),
// where P is the first level's prolongation and V a V-cycle on the levels below:
// `sweeps` damped Jacobi sweeps before and after each level's own correction and a dense
// inverse at the coarsest level.  By default the first P is smoothed,
// P = (I - omega D^-1 Ahat) P_tent (smoothed aggregation); the deeper levels, and the
// first one with `smoothed` off, use the piecewise-constant P_tent with every correction
// scaled by alpha.  Everything runs in FP32 on the Jacobi-scaled matrix
// Ahat = D^-1/2 A D^-1/2.  The level matrices P^T A P are recomputed from the current
// matrix on every solve, summed in FP32 in a fixed order: one warp per coarse row, its
// lanes holding the coarse entries and scanning the contributions in order (FP64 sums
// would run at GB300's low FP64 rate).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "coarse.h"
#include "krylov_common.cuh"
#include "launch.h"

namespace fcg {
namespace ml {
namespace {

constexpr int kDenseThreads = 1024;
constexpr int kDenseMaxRows = 160;  // 2 n^2 floats fit the shared memory of a block

__device__ __forceinline__ bool stopped(const int *done) { return done && __ldcg(done); }

// Values a of the coarse rows from the parent matrix (pptr, pcol, pval), summed in FP32
// in the fixed order; dinv = 1 / diagonal (0 if not positive).
__global__ void __launch_bounds__(kTPB)
    k_ml_galerkin(int nc, const int *__restrict__ cptr, const int *__restrict__ ccol,
                  const int *__restrict__ mptr, const int *__restrict__ mem,
                  const int *__restrict__ pptr, const int *__restrict__ pcol,
                  const float *__restrict__ pval, const int *__restrict__ agg,
                  float *__restrict__ a, float *__restrict__ dinv) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long I = warp; I < nc; I += nwarps) {
    const int cb = cptr[I], ce = cptr[I + 1];
    const int mb = mptr[I], me = mptr[I + 1];
    for (int sb = cb; sb < ce; sb += 32) {
      const int my = sb + lane;
      const int mycol = my < ce ? ccol[my] : -1;
      float acc = 0.f;
      for (int m = mb; m < me; ++m) {
        const int i = mem[m];
        const int kb0 = pptr[i], ke = pptr[i + 1];
        for (int kb = kb0; kb < ke; kb += 32) {
          const int k = kb + lane;
          int J = -1;
          float v = 0.f;
          if (k < ke) {
            v = pval[k];
            J = agg[pcol[k]];
          }
          const int cnt = min(32, ke - kb);
          for (int e = 0; e < cnt; ++e) {
            const int Je = __shfl_sync(0xffffffffu, J, e);
            const float ve = __shfl_sync(0xffffffffu, v, e);
            if (Je == mycol) acc = __fadd_rn(acc, ve);
          }
        }
      }
      if (my < ce) {
        a[my] = acc;
        if (mycol == (int)I) dinv[I] = acc > 0.f ? 1.f / acc : 0.f;
      }
    }
  }
}

// Level 1 from the fine matrix in the context's sliced layout (the FP32 scaled values
// Ahat `val`, slot -> CSR position `src`, pads skipped).  A row's slots hold its entries
// in column order, so the sums run in the order of k_ml_galerkin.
// When every member row has at most 8 slots, four member rows are loaded per round
// (lanes 8g..8g+7 hold member g's slots) and the lanes of the coarse entries then scan
// the 32 loaded entries in lane order -- member by member, slot by slot: the same order.
__device__ __forceinline__ void g0_entry(const SellView &sv, int n, const float *val,
                                         const int *agg, int i, int j, int &J, float &v) {
  J = -1;
  v = 0.f;
  const int slice = i >> 5, rl = i & 31;
  const int w = sv.width[slice];
  if (j >= w) return;
  const long long pos = sv.ptr[slice] + rl + 32LL * j;
  if (sv.src[pos] < 0) return;
  const int op = sv.offp[slice];
  int c = sv.kind[slice] == 0 ? i + sv.off[op + j] : sv.off[op + 32 * j + rl];
  c = c < 0 ? 0 : (c >= n ? n - 1 : c);
  v = val[pos];
  J = agg[c];
}

__global__ void __launch_bounds__(kTPB)
    k_ml_galerkin0(int nc, const int *__restrict__ cptr, const int *__restrict__ ccol,
                   const int *__restrict__ mptr, const int *__restrict__ mem, SellView sv, int n,
                   const float *__restrict__ val, const int *__restrict__ agg,
                   float *__restrict__ a, float *__restrict__ dinv) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long I = warp; I < nc; I += nwarps) {
    const int cb = cptr[I], ce = cptr[I + 1];
    const int mb = mptr[I], me = mptr[I + 1];
    int wide = 0;  // a member row wider than 8 slots
    for (int m = mb + lane; m < me; m += 32) wide |= sv.width[mem[m] >> 5] > 8;
    const bool grouped = !__any_sync(0xffffffffu, wide);
    for (int sb = cb; sb < ce; sb += 32) {
      const int my = sb + lane;
      const int mycol = my < ce ? ccol[my] : -1;
      float acc = 0.f;
      if (grouped) {
        const int g = lane >> 3, j = lane & 7;
        for (int m0 = mb; m0 < me; m0 += 4) {
          int J = -1;
          float v = 0.f;
          if (m0 + g < me) g0_entry(sv, n, val, agg, mem[m0 + g], j, J, v);
          const int cnt = min(4, me - m0) * 8;
          for (int e = 0; e < cnt; ++e) {
            const int Je = __shfl_sync(0xffffffffu, J, e);
            const float ve = __shfl_sync(0xffffffffu, v, e);
            if (Je == mycol) acc = __fadd_rn(acc, ve);
          }
        }
      } else {
        for (int m = mb; m < me; ++m) {
          const int i = mem[m];
          const int w = sv.width[i >> 5];
          for (int jb = 0; jb < w; jb += 32) {
            int J;
            float v;
            g0_entry(sv, n, val, agg, i, jb + lane, J, v);
            const int cnt = min(32, w - jb);
            for (int e = 0; e < cnt; ++e) {
              const int Je = __shfl_sync(0xffffffffu, J, e);
              const float ve = __shfl_sync(0xffffffffu, v, e);
              if (Je == mycol) acc = __fadd_rn(acc, ve);
            }
          }
        }
      }
      if (my < ce) {
        a[my] = acc;
        if (mycol == (int)I) dinv[I] = acc > 0.f ? 1.f / acc : 0.f;
      }
    }
  }
}

// Gauss-Jordan inverse of the (small, symmetric positive definite) coarsest matrix in
// FP32, one block, the matrix and its inverse in shared memory (2 n^2 floats).  M
// receives the inverse, row-major.  A pivot below 1e-5 of the largest diagonal entry
// drops its row (a zero row and column of M), which keeps a singular coarsest matrix (no
// Dirichlet boundary) from producing infinities.
__global__ void __launch_bounds__(kDenseThreads)
    k_ml_dense_inv(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                   const float *__restrict__ a, float *__restrict__ M) {
  extern __shared__ float dsm[];
  float *W = dsm, *V = dsm + n * n;
  __shared__ float fcol[kDenseMaxRows];
  __shared__ float pinv, tiny;
  const int tid = threadIdx.x, bs = blockDim.x;
  const int nn = n * n;
  for (int i = tid; i < nn; i += bs) {
    W[i] = 0.f;
    V[i] = (i / n == i % n) ? 1.f : 0.f;
  }
  __syncthreads();
  for (int r = tid; r < n; r += bs)
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) W[r * n + col[k]] = a[k];
  __syncthreads();
  if (tid == 0) {
    float dmax = 0.f;
    for (int r = 0; r < n; ++r) dmax = fmaxf(dmax, W[r * n + r]);
    tiny = 1e-5f * dmax;
  }
  __syncthreads();
  for (int p = 0; p < n; ++p) {
    if (tid == 0) {
      const float piv = W[p * n + p];
      pinv = piv > tiny ? 1.f / piv : 0.f;
    }
    __syncthreads();
    for (int c = tid; c < n; c += bs) {
      W[p * n + c] *= pinv;
      V[p * n + c] *= pinv;
    }
    for (int r = tid; r < n; r += bs) fcol[r] = (r == p) ? 0.f : W[r * n + p];
    __syncthreads();
    for (int i = tid; i < nn; i += bs) {
      const int r = i / n, c = i - r * n;
      const float f = fcol[r];
      if (f != 0.f) {
        W[i] -= f * W[p * n + c];
        V[i] -= f * V[p * n + c];
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < nn; i += bs) M[i] = V[i];
}

// x = M b, one warp per row
__global__ void __launch_bounds__(kTPB)
    k_ml_dense_apply(int n, const float *__restrict__ M, const float *__restrict__ b,
                     float *__restrict__ x, const int *done) {
  if (stopped(done)) return;
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= n) return;
  float acc = 0.f;
  for (int c = lane; c < n; c += 32) acc += M[(long long)r * n + c] * b[c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) x[r] = acc;
}

// Row products of the coarse levels: LPR lanes per row (32 / LPR rows per warp), each
// lane summing every LPR-th entry, then a shuffle sum.  Four lanes on the sparse levels;
// eight on the first level of the smoothed hierarchy (about 45 entries per row), so that
// a row's lanes read whole 32-byte sectors of values and columns.  Loops are warp-uniform.
template <int LPR>
__device__ __forceinline__ float row_lanes(const int *ptr, const int *col, const float *a,
                                          const float *x, int row, int n, int q) {
  float acc = 0.f;
  if (row < n)
    for (int k = ptr[row] + q; k < ptr[row + 1]; k += LPR) acc += a[k] * x[col[k]];
#pragma unroll
  for (int o = 1; o < LPR; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

// y = x + omega dinv (b - A x); x == NULL stands for x = 0
template <int LPR>
__global__ void __launch_bounds__(kTPB)
    k_ml_jacobi(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                const float *__restrict__ a, const float *__restrict__ dinv,
                const float *__restrict__ b, const float *__restrict__ x, float *__restrict__ y,
                float omega, const int *done) {
  if (stopped(done)) return;
  constexpr int RPW = 32 / LPR;  // rows per warp
  const int lane = threadIdx.x & 31, q = lane & (LPR - 1);
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = w0 * RPW; base < n; base += nw * RPW) {
    const int row = (int)base + lane / LPR;
    if (!x) {
      if (q == 0 && row < n) y[row] = omega * dinv[row] * b[row];
      continue;
    }
    const float ax = row_lanes<LPR>(ptr, col, a, x, row, n, q);
    if (q == 0 && row < n) y[row] = x[row] + omega * dinv[row] * (b[row] - ax);
  }
}

// t = b - A x
template <int LPR>
__global__ void __launch_bounds__(kTPB)
    k_ml_resid(int n, const int *__restrict__ ptr, const int *__restrict__ col,
               const float *__restrict__ a, const float *__restrict__ b,
               const float *__restrict__ x, float *__restrict__ t, const int *done) {
  if (stopped(done)) return;
  constexpr int RPW = 32 / LPR;
  const int lane = threadIdx.x & 31, q = lane & (LPR - 1);
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = w0 * RPW; base < n; base += nw * RPW) {
    const int row = (int)base + lane / LPR;
    const float ax = row_lanes<LPR>(ptr, col, a, x, row, n, q);
    if (q == 0 && row < n) t[row] = b[row] - ax;
  }
}

// bc[I] = sum over the member rows i of I of t_i
__global__ void __launch_bounds__(kTPB)
    k_ml_restrict(int nc, const int *__restrict__ mptr, const int *__restrict__ mem,
                  const float *__restrict__ t, float *__restrict__ bc, const int *done) {
  if (stopped(done)) return;
  FCG_GRID_STRIDE(I, nc) {
    float acc = 0.f;
    for (int m = mptr[I]; m < mptr[I + 1]; ++m) acc += t[mem[m]];
    bc[I] = acc;
  }
}

// x_i += alpha xc[agg_i]
__global__ void __launch_bounds__(kTPB)
    k_ml_prolong(int n, const int *__restrict__ agg, const float *__restrict__ xc,
                 float *__restrict__ x, float alpha, const int *done) {
  if (stopped(done)) return;
  FCG_GRID_STRIDE(i, n) x[i] += alpha * xc[agg[i]];
}

// fine level (sliced matrix, unit diagonal): t = r - Ahat z
__global__ void __launch_bounds__(kTPB, 6)
    k_ml_resid0(SellView s, int n, const float *__restrict__ val, const float *__restrict__ r,
                const float *__restrict__ z, float *__restrict__ t, const int *done) {
  if (stopped(done)) return;
  FCG_SLICE_LOOP(slice, lane, s) {
    const float az = sell_row(s, n, val, z, slice, lane);
    const int row = slice * 32 + lane;
    if (row < n) t[row] = r[row] - az;
  }
}

// fine level Jacobi sweep: zout = zin + omega (r - Ahat zin); zin == NULL: zout = omega r
__global__ void __launch_bounds__(kTPB, 6)
    k_ml_jac0(SellView s, int n, const float *__restrict__ val, const float *__restrict__ r,
              const float *__restrict__ zin, float *__restrict__ zout, float omega,
              const int *done) {
  if (stopped(done)) return;
  FCG_SLICE_LOOP(slice, lane, s) {
    const int row = slice * 32 + lane;
    if (!zin) {
      if (row < n) zout[row] = omega * r[row];
      continue;
    }
    const float az = sell_row(s, n, val, zin, slice, lane);
    if (row < n) zout[row] = zin[row] + omega * (r[row] - az);
  }
}

__global__ void __launch_bounds__(kTPB)
    k_ml_copy(int n, const float *__restrict__ a, float *__restrict__ b, const int *done) {
  if (stopped(done)) return;
  FCG_GRID_STRIDE(i, n) b[i] = a[i];
}

// ---- smoothed first level: P = (I - omega D^-1 Ahat) P_tent, A P, P^T A P -----------
// Column and value of slot j of fine row i in the sliced layout (c = -1 for a pad).
__device__ __forceinline__ void sell_entry(const SellView &sv, int n, const float *val, int i,
                                           int j, int &c, float &v) {
  const int slice = i >> 5, rl = i & 31;
  const long long pos = sv.ptr[slice] + rl + 32LL * j;
  c = -1;
  v = 0.f;
  if (sv.src[pos] < 0) return;
  const int op = sv.offp[slice];
  int cc = sv.kind[slice] == 0 ? i + sv.off[op + j] : sv.off[op + 32 * j + rl];
  c = cc < 0 ? 0 : (cc >= n ? n - 1 : cc);
  v = val[pos];
}

// P row i: 1 at the own aggregate, then minus (omega / a_ii) a_ik for the row's entries
// in column order, each product and difference rounded to FP32 on its own
__global__ void __launch_bounds__(kTPB)
    k_sa_p(SellView sv, int n, const float *__restrict__ val, const int *__restrict__ agg,
           const int *__restrict__ p_ptr, const int *__restrict__ p_col, float omega,
           float *__restrict__ p_val) {
  FCG_GRID_STRIDE(i, n) {
    const int w = sv.width[i >> 5];
    float d = 0.f;
    for (int j = 0; j < w; ++j) {
      int c;
      float v;
      sell_entry(sv, n, val, (int)i, j, c, v);
      if (c == i) d = v;
    }
    const float wgt = d > 0.f ? __fdiv_rn(omega, d) : 0.f;
    const int pb = p_ptr[i], pe = p_ptr[i + 1], own = agg[i];
    for (int p = pb; p < pe; ++p) p_val[p] = p_col[p] == own ? 1.f : 0.f;
    for (int j = 0; j < w; ++j) {
      int c;
      float v;
      sell_entry(sv, n, val, (int)i, j, c, v);
      if (c < 0) continue;
      const int J = agg[c];
      int p = pb;
      while (p < pe - 1 && p_col[p] != J) ++p;
      p_val[p] = __fsub_rn(p_val[p], __fmul_rn(wgt, v));
    }
  }
}

// (A P) row i: for the row's entries in column order, a_ik P_k in P_k's column order
__global__ void __launch_bounds__(kTPB)
    k_sa_ap(SellView sv, int n, const float *__restrict__ val, const int *__restrict__ p_ptr,
            const int *__restrict__ p_col, const float *__restrict__ p_val,
            const int *__restrict__ ap_ptr, const int *__restrict__ ap_col,
            float *__restrict__ ap_val) {
  FCG_GRID_STRIDE(i, n) {
    const int w = sv.width[i >> 5];
    const int qb = ap_ptr[i], qe = ap_ptr[i + 1];
    for (int q = qb; q < qe; ++q) ap_val[q] = 0.f;
    for (int j = 0; j < w; ++j) {
      int c;
      float v;
      sell_entry(sv, n, val, (int)i, j, c, v);
      if (c < 0) continue;
      for (int p = p_ptr[c]; p < p_ptr[c + 1]; ++p) {
        const int J = p_col[p];
        int lo = qb, hi = qe - 1;  // the row's columns ascend; J is among them
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (ap_col[mid] < J) lo = mid + 1;
          else hi = mid;
        }
        ap_val[lo] = __fadd_rn(ap_val[lo], __fmul_rn(v, p_val[p]));
      }
    }
  }
}

// P^T (A P): one warp per coarse row, two coarse entries per lane (entry e of a 64-entry
// chunk of the row belongs to lane e mod 32); the rows holding the aggregate in ascending
// order, each row's (A P) entries in column order.  The contributions come 32 at a time,
// one per lane.  Each lane finds its entry by binary search in the row's columns, the
// lanes with the same entry are grouped, and the entry's owner adds the group's values in
// lane order: the same FP32 sums in the same order as adding every contribution in turn.
constexpr int kA1Warps = kTPB / 32;

__global__ void __launch_bounds__(kTPB, 4)
    k_sa_a1(int nc, const int *__restrict__ cptr, const int *__restrict__ ccol,
            const int *__restrict__ t_ptr, const int *__restrict__ t_row,
            const float *__restrict__ pt_val,
            const int *__restrict__ ap_ptr, const int *__restrict__ ap_col,
            const float *__restrict__ ap_val, float *__restrict__ a, float *__restrict__ dinv) {
  __shared__ unsigned gmask[kA1Warps][64];  // lanes holding a contribution to each entry
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned *gm = gmask[wib];
  gm[lane] = 0u;
  gm[lane + 32] = 0u;
  __syncwarp();
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long I = warp; I < nc; I += nwarps) {
    const int cb = cptr[I], ce = cptr[I + 1];
    const int mb = t_ptr[I], me = t_ptr[I + 1];
    for (int sb = cb; sb < ce; sb += 64) {  // two coarse entries per lane
      const int my0 = sb + lane, my1 = sb + 32 + lane;
      const int send = min(sb + 64, ce);
      float acc0 = 0.f, acc1 = 0.f;
      // up to 32 supporting rows at a time, one per lane; their (A P) entries are
      // numbered consecutively (row by row, entries in column order) and taken in full
      // chunks of 32, each lane finding its row by a binary search over the lanes'
      // inclusive prefix sums
      for (int gb = mb; gb < me; gb += 32) {
        const int m = gb + lane;
        int st = 0, len = 0;
        float p = 0.f;
        if (m < me) {
          const int i = t_row[m];
          p = pt_val[m];
          st = ap_ptr[i];
          len = ap_ptr[i + 1] - st;
        }
        int inc = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, inc, o);
          if (lane >= o) inc += t;
        }
        const int total = __shfl_sync(0xffffffffu, inc, 31);
        for (int fb = 0; fb < total; fb += 32) {
          const int f = fb + lane;
          int lo = 0;  // lanes whose rows end at or before entry f
#pragma unroll
          for (int step = 16; step > 0; step >>= 1) {
            const int iv = __shfl_sync(0xffffffffu, inc, lo + step - 1);
            if (iv <= f) lo += step;
          }
          const int src = lo & 31;
          const int ost = __shfl_sync(0xffffffffu, st, src);
          const int oinc = __shfl_sync(0xffffffffu, inc, src);
          const int olen = __shfl_sync(0xffffffffu, len, src);
          const float op = __shfl_sync(0xffffffffu, p, src);
          int e = -1;  // entry of this chunk that the contribution adds to
          float v = 0.f;
          if (f < total) {
            const int q = ost + (f - (oinc - olen));
            const int J = ap_col[q];
            v = __fmul_rn(op, ap_val[q]);
            int l = sb, h = send - 1;
            while (l < h) {
              const int mid = (l + h) >> 1;
              if (ccol[mid] < J) l = mid + 1;
              else h = mid;
            }
            if (l < send && ccol[l] == J) e = l - sb;
          }
          const unsigned grp = __match_any_sync(0xffffffffu, e);
          if (e >= 0 && lane == __ffs(grp) - 1) gm[e] = grp;
          __syncwarp();
          unsigned g0 = gm[lane], g1 = gm[lane + 32];
          while (__any_sync(0xffffffffu, (g0 | g1) != 0u)) {
            const int s0 = g0 ? __ffs(g0) - 1 : lane, s1 = g1 ? __ffs(g1) - 1 : lane;
            const float v0 = __shfl_sync(0xffffffffu, v, s0);
            const float v1 = __shfl_sync(0xffffffffu, v, s1);
            if (g0) {
              acc0 = __fadd_rn(acc0, v0);
              g0 &= g0 - 1;
            }
            if (g1) {
              acc1 = __fadd_rn(acc1, v1);
              g1 &= g1 - 1;
            }
          }
          gm[lane] = 0u;
          gm[lane + 32] = 0u;
          __syncwarp();
        }
      }
      if (my0 < ce) {
        const int c0 = ccol[my0];
        a[my0] = acc0;
        if (c0 == (int)I) dinv[I] = acc0 > 0.f ? 1.f / acc0 : 0.f;
      }
      if (my1 < ce) {
        const int c1 = ccol[my1];
        a[my1] = acc1;
        if (c1 == (int)I) dinv[I] = acc1 > 0.f ? 1.f / acc1 : 0.f;
      }
    }
  }
}

// P's values in the order of its transpose lists (once per solve): pt_val[m] = p_val[t_pos[m]]
__global__ void __launch_bounds__(kTPB)
    k_sa_pt(long long nnz, const int *__restrict__ t_pos, const float *__restrict__ p_val,
            float *__restrict__ pt_val) {
  FCG_GRID_STRIDE(m, nnz) pt_val[m] = p_val[t_pos[m]];
}

// b1 = P^T t
__global__ void __launch_bounds__(kTPB)
    k_sa_restrict(int nc, const int *__restrict__ t_ptr, const int *__restrict__ t_row,
                  const float *__restrict__ pt_val, const float *__restrict__ t,
                  float *__restrict__ bc, const int *done) {
  if (stopped(done)) return;
  FCG_GRID_STRIDE(I, nc) {
    float acc = 0.f;
    for (int m = t_ptr[I]; m < t_ptr[I + 1]; ++m) acc += pt_val[m] * t[t_row[m]];
    bc[I] = acc;
  }
}

// z += alpha P e
__global__ void __launch_bounds__(kTPB)
    k_sa_prolong(int n, const int *__restrict__ p_ptr, const int *__restrict__ p_col,
                 const float *__restrict__ p_val, const float *__restrict__ e,
                 float *__restrict__ z, float alpha, const int *done) {
  if (stopped(done)) return;
  FCG_GRID_STRIDE(i, n) {
    float s = 0.f;
    for (int p = p_ptr[i]; p < p_ptr[i + 1]; ++p) s += p_val[p] * e[p_col[p]];
    z[i] += alpha * s;
  }
}

// One V-cycle on level k of H.lv for right-hand side lv[k].b; returns the vector holding
// the result (lv[k].x or lv[k].y).
float *enqueue_vcycle(Hierarchy &H, int num_sms, const Options &o, cudaStream_t st, int k,
                      const int *done) {
  DevLevel &L = H.lv[k];
  const float om = (float)o.omega, al = (float)o.alpha;
  const int g = grid_for(L.n, num_sms, 8);
  // eight lanes per row on a level of 24 or more entries per row, else four
  const bool wide = L.nnz >= 24LL * L.n;
  const int g4 = grid_for((wide ? 8LL : 4LL) * L.n, num_sms, 8);
  auto jacobi = wide ? k_ml_jacobi<8> : k_ml_jacobi<4>;
  auto resid = wide ? k_ml_resid<8> : k_ml_resid<4>;
  const bool last = k + 1 == (int)H.lv.size();
  if (last && H.has_dense) {
    const int blocks = (L.n * 32 + kTPB - 1) / kTPB;
    k_ml_dense_apply<<<blocks, kTPB, 0, st>>>(L.n, H.dense.as<float>(), L.b, L.x, done);
    return L.x;
  }
  float *cur = L.x, *oth = L.y;
  jacobi<<<g4, kTPB, 0, st>>>(L.n, L.ptr, L.col, L.a32, L.dinv, L.b, nullptr, cur, om, done);
  const int pre = last ? 2 * o.sweeps + 2 : o.sweeps;  // coarsest without a dense inverse
  for (int s = 1; s < pre; ++s) {
    jacobi<<<g4, kTPB, 0, st>>>(L.n, L.ptr, L.col, L.a32, L.dinv, L.b, cur, oth, om, done);
    std::swap(cur, oth);
  }
  if (last) return cur;
  DevLevel &Lc = H.lv[k + 1];
  resid<<<g4, kTPB, 0, st>>>(L.n, L.ptr, L.col, L.a32, L.b, cur, oth, done);
  k_ml_restrict<<<grid_for(Lc.n, num_sms, 8), kTPB, 0, st>>>(Lc.n, Lc.mptr, Lc.mem, oth, Lc.b,
                                                            done);
  const float *e = enqueue_vcycle(H, num_sms, o, st, k + 1, done);
  k_ml_prolong<<<g, kTPB, 0, st>>>(L.n, Lc.agg, e, cur, al, done);
  for (int s = 0; s < o.sweeps; ++s) {
    jacobi<<<g4, kTPB, 0, st>>>(L.n, L.ptr, L.col, L.a32, L.dinv, L.b, cur, oth, om, done);
    std::swap(cur, oth);
  }
  return cur;
}

// Restriction of the fine residual t to level 1 and prolongation of its correction e:
// the smoothed P (correction not scaled) or the aggregation (scaled by alpha).
void fine_restrict(Hierarchy &H, int num_sms, cudaStream_t st, const float *t, const int *done) {
  DevLevel &L1 = H.lv[0];
  if (H.smoothed)
    k_sa_restrict<<<grid_for(L1.n, num_sms, 8), kTPB, 0, st>>>(L1.n, H.t_ptr, H.t_row,
                                                              H.pt_val, t, L1.b, done);
  else
    k_ml_restrict<<<grid_for(L1.n, num_sms, 8), kTPB, 0, st>>>(L1.n, L1.mptr, L1.mem, t, L1.b,
                                                              done);
}

void fine_prolong(Hierarchy &H, int n, int num_sms, const Options &o, cudaStream_t st,
                  const float *e, float *z, const int *done) {
  if (H.smoothed)
    k_sa_prolong<<<grid_for(n, num_sms, 8), kTPB, 0, st>>>(n, H.p_ptr, H.p_col, H.p_val, e, z,
                                                          1.f, done);
  else
    k_ml_prolong<<<grid_for(n, num_sms, 8), kTPB, 0, st>>>(n, H.lv[0].agg, e, z, (float)o.alpha,
                                                          done);
}

template <class T>
T *carve(char *&p, size_t count) {
  T *r = (T *)p;
  p += ((count * sizeof(T) + 255) / 256) * 256;
  return r;
}

size_t pad256(size_t b) { return ((b + 255) / 256) * 256; }

}  // namespace

void Hierarchy::release() {
  for (auto &L : lv) {
    L.ints.release();
    L.vals.release();
    L.vecs.release();
  }
  lv.clear();
  dense.release();
  fine_tmp.release();
  sa_ints.release();
  sa_vals.release();
  p_nnz = ap_nnz = 0;
  has_dense = false;
  uid = 0;
}

namespace {

// The arrays of one level below the fine one, on the host or on the device.
struct LevelSrc {
  int n = 0, np = 0;  // rows, rows of the level above
  long long nnz = 0;
  const int *ptr = nullptr, *mptr = nullptr, *col = nullptr, *agg = nullptr, *mem = nullptr;
};

// The smoothed first level's patterns.
struct SmoothSrc {
  long long p_nnz = 0, ap_nnz = 0;
  const int *p_ptr = nullptr, *ap_ptr = nullptr, *p_col = nullptr, *t_row = nullptr,
            *t_pos = nullptr, *t_ptr = nullptr, *ap_col = nullptr;
};

// Allocates H's levels and copies the patterns in (kind: host or device sources).
int fill(Hierarchy &H, fcg_context *c, const Options &o, const std::vector<LevelSrc> &ls,
         const SmoothSrc *sm, cudaMemcpyKind kind, std::string &err) {
  const int n = c->n;
  cudaError_t e;
  auto cp = [&](void *dst, const void *src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, kind, c->stream);
  };
  H.lv.resize(ls.size());
  for (size_t l = 0; l < ls.size(); ++l) {
    const LevelSrc &h = ls[l];
    DevLevel &L = H.lv[l];
    const int np = h.np;
    L.n = h.n;
    L.nnz = h.nnz;
    const size_t ib = pad256(sizeof(int) * (h.n + 1)) * 2 + pad256(sizeof(int) * L.nnz) +
                      pad256(sizeof(int) * np) * 2;
    const size_t vb = pad256(sizeof(float) * L.nnz) + pad256(sizeof(float) * h.n);
    const size_t xb = 3 * pad256(sizeof(float) * h.n);
    if ((e = L.ints.ensure(ib)) || (e = L.vals.ensure(vb)) || (e = L.vecs.ensure(xb))) {
      err = std::string("hierarchy allocation: ") + cudaGetErrorString(e);
      return FCG_ERR_CUDA;
    }
    char *p = (char *)L.ints.p;
    L.ptr = carve<int>(p, h.n + 1);
    L.mptr = carve<int>(p, h.n + 1);
    L.col = carve<int>(p, L.nnz);
    L.agg = carve<int>(p, np);
    L.mem = carve<int>(p, np);
    p = (char *)L.vals.p;
    L.a32 = carve<float>(p, L.nnz);
    L.dinv = carve<float>(p, h.n);
    p = (char *)L.vecs.p;
    L.b = carve<float>(p, h.n);
    L.x = carve<float>(p, h.n);
    L.y = carve<float>(p, h.n);
    if ((e = cp(L.ptr, h.ptr, sizeof(int) * (h.n + 1))) ||
        (e = cp(L.mptr, h.mptr, sizeof(int) * (h.n + 1))) ||
        (e = cp(L.col, h.col, sizeof(int) * L.nnz)) || (e = cp(L.agg, h.agg, sizeof(int) * np)) ||
        (e = cp(L.mem, h.mem, sizeof(int) * np))) {
      err = std::string("hierarchy upload: ") + cudaGetErrorString(e);
      return FCG_ERR_CUDA;
    }
  }
  if (sm) {
    H.p_nnz = sm->p_nnz;
    H.ap_nnz = sm->ap_nnz;
    const int n1 = ls[0].n;
    const size_t ib = pad256(sizeof(int) * (n + 1)) * 2 + pad256(sizeof(int) * H.p_nnz) * 3 +
                      pad256(sizeof(int) * (n1 + 1)) + pad256(sizeof(int) * H.ap_nnz);
    const size_t vb = 2 * pad256(sizeof(float) * H.p_nnz) + pad256(sizeof(float) * H.ap_nnz);
    if ((e = H.sa_ints.ensure(ib)) || (e = H.sa_vals.ensure(vb))) {
      err = std::string("hierarchy allocation: ") + cudaGetErrorString(e);
      return FCG_ERR_CUDA;
    }
    char *p = (char *)H.sa_ints.p;
    H.p_ptr = carve<int>(p, n + 1);
    H.ap_ptr = carve<int>(p, n + 1);
    H.p_col = carve<int>(p, H.p_nnz);
    H.t_row = carve<int>(p, H.p_nnz);
    H.t_pos = carve<int>(p, H.p_nnz);
    H.t_ptr = carve<int>(p, n1 + 1);
    H.ap_col = carve<int>(p, H.ap_nnz);
    p = (char *)H.sa_vals.p;
    H.p_val = carve<float>(p, H.p_nnz);
    H.pt_val = carve<float>(p, H.p_nnz);
    H.ap_val = carve<float>(p, H.ap_nnz);
    if ((e = cp(H.p_ptr, sm->p_ptr, sizeof(int) * (n + 1))) ||
        (e = cp(H.ap_ptr, sm->ap_ptr, sizeof(int) * (n + 1))) ||
        (e = cp(H.p_col, sm->p_col, sizeof(int) * H.p_nnz)) ||
        (e = cp(H.t_row, sm->t_row, sizeof(int) * H.p_nnz)) ||
        (e = cp(H.t_pos, sm->t_pos, sizeof(int) * H.p_nnz)) ||
        (e = cp(H.t_ptr, sm->t_ptr, sizeof(int) * (n1 + 1))) ||
        (e = cp(H.ap_col, sm->ap_col, sizeof(int) * H.ap_nnz))) {
      err = std::string("hierarchy upload: ") + cudaGetErrorString(e);
      return FCG_ERR_CUDA;
    }
  }
  if ((e = cudaStreamSynchronize(c->stream))) {
    err = std::string("hierarchy upload: ") + cudaGetErrorString(e);
    return FCG_ERR_CUDA;
  }
  (void)o;
  return FCG_OK;
}

// The levels built on the device (aggregation_gpu.cu) from the scaled fine matrix.
// Returns FCG_OK, FCG_ERR_CUDA, or another code when the host should build instead.
int build_on_device(Hierarchy &H, fcg_context *c, const Options &o, int dmax, std::string &err) {
  const int n = c->n;
  const long long nnz = c->nnz;
  DevMat fine;
  cudaError_t e;
  if ((e = fine.val.ensure(sizeof(double) * (nnz > 0 ? nnz : 1)))) {
    err = std::string("hierarchy allocation: ") + cudaGetErrorString(e);
    return FCG_ERR_CUDA;
  }
  fine_values(c, sliced64(c), c->sv.src, c->sell_len, scale64(c), fine.val.as<double>());
  const DevCsr fv{n, nnz, c->mv.ioffset, c->mv.ja, fine.val.as<double>()};
  std::vector<DevBuiltLevel> dl;
  int rc = build_levels_device(c, fv, std::max(2, o.max_levels), dmax, H.passes,
                               o.smoothed ? o.omega : 0.0, dl, err);
  fine.release();
  if (rc == FCG_OK) {
    std::vector<LevelSrc> ls(dl.size());
    for (size_t l = 0; l < dl.size(); ++l) {
      const DevBuiltLevel &d = dl[l];
      ls[l] = {d.n, d.np, d.A.nnz, d.A.ptr.as<int>(), d.mptr.as<int>(), d.A.col.as<int>(),
               d.agg.as<int>(), d.mem.as<int>()};
    }
    SmoothSrc sm;
    const bool smooth = !dl.empty() && o.smoothed;
    if (smooth) {
      const DevBuiltLevel &d = dl[0];
      sm = {d.p_nnz, d.ap_nnz, d.p_ptr.as<int>(), d.ap_ptr.as<int>(), d.p_col.as<int>(),
            d.t_row.as<int>(), d.t_pos.as<int>(), d.t_ptr.as<int>(), d.ap_col.as<int>()};
    }
    rc = fill(H, c, o, ls, smooth ? &sm : nullptr, cudaMemcpyDeviceToDevice, err);
  }
  for (auto &d : dl) d.release();
  return rc;
}

int build_on_host(Hierarchy &H, fcg_context *c, const Options &o, int dmax, std::string &err) {
  const int n = c->n;
  const long long nnz = c->nnz, len = c->sell_len;
  HostCsr fine;
  fine.n = n;
  fine.ptr.resize(n + 1);
  fine.col.resize(nnz);
  fine.val.resize(nnz);
  std::vector<double> s(n), sval(len);
  std::vector<int> src(len);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(fine.ptr.data(), c->mv.ioffset, sizeof(int) * (n + 1),
                           cudaMemcpyDeviceToHost, c->stream)) ||
      (e = cudaMemcpyAsync(fine.col.data(), c->mv.ja, sizeof(int) * nnz, cudaMemcpyDeviceToHost,
                           c->stream)) ||
      (e = cudaMemcpyAsync(sval.data(), sliced64(c), sizeof(double) * len, cudaMemcpyDeviceToHost,
                           c->stream)) ||
      (e = cudaMemcpyAsync(src.data(), c->sv.src, sizeof(int) * len, cudaMemcpyDeviceToHost,
                           c->stream)) ||
      (e = cudaMemcpyAsync(s.data(), scale64(c), sizeof(double) * n, cudaMemcpyDeviceToHost,
                           c->stream)) ||
      (e = cudaStreamSynchronize(c->stream))) {
    err = std::string("hierarchy download: ") + cudaGetErrorString(e);
    return FCG_ERR_CUDA;
  }
  for (long long p = 0; p < len; ++p)
    if (src[p] >= 0) fine.val[src[p]] = sval[p];
  sval = std::vector<double>();
  src = std::vector<int>();
  for (int i = 0; i < n; ++i)
    for (int k = fine.ptr[i]; k < fine.ptr[i + 1]; ++k)
      fine.val[k] = (fine.val[k] * s[i]) * s[fine.col[k]];
  std::vector<HostLevel> hl;
  build_levels(fine, std::max(2, o.max_levels), dmax, H.passes, hl, o.smoothed ? o.omega : 0.0);
  fine = HostCsr();
  std::vector<LevelSrc> ls(hl.size());
  int np = n;
  for (size_t l = 0; l < hl.size(); ++l) {
    const HostLevel &h = hl[l];
    ls[l] = {h.n, np, (long long)h.A.col.size(), h.A.ptr.data(), h.mptr.data(), h.A.col.data(),
             h.agg.data(), h.mem.data()};
    np = h.n;
  }
  SmoothSrc sm;
  const bool smooth = !hl.empty() && o.smoothed;
  if (smooth) {
    const HostLevel &h = hl[0];
    sm = {(long long)h.p_col.size(), (long long)h.ap_col.size(), h.p_ptr.data(),
          h.ap_ptr.data(), h.p_col.data(), h.t_row.data(), h.t_pos.data(), h.t_ptr.data(),
          h.ap_col.data()};
  }
  return fill(H, c, o, ls, smooth ? &sm : nullptr, cudaMemcpyHostToDevice, err);
}

}  // namespace

int build(Hierarchy &H, fcg_context *c, const Options &o, std::string &err) {
  const auto t0 = std::chrono::steady_clock::now();
  H.release();
  const int n = c->n;
  const int dmax = std::min(std::max(o.dense_max, 1), kDenseMaxRows);
  // FCG_AGG=host builds the levels on the host (aggregation.cpp); the device build gives
  // the same arrays and falls back to the host when a matching wait gives up or a coarse
  // row outgrows its accumulation table
  const char *where = std::getenv("FCG_AGG");
  int rc = FCG_ERR_UNSUPPORTED;
  H.built_on_device = false;
  if (!(where && std::string(where) == "host")) {
    rc = build_on_device(H, c, o, dmax, err);
    if (rc == FCG_ERR_CUDA) {
      H.release();
      return rc;
    }
    H.built_on_device = rc == FCG_OK;
  }
  if (rc != FCG_OK) {
    H.release();
    err.clear();
    if ((rc = build_on_host(H, c, o, dmax, err))) {
      H.release();
      return rc;
    }
  }
  cudaError_t e;
  H.smoothed = o.smoothed;
  H.sa_omega = o.omega;
  if (!H.lv.empty()) {
    const int nl = H.lv.back().n;
    H.has_dense = nl <= dmax;
    if (H.has_dense) {
      if ((e = H.dense.ensure(sizeof(float) * nl * nl))) {
        err = std::string("hierarchy allocation: ") + cudaGetErrorString(e);
        H.release();
        return FCG_ERR_CUDA;
      }
    }
  }
  if ((e = H.fine_tmp.ensure(2 * pad256(sizeof(float) * n)))) {
    err = std::string("hierarchy allocation: ") + cudaGetErrorString(e);
    H.release();
    return FCG_ERR_CUDA;
  }
  H.uid = c->uid;
  H.gen = c->bind_gen;
  H.n0 = n;
  H.max_levels = o.max_levels;
  H.dense_max = o.dense_max;
  H.build_id++;
  H.setup_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return FCG_OK;
}

int values(Hierarchy &H, fcg_context *c, cudaStream_t st) {
  const int ns = c->num_sms;
  for (size_t l = 0; l < H.lv.size(); ++l) {
    DevLevel &L = H.lv[l];
    const int g = grid_for(32LL * L.n, ns, 8);
    if (l == 0 && H.smoothed) {
      const int gn = grid_for(c->n, ns, 8);
      k_sa_p<<<gn, kTPB, 0, st>>>(c->sv, c->n, scaled32(c), L.agg, H.p_ptr, H.p_col,
                                  (float)H.sa_omega, H.p_val);
      k_sa_ap<<<gn, kTPB, 0, st>>>(c->sv, c->n, scaled32(c), H.p_ptr, H.p_col, H.p_val, H.ap_ptr,
                                   H.ap_col, H.ap_val);
      k_sa_pt<<<grid_for(H.p_nnz, ns, 8), kTPB, 0, st>>>(H.p_nnz, H.t_pos, H.p_val, H.pt_val);
      k_sa_a1<<<g, kTPB, 0, st>>>(L.n, L.ptr, L.col, H.t_ptr, H.t_row, H.pt_val, H.ap_ptr,
                                  H.ap_col, H.ap_val, L.a32, L.dinv);
    } else if (l == 0) {
      k_ml_galerkin0<<<g, kTPB, 0, st>>>(L.n, L.ptr, L.col, L.mptr, L.mem, c->sv, c->n,
                                         scaled32(c), L.agg, L.a32, L.dinv);
    } else {
      const DevLevel &P = H.lv[l - 1];
      k_ml_galerkin<<<g, kTPB, 0, st>>>(L.n, L.ptr, L.col, L.mptr, L.mem, P.ptr, P.col, P.a32,
                                        L.agg, L.a32, L.dinv);
    }
  }
  if (H.has_dense) {
    const DevLevel &L = H.lv.back();
    const size_t smem = sizeof(float) * 2 * L.n * L.n;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_ml_dense_inv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return FCG_ERR_CUDA;
    k_ml_dense_inv<<<1, kDenseThreads, smem, st>>>(L.n, L.ptr, L.col, L.a32,
                                                   H.dense.as<float>());
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FCG_OK : FCG_ERR_CUDA;
}

void enqueue_correction(Hierarchy &H, fcg_context *c, const Options &o, cudaStream_t st,
                        const float *r, float *z, const int *done) {
  if (H.lv.empty()) return;
  const int n = c->n, ns = c->num_sms;
  float *t = H.fine_tmp.as<float>();
  k_ml_resid0<<<grid_for(n, ns, 6), kTPB, 0, st>>>(c->sv, n, scaled32(c), r, z, t, done);
  fine_restrict(H, ns, st, t, done);
  const float *e = enqueue_vcycle(H, ns, o, st, 0, done);
  fine_prolong(H, n, ns, o, st, e, z, done);
}

void enqueue_jacobi_cycle(Hierarchy &H, fcg_context *c, const Options &o, cudaStream_t st,
                          const float *r, float *z, const int *done) {
  const int n = c->n, ns = c->num_sms;
  const float om = (float)o.omega;
  float *t = H.fine_tmp.as<float>();
  float *u = t + pad256(sizeof(float) * n) / sizeof(float);
  const int gs = grid_for(n, ns, 6);
  float *cur = z, *oth = u;
  k_ml_jac0<<<gs, kTPB, 0, st>>>(c->sv, n, scaled32(c), r, nullptr, cur, om, done);
  for (int s = 1; s < o.sweeps; ++s) {
    k_ml_jac0<<<gs, kTPB, 0, st>>>(c->sv, n, scaled32(c), r, cur, oth, om, done);
    std::swap(cur, oth);
  }
  if (!H.lv.empty()) {
    k_ml_resid0<<<gs, kTPB, 0, st>>>(c->sv, n, scaled32(c), r, cur, t, done);
    fine_restrict(H, ns, st, t, done);
    const float *e = enqueue_vcycle(H, ns, o, st, 0, done);
    fine_prolong(H, n, ns, o, st, e, cur, done);
  }
  for (int s = 0; s < o.sweeps; ++s) {
    k_ml_jac0<<<gs, kTPB, 0, st>>>(c->sv, n, scaled32(c), r, cur, oth, om, done);
    std::swap(cur, oth);
  }
  if (cur != z) k_ml_copy<<<grid_for(n, ns, 8), kTPB, 0, st>>>(n, cur, z, done);
}

}  // namespace ml
}  // namespace fcg
