// Multi-RHS BiCGStab: several systems on one sparsity pattern (the u/v/w momentum
// systems of calcuvw.f90 share their off-diagonals; k and epsilon have their own values)
// solved together by the DILU-preconditioned BiCGStab of bicgstab.f90.
//
// Precision split: the sweeps (SpMV, DILU triangular solves, vector updates) run in
// FP32 on FP32 copies of the matrices; an FP64 outer defect-correction loop recomputes
// r = su - A x in FP64, applies the reference's stop test resl/(res0+small) < sor to
// that FP64 residual, solves A dx = r in FP32 until each system's L1 residual has
// dropped by `inner_tol`, and adds dx to x in FP64.  Global sums are formed in FP64.
//
// Layout: systems are planar (vector of system k at v + k*n, sliced values of system k
// at sval + k*sell_len).  Every kernel of a sweep covers all systems (templated on their
// count NS); a system whose inner solve has finished runs on with zero step lengths.
// One inner solve is one CUDA-graph WHILE loop; the outer loop is driven from the host
// (a handful of iterations).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fcg_internal.h"
#include "krylov_common.cuh"
#include "launch.h"

namespace fcg {

constexpr int kMaxSys = 8;

struct MScal {
  double bet[kMaxSys], om[kMaxSys], beto[kMaxSys], alf[kMaxSys], gam[kMaxSys];
  double r0in[kMaxSys], rl[kMaxSys];    // inner residual L1: at the inner start, current
  double res0[kMaxSys], resl[kMaxSys];  // FP64 residual L1: first, latest
  double scale[kMaxSys];  // the inner solve works on r / scale (entries of order one)
  double l2r[kMaxSys], l2b[kMaxSys];    // final FP64 ||su - A x||^2 and ||su||^2
  double small, resmax, inner_tol;
  int active[kMaxSys], conv[kMaxSys];
  int iter, inner_iter, inner_max, nsw, idone, status, any_active, pad;
  unsigned int ticket[8];
  unsigned int body_count;
};

struct MultiState {
  int n = 0, ns = 0;
  long long nnz = 0, len = 0;
  unsigned bind_gen = 0;
  DBuf buf;
  double *sv64 = nullptr, *x = nullptr, *su = nullptr, *res64 = nullptr, *partials = nullptr;
  float *sv32 = nullptr, *a32 = nullptr, *d32 = nullptr;
  float *r = nullptr, *rh = nullptr, *p = nullptr, *u = nullptr, *z = nullptr, *v = nullptr,
        *dx = nullptr;
  MScal *S = nullptr, *hS = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int G = 0;
  // one-launch DILU sweeps (as krylov.cu): forward results and the control words
  // {forward claim counter, backward claim counter, -, error}
  DBuf sfb;
  float *y32 = nullptr;
  int *ctl = nullptr;
  int sf_grid = 0;
  bool sf_on = true;
};

void destroy_multi(MultiState *m) {
  if (!m) return;
  if (m->exec) cudaGraphExecDestroy(m->exec);
  if (m->graph) cudaGraphDestroy(m->graph);
  if (m->cap) cudaStreamDestroy(m->cap);
  if (m->S) cudaFree(m->S);
  if (m->hS) cudaFreeHost(m->hS);
  m->buf.release();
  m->sfb.release();
  delete m;
}

namespace {

__device__ __forceinline__ bool inner_done(const MScal *S) { return __ldcg(&S->idone) != 0; }

// Sliced FP64/FP32 values and FP32 CSR values of every system from CSR a[k*nnz + ...].
__global__ void k_m_fill(SellView s, int ns, long long nnz, long long len,
                         const double *__restrict__ a, double *__restrict__ sv64,
                         float *__restrict__ sv32, float *__restrict__ a32) {
  FCG_GRID_STRIDE(p, len) {
    const int src = s.src[p];
    for (int k = 0; k < ns; ++k) {
      double v = src >= 0 ? a[k * nnz + src] : 0.0;
      sv64[k * len + p] = v;
      sv32[k * len + p] = (float)v;
    }
  }
  FCG_GRID_STRIDE(q, nnz) {
    for (int k = 0; k < ns; ++k) a32[k * nnz + q] = (float)a[k * nnz + q];
  }
}

// DILU diagonal of each system, level by level (bicgstab.f90:68-79), in FP32.
template <int NS>
__global__ void k_m_factor(const int *__restrict__ rows, int count, long long nnz, int n,
                           const int *__restrict__ io, const int *__restrict__ ja,
                           const int *__restrict__ dg, const int *__restrict__ tpos,
                           const float *__restrict__ a32, float *__restrict__ d32, MScal *S) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const float *a = a32 + k * nnz;
    float *d = d32 + (long long)k * n;
    float di = a[dg[i]];
    for (int q = io[i]; q < dg[i]; ++q)
      di = __fsub_rn(di, __fmul_rn(__fmul_rn(a[q], d[ja[q]]), a[tpos[q]]));
    const float inv = 1.0f / di;
    d[i] = inv;
    if (!isfinite(inv)) atomicCAS(&S->status, 0, FCG_ERR_PIVOT);
  }
}

// Outer FP64 step: r = su - A x in FP64, its L1 per system and the stop test; FP32
// start vectors of the next inner solve (r = rh = FP32 residual, p = u = dx = 0).
template <int NS>
__global__ void __launch_bounds__(kTPB, 4)
    k_m_residual(SellView s, int n, long long len, const double *__restrict__ sv64,
                 const double *__restrict__ su, const double *__restrict__ x,
                 double *__restrict__ x_res, float *__restrict__ p, float *__restrict__ u,
                 float *__restrict__ dx, MScal *S, double *partials, int first) {
  double l1[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) l1[k] = 0.0;
  FCG_SLICE_LOOP(slice, lane, s) {
    const int row = slice * 32 + lane;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const double ax = sell_row(s, n, sv64 + k * len, x + (long long)k * n, slice, lane);
      if (row < n) {
        const long long o = (long long)k * n + row;
        const double rr = su[o] - ax;
        l1[k] += fabs(rr);
        x_res[o] = rr;  // kept in FP64 until its scale is known
        p[o] = 0.f;
        u[o] = 0.f;
        dx[o] = 0.f;
      }
    }
  }
  if (reduce_commit<NS>(l1, partials, &S->ticket[0]) && threadIdx.x == 0) {
    int any = 0;
    for (int k = 0; k < NS; ++k) {
      if (first) S->res0[k] = l1[k];
      S->resl[k] = l1[k];
      S->conv[k] = (l1[k] / (S->res0[k] + S->small) < S->resmax) ? 1 : 0;
      S->scale[k] = l1[k] > 0 ? l1[k] / (double)n : 1.0;
      S->r0in[k] = l1[k] / S->scale[k];  // L1 of the scaled inner start residual
      S->rl[k] = S->r0in[k];
      S->active[k] = !S->conv[k];
      any |= S->active[k];
      S->alf[k] = 1.0;  // bicgstab.f90:90-92
      S->beto[k] = 1.0;
      S->gam[k] = 1.0;
      if (!isfinite(l1[k])) atomicCAS(&S->status, 0, FCG_ERR_NONFINITE);
    }
    S->any_active = any;
    S->inner_iter = 0;
    S->idone = (!any || S->iter >= S->nsw || S->status) ? 1 : 0;
  }
}

// r = rh = (FP64 residual) / scale, in FP32: the inner solve sees entries of order one,
// so the reference's absolute `small` stays negligible however far the outer loop got.
// Final FP64 check per system: ||su - A x||^2 and ||su||^2.
template <int NS>
__global__ void __launch_bounds__(kTPB, 4)
    k_m_final(SellView s, int n, long long len, const double *__restrict__ sv64,
              const double *__restrict__ su, const double *__restrict__ x, MScal *S,
              double *partials) {
  double v[2 * NS];
#pragma unroll
  for (int k = 0; k < 2 * NS; ++k) v[k] = 0.0;
  FCG_SLICE_LOOP(slice, lane, s) {
    const int row = slice * 32 + lane;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const double ax = sell_row(s, n, sv64 + k * len, x + (long long)k * n, slice, lane);
      if (row < n) {
        const long long o = (long long)k * n + row;
        const double rr = su[o] - ax;
        v[k] += rr * rr;
        v[NS + k] += su[o] * su[o];
      }
    }
  }
  if (reduce_commit<2 * NS>(v, partials, &S->ticket[5]) && threadIdx.x == 0)
    for (int k = 0; k < NS; ++k) {
      S->l2r[k] = v[k];
      S->l2b[k] = v[NS + k];
    }
}

template <int NS>
__global__ void k_m_normalise(int n, const double *__restrict__ x_res, float *__restrict__ r,
                              float *__restrict__ rh, const MScal *S) {
  double inv[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) inv[k] = 1.0 / __ldcg(&S->scale[k]);
  FCG_GRID_STRIDE(i, n) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const long long o = (long long)k * n + i;
      const float v = (float)(x_res[o] * inv[k]);
      r[o] = v;
      rh[o] = v;
    }
  }
}

// bet = r.rh; om = bet*gam/(alf*beto+small); beto = bet   (bicgstab.f90:104-106)
template <int NS>
__global__ void __launch_bounds__(kTPB, 6)
    k_m_dot1(int n, const float *__restrict__ r, const float *__restrict__ rh, MScal *S,
             double *partials) {
  if (inner_done(S)) return;
  float t[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) t[k] = 0.f;
  FCG_GRID_STRIDE(i, n) {
#pragma unroll
    for (int k = 0; k < NS; ++k) t[k] += r[(long long)k * n + i] * rh[(long long)k * n + i];
  }
  double v[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) v[k] = t[k];
  if (reduce_commit<NS>(v, partials, &S->ticket[1]) && threadIdx.x == 0) {
    for (int k = 0; k < NS; ++k) {
      S->bet[k] = v[k];
      S->om[k] = S->active[k] ? v[k] * S->gam[k] / (S->alf[k] * S->beto[k] + S->small) : 0.0;
      S->beto[k] = v[k];
    }
  }
}

// p = r + om*(p - alf*u)   (bicgstab.f90:111)
template <int NS>
__global__ void __launch_bounds__(kTPB, 6)
    k_m_p(int n, const float *__restrict__ r, const float *__restrict__ u, float *__restrict__ p,
          const MScal *S) {
  if (inner_done(S)) return;
  float om[NS], alf[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    om[k] = (float)__ldcg(&S->om[k]);
    alf[k] = (float)__ldcg(&S->alf[k]);
  }
  FCG_GRID_STRIDE(i, n) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const long long o = (long long)k * n + i;
      p[o] = r[o] + om[k] * (p[o] - alf[k] * u[o]);
    }
  }
}

// z = M^-1 b, forward part of one level: z_i = (b_i - sum_{q<diag} a_q z_ja) d_i
template <int NS>
__global__ void k_m_fwd(const int *__restrict__ rows, int count, long long nnz, int n,
                        const int *__restrict__ io, const int *__restrict__ ja,
                        const int *__restrict__ dg, const float *__restrict__ a32,
                        const float *__restrict__ d32, const float *__restrict__ b,
                        float *__restrict__ z, const MScal *S) {
  if (inner_done(S)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const float *a = a32 + k * nnz;
    const float *zk = z + (long long)k * n;
    float zi = b[(long long)k * n + i];
    for (int q = io[i]; q < dg[i]; ++q) zi = __fsub_rn(zi, __fmul_rn(a[q], zk[ja[q]]));
    z[(long long)k * n + i] = zi * d32[(long long)k * n + i];
  }
}

// backward part with the reference's rescale z/(d+small) folded in (bicgstab.f90:125-136)
template <int NS>
__global__ void k_m_bwd(const int *__restrict__ rows, int count, long long nnz, int n,
                        const int *__restrict__ io, const int *__restrict__ ja,
                        const int *__restrict__ dg, const float *__restrict__ a32,
                        const float *__restrict__ d32, float *__restrict__ z, const MScal *S) {
  if (inner_done(S)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t];
  const float small = (float)S->small;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const float *a = a32 + k * nnz;
    float *zk = z + (long long)k * n;
    const float di = d32[(long long)k * n + i];
    float zi = zk[i] / (di + small);
    for (int q = dg[i] + 1; q < io[i + 1]; ++q) zi = __fsub_rn(zi, __fmul_rn(a[q], zk[ja[q]]));
    zk[i] = zi * di;
  }
}

// --- DILU sweeps in one launch (the scheme of krylov.cu's k_fwd_sf): rows claimed in
// level order by warps, each waiting on the FP32 values it reads, which are filled with
// a signalling-NaN sentinel before the sweep.  The same row arithmetic as the level
// kernels above.
constexpr unsigned kSent32 = 0x7f80deadu;
constexpr int kSfSpin = 1 << 20;

__device__ __forceinline__ float ld_relaxed32(const float *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return __uint_as_float(v);
}

__device__ __forceinline__ void st_relaxed32(float *p, float x) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(__float_as_uint(x)) : "memory");
}

__device__ __forceinline__ bool sent32(float v) { return __float_as_uint(v) == kSent32; }

__device__ __forceinline__ float sf_value32(const float *p, const int *err, bool *ok) {
  float v = ld_relaxed32(p);
  if (!sent32(v)) return v;
  for (int it = 0; it < kSfSpin; ++it) {
    if (it >= 16) __nanosleep(32);
    v = ld_relaxed32(p);
    if (!sent32(v)) return v;
    if ((it & 63) == 63 && *(volatile const int *)err) break;
  }
  *ok = false;
  return v;
}

__device__ __forceinline__ void sf_fail32(int *err, MScal *S) {
  if (atomicExch(err, 1) == 0) atomicCAS(&S->status, 0, FCG_ERR_TIMEOUT);
}

__global__ void k_m_sf_fill(long long count, float *__restrict__ o1, float *__restrict__ o2,
                            int *ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl[0] = 0;
    ctl[1] = 0;
    ctl[3] = 0;
  }
  const float s = __uint_as_float(kSent32);
  FCG_GRID_STRIDE(i, count) {
    o1[i] = s;
    if (o2) o2[i] = s;
  }
}

// Claims the next 32 entries of the level list for the calling warp (-1: none left).
__device__ __forceinline__ int sf_claim(int *ctr) {
  int base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(ctr, 32);
  return __shfl_sync(0xffffffffu, base, 0);
}

template <int NS>
__global__ void k_m_fwd_sf(const int *__restrict__ rows, int len, long long nnz, int n,
                           const int *__restrict__ io, const int *__restrict__ ja,
                           const int *__restrict__ dg, const float *__restrict__ a32,
                           const float *__restrict__ d32, const float *__restrict__ b, float *y,
                           int *ctl, MScal *S) {
  if (inner_done(S)) return;
  for (;;) {
    const int base = sf_claim(&ctl[0]);
    if (base >= len) break;
    const int i = rows[base + (threadIdx.x & 31)];
    if (i < 0) continue;
    float zi[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) zi[k] = b[(long long)k * n + i];
    bool ok = true;
    for (int q = io[i]; q < dg[i]; ++q) {
      const int j = ja[q];
      float v[NS];
#pragma unroll
      for (int k = 0; k < NS; ++k) v[k] = ld_relaxed32(&y[(long long)k * n + j]);
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        if (sent32(v[k])) v[k] = sf_value32(&y[(long long)k * n + j], &ctl[3], &ok);
        zi[k] = __fsub_rn(zi[k], __fmul_rn(a32[k * nnz + q], v[k]));
      }
    }
    if (!ok) sf_fail32(&ctl[3], S);
#pragma unroll
    for (int k = 0; k < NS; ++k)
      st_relaxed32(&y[(long long)k * n + i], zi[k] * d32[(long long)k * n + i]);
  }
}

template <int NS>
__global__ void k_m_bwd_sf(const int *__restrict__ rows, int len, long long nnz, int n,
                           const int *__restrict__ io, const int *__restrict__ ja,
                           const int *__restrict__ dg, const float *__restrict__ a32,
                           const float *__restrict__ d32, const float *__restrict__ y, float *z,
                           int *ctl, MScal *S) {
  if (inner_done(S)) return;
  const float small = (float)S->small;
  for (;;) {
    const int base = sf_claim(&ctl[1]);
    if (base >= len) break;
    const int i = rows[base + (threadIdx.x & 31)];
    if (i < 0) continue;
    float zi[NS], di[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      di[k] = d32[(long long)k * n + i];
      zi[k] = y[(long long)k * n + i] / (di[k] + small);
    }
    bool ok = true;
    for (int q = dg[i] + 1; q < io[i + 1]; ++q) {
      const int j = ja[q];
      float v[NS];
#pragma unroll
      for (int k = 0; k < NS; ++k) v[k] = ld_relaxed32(&z[(long long)k * n + j]);
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        if (sent32(v[k])) v[k] = sf_value32(&z[(long long)k * n + j], &ctl[3], &ok);
        zi[k] = __fsub_rn(zi[k], __fmul_rn(a32[k * nnz + q], v[k]));
      }
    }
    if (!ok) sf_fail32(&ctl[3], S);
#pragma unroll
    for (int k = 0; k < NS; ++k) st_relaxed32(&z[(long long)k * n + i], zi[k] * di[k]);
  }
}

template <int NS>
__global__ void k_m_factor_sf(const int *__restrict__ rows, int len, long long nnz, int n,
                              const int *__restrict__ io, const int *__restrict__ ja,
                              const int *__restrict__ dg, const int *__restrict__ tpos,
                              const float *__restrict__ a32, float *d32, int *ctl, MScal *S) {
  for (;;) {
    const int base = sf_claim(&ctl[0]);
    if (base >= len) break;
    const int i = rows[base + (threadIdx.x & 31)];
    if (i < 0) continue;
    float di[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) di[k] = a32[k * nnz + dg[i]];
    bool ok = true;
    for (int q = io[i]; q < dg[i]; ++q) {
      const int j = ja[q];
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        const float *a = a32 + k * nnz;
        const float dj = sf_value32(&d32[(long long)k * n + j], &ctl[3], &ok);
        di[k] = __fsub_rn(di[k], __fmul_rn(__fmul_rn(a[q], dj), a[tpos[q]]));
      }
    }
    if (!ok) sf_fail32(&ctl[3], S);
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const float inv = 1.0f / di[k];
      st_relaxed32(&d32[(long long)k * n + i], inv);
      if (!isfinite(inv)) atomicCAS(&S->status, 0, FCG_ERR_PIVOT);
    }
  }
}

// y = A z for every system; sums y.w (and y.y when TWO) per system.
template <int NS, bool TWO>
__global__ void __launch_bounds__(kTPB, 4)
    k_m_spmv(SellView s, int n, long long len, const float *__restrict__ sv32,
             const float *__restrict__ z, const float *__restrict__ w, float *__restrict__ y,
             MScal *S, double *partials, int which) {
  if (inner_done(S)) return;
  float t1[NS], t2[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) t1[k] = t2[k] = 0.f;
  FCG_SLICE_LOOP(slice, lane, s) {
    const int row = slice * 32 + lane;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const float q = sell_row(s, n, sv32 + k * len, z + (long long)k * n, slice, lane);
      if (row < n) {
        const long long o = (long long)k * n + row;
        y[o] = q;
        t1[k] += q * w[o];
        if (TWO) t2[k] += q * q;
      }
    }
  }
  constexpr int NV = TWO ? 2 * NS : NS;
  double v[NV];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    v[k] = t1[k];
    if (TWO) v[NS + k] = t2[k];
  }
  if (reduce_commit<NV>(v, partials, &S->ticket[2 + which]) && threadIdx.x == 0) {
    for (int k = 0; k < NS; ++k) {
      if (which == 0) {  // gam = bet / (u.rh)   (bicgstab.f90:153-154)
        S->gam[k] = S->active[k] ? S->bet[k] / v[k] : 0.0;
        if (S->active[k] && !isfinite(S->gam[k])) atomicCAS(&S->status, 0, FCG_ERR_NONFINITE);
      } else {  // alf = (v.r) / (v.v + small)   (bicgstab.f90:200)
        S->alf[k] = S->active[k] ? v[k] / (v[NS + k] + S->small) : 0.0;
        if (S->active[k] && !isfinite(S->alf[k])) atomicCAS(&S->status, 0, FCG_ERR_NONFINITE);
      }
    }
  }
}

// dx += gam z; r -= gam u   (bicgstab.f90:160-161)
template <int NS>
__global__ void __launch_bounds__(kTPB, 6)
    k_m_upd1(int n, float *__restrict__ dx, float *__restrict__ r, const float *__restrict__ z,
             const float *__restrict__ u, const MScal *S) {
  if (inner_done(S)) return;
  float g[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) g[k] = (float)__ldcg(&S->gam[k]);
  FCG_GRID_STRIDE(i, n) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const long long o = (long long)k * n + i;
      dx[o] = dx[o] + g[k] * z[o];
      r[o] = r[o] - g[k] * u[o];
    }
  }
}

__device__ __noinline__ void m_close(MScal *S, const double *l1, int ns,
                                     cudaGraphConditionalHandle h, int use_cond) {
  S->inner_iter++;
  S->iter++;
  int any = 0;
  for (int k = 0; k < ns; ++k) {
    if (!S->active[k]) continue;
    S->rl[k] = l1[k];
    if (!isfinite(l1[k])) atomicCAS(&S->status, 0, FCG_ERR_NONFINITE);
    if (l1[k] < S->inner_tol * S->r0in[k]) S->active[k] = 0;
    any |= S->active[k];
  }
  S->any_active = any;
  if (!any || S->inner_iter >= S->inner_max || S->iter >= S->nsw || S->status) {
    S->idone = 1;
    if (use_cond) cudaGraphSetConditional(h, 0);
  }
}

// dx += alf z; r -= alf v; L1 of r; inner stop test; closes the loop body
template <int NS>
__global__ void __launch_bounds__(kTPB, 6)
    k_m_upd2(int n, float *__restrict__ dx, float *__restrict__ r, const float *__restrict__ z,
             const float *__restrict__ vv, MScal *S, double *partials,
             cudaGraphConditionalHandle h, int use_cond) {
  if (inner_done(S)) {
    if (use_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(h, 0);
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {  // bound on the loop, independent of the sums
    unsigned int c = atomicAdd(&S->body_count, 1u) + 1u;
    if (c > (unsigned int)S->inner_max + 2u) {
      atomicCAS(&S->status, 0, FCG_ERR_TIMEOUT);
      S->idone = 1;
      if (use_cond) cudaGraphSetConditional(h, 0);
    }
  }
  float a[NS], t[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    a[k] = (float)__ldcg(&S->alf[k]);
    t[k] = 0.f;
  }
  FCG_GRID_STRIDE(i, n) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const long long o = (long long)k * n + i;
      dx[o] = dx[o] + a[k] * z[o];
      const float rr = r[o] - a[k] * vv[o];
      r[o] = rr;
      t[k] += fabsf(rr);
    }
  }
  double v[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) v[k] = t[k];
  if (reduce_commit<NS>(v, partials, &S->ticket[4]) && threadIdx.x == 0)
    m_close(S, v, NS, h, use_cond);
}

// x += scale * dx in FP64
template <int NS>
__global__ void k_m_correct(int n, double *__restrict__ x, const float *__restrict__ dx,
                            const MScal *S) {
  FCG_GRID_STRIDE(i, (long long)NS * n) {
    const double sc = __ldcg(&S->scale[i / n]);
    x[i] = x[i] + sc * (double)dx[i];
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int NS>
struct Launch {
  static void sweeps(fcg_context *c, cudaStream_t st, const Level &lv, bool fwd, const float *b,
                     float *z) {
    MultiState *m = c->ms;
    if (m->sf_on) {
      if (fwd) {  // b -> y32, after the sentinel fill of y32 and z
        k_m_sf_fill<<<grid_for((long long)NS * m->n, c->num_sms), kTPB, 0, st>>>(
            (long long)NS * m->n, m->y32, z, m->ctl);
        k_m_fwd_sf<NS><<<m->sf_grid, kTPB, 0, st>>>(lv.pad, lv.pad_len, m->nnz, m->n,
                                                    c->mv.ioffset, c->mv.ja, c->mv.diag, m->a32,
                                                    m->d32, b, m->y32, m->ctl, m->S);
      } else {  // y32 -> z
        k_m_bwd_sf<NS><<<m->sf_grid, kTPB, 0, st>>>(lv.pad, lv.pad_len, m->nnz, m->n,
                                                    c->mv.ioffset, c->mv.ja, c->mv.diag, m->a32,
                                                    m->d32, m->y32, z, m->ctl, m->S);
      }
      return;
    }
    for (int l = 0; l < lv.count; ++l) {
      const int start = lv.ptr[l], cnt = lv.ptr[l + 1] - lv.ptr[l];
      const int g = (cnt + kTPB - 1) / kTPB;
      if (fwd)
        k_m_fwd<NS><<<g, kTPB, 0, st>>>(lv.rows + start, cnt, m->nnz, m->n, c->mv.ioffset,
                                         c->mv.ja, c->mv.diag, m->a32, m->d32, b, z, m->S);
      else
        k_m_bwd<NS><<<g, kTPB, 0, st>>>(lv.rows + start, cnt, m->nnz, m->n, c->mv.ioffset,
                                         c->mv.ja, c->mv.diag, m->a32, m->d32, z, m->S);
    }
  }

  static void sweep(fcg_context *c, cudaStream_t st, cudaGraphConditionalHandle h, int use_cond) {
    MultiState *m = c->ms;
    const int n = m->n, G = m->G;
    k_m_dot1<NS><<<G, kTPB, 0, st>>>(n, m->r, m->rh, m->S, m->partials);
    k_m_p<NS><<<G, kTPB, 0, st>>>(n, m->r, m->u, m->p, m->S);
    sweeps(c, st, c->lf, true, m->p, m->z);
    sweeps(c, st, c->lb, false, nullptr, m->z);
    k_m_spmv<NS, false><<<G, kTPB, 0, st>>>(c->sv, n, m->len, m->sv32, m->z, m->rh, m->u, m->S,
                                             m->partials, 0);
    k_m_upd1<NS><<<G, kTPB, 0, st>>>(n, m->dx, m->r, m->z, m->u, m->S);
    sweeps(c, st, c->lf, true, m->r, m->z);
    sweeps(c, st, c->lb, false, nullptr, m->z);
    k_m_spmv<NS, true><<<G, kTPB, 0, st>>>(c->sv, n, m->len, m->sv32, m->z, m->r, m->v, m->S,
                                            m->partials, 1);
    k_m_upd2<NS><<<G, kTPB, 0, st>>>(n, m->dx, m->r, m->z, m->v, m->S, m->partials, h, use_cond);
  }

  static void factor(fcg_context *c) {
    MultiState *m = c->ms;
    if (m->sf_on) {
      k_m_sf_fill<<<grid_for((long long)NS * m->n, c->num_sms), kTPB, 0, c->stream>>>(
          (long long)NS * m->n, m->d32, nullptr, m->ctl);
      k_m_factor_sf<NS><<<m->sf_grid, kTPB, 0, c->stream>>>(
          c->lf.pad, c->lf.pad_len, m->nnz, m->n, c->mv.ioffset, c->mv.ja, c->mv.diag, c->tpos,
          m->a32, m->d32, m->ctl, m->S);
      return;
    }
    for (int l = 0; l < c->lf.count; ++l) {
      const int start = c->lf.ptr[l], cnt = c->lf.ptr[l + 1] - c->lf.ptr[l];
      k_m_factor<NS><<<(cnt + kTPB - 1) / kTPB, kTPB, 0, c->stream>>>(
          c->lf.rows + start, cnt, m->nnz, m->n, c->mv.ioffset, c->mv.ja, c->mv.diag, c->tpos,
          m->a32, m->d32, m->S);
    }
  }

  static void residual(fcg_context *c, int first) {
    MultiState *m = c->ms;
    k_m_residual<NS><<<m->G, kTPB, 0, c->stream>>>(c->sv, m->n, m->len, m->sv64, m->su, m->x,
                                                    m->res64, m->p, m->u, m->dx, m->S,
                                                    m->partials, first);
    k_m_normalise<NS><<<grid_for(m->n, c->num_sms), kTPB, 0, c->stream>>>(m->n, m->res64, m->r,
                                                                          m->rh, m->S);
  }

  static void correct(fcg_context *c) {
    MultiState *m = c->ms;
    k_m_correct<NS><<<grid_for((long long)NS * m->n, c->num_sms), kTPB, 0, c->stream>>>(
        m->n, m->x, m->dx, m->S);
  }
};

template <int NS>
int build_inner_graph(fcg_context *c) {
  MultiState *m = c->ms;
  if (m->exec) return FCG_OK;
  cudaGraph_t g;
  FCG_CUDA_TRY(c, cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  FCG_CUDA_TRY(c, cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  FCG_CUDA_TRY(c, cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np));
  FCG_CUDA_TRY(c, cudaStreamBeginCaptureToGraph(m->cap, np.conditional.phGraph_out[0], nullptr,
                                                nullptr, 0, cudaStreamCaptureModeThreadLocal));
  Launch<NS>::sweep(c, m->cap, h, 1);
  cudaGraph_t captured = nullptr;
  cudaError_t e = cudaStreamEndCapture(m->cap, &captured);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&m->exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(c, e, "multi-RHS inner graph");
  }
  m->graph = g;
  return FCG_OK;
}

template <int NS>
int solve_multi(fcg_context *c, const double *da, const double *dsu, double *dfi, double sor,
                int nsw, double *resor, fcg_solve_report *rep) {
  MultiState *m = c->ms;
  const size_t nb = sizeof(double) * (size_t)NS * m->n;
  k_m_fill<<<grid_for(std::max(m->len, m->nnz), c->num_sms), kTPB, 0, c->stream>>>(
      c->sv, NS, m->nnz, m->len, da, m->sv64, m->sv32, m->a32);
  FCG_CHECK_LAUNCH(c, "k_m_fill");
  FCG_CUDA_TRY(c, cudaMemcpyAsync(m->x, dfi, nb, cudaMemcpyDeviceToDevice, c->stream));
  FCG_CUDA_TRY(c, cudaMemcpyAsync(m->su, dsu, nb, cudaMemcpyDeviceToDevice, c->stream));
  MScal init;
  std::memset(&init, 0, sizeof init);
  init.small = (double)1e-20f;  // parameters::small
  init.resmax = sor;
  init.inner_tol = 1e-4;
  init.inner_max = std::max(1, nsw);
  init.nsw = nsw;
  *m->hS = init;
  FCG_CUDA_TRY(c, cudaMemcpyAsync(m->S, m->hS, sizeof(MScal), cudaMemcpyHostToDevice, c->stream));
  Launch<NS>::factor(c);
  FCG_CHECK_LAUNCH(c, "k_m_factor");
  int rc = build_inner_graph<NS>(c);
  if (rc) return rc;
  for (int outer = 0; outer < 64; ++outer) {
    Launch<NS>::residual(c, outer == 0);
    FCG_CHECK_LAUNCH(c, "k_m_residual");
    FCG_CUDA_TRY(c, cudaMemcpyAsync(m->hS, m->S, sizeof(MScal), cudaMemcpyDeviceToHost, c->stream));
    FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (m->hS->idone) break;  // every system met the stop test, or the sweeps ran out
    // fresh loop-body counter for this inner solve
    FCG_CUDA_TRY(c, cudaMemsetAsync(&m->S->body_count, 0, sizeof(unsigned int), c->stream));
    FCG_CUDA_TRY(c, cudaGraphLaunch(m->exec, c->stream));
    Launch<NS>::correct(c);
    FCG_CHECK_LAUNCH(c, "k_m_correct");
  }
  k_m_final<NS><<<m->G, kTPB, 0, c->stream>>>(c->sv, m->n, m->len, m->sv64, m->su, m->x, m->S,
                                             m->partials);
  FCG_CHECK_LAUNCH(c, "k_m_final");
  FCG_CUDA_TRY(c, cudaMemcpyAsync(dfi, m->x, nb, cudaMemcpyDeviceToDevice, c->stream));
  FCG_CUDA_TRY(c, cudaMemcpyAsync(m->hS, m->S, sizeof(MScal), cudaMemcpyDeviceToHost, c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const MScal &S = *m->hS;
  for (int k = 0; k < NS; ++k) {
    if (resor && S.iter > 0) resor[k] = S.res0[k];
    if (rep) {
      rep[k].res0 = S.res0[k];
      rep[k].resl = S.resl[k];
      rep[k].iters = S.iter;
      rep[k].converged = S.conv[k];
      rep[k].l2_rel = S.l2b[k] > 0 ? std::sqrt(S.l2r[k] / S.l2b[k]) : std::sqrt(S.l2r[k]);
      rep[k].seconds = 0.0;
    }
  }
  if (S.status) return set_error(c, S.status, "multi-RHS BiCGStab: non-finite value, pivot or loop bound");
  return FCG_OK;
}

int ensure_multi(fcg_context *c, int ns) {
  MultiState *m = c->ms;
  if (!m) {
    m = c->ms = new MultiState();
    FCG_CUDA_TRY(c, cudaMalloc(&m->S, sizeof(MScal)));
    FCG_CUDA_TRY(c, cudaMallocHost(&m->hS, sizeof(MScal)));
    FCG_CUDA_TRY(c, cudaStreamCreateWithFlags(&m->cap, cudaStreamNonBlocking));
  }
  if (m->n == c->n && m->ns == ns && m->nnz == c->nnz && m->len == c->sell_len &&
      m->bind_gen == c->bind_gen)
    return FCG_OK;
  if (m->exec) cudaGraphExecDestroy(m->exec);
  if (m->graph) cudaGraphDestroy(m->graph);
  m->exec = nullptr;
  m->graph = nullptr;
  const size_t n = c->n, nn = ((size_t)ns * n + 63) & ~(size_t)63;
  m->G = c->num_sms * 4;
  const size_t dbl = 2 * (size_t)ns * c->sell_len + 3 * nn + (size_t)16 * kMaxSys * m->G + 64;
  const size_t flt = (size_t)ns * c->sell_len + (size_t)ns * c->nnz + 8 * nn + 64;
  FCG_CUDA_TRY(c, m->buf.ensure(dbl * sizeof(double) + flt * sizeof(float)));
  double *d = m->buf.as<double>();
  m->sv64 = d;
  d += (size_t)ns * c->sell_len;
  m->x = d;
  d += nn;
  m->su = d;
  d += nn;
  m->res64 = d;
  d += nn;
  m->partials = d;
  d += (size_t)16 * kMaxSys * m->G;
  float *f = (float *)(d + 64);
  m->sv32 = f;
  f += (size_t)ns * c->sell_len;
  m->a32 = f;
  f += (size_t)ns * c->nnz;
  float **vecs[] = {&m->d32, &m->r, &m->rh, &m->p, &m->u, &m->z, &m->v, &m->dx};
  for (float **v : vecs) {
    *v = f;
    f += nn;
  }
  FCG_CUDA_TRY(c, m->sfb.ensure(nn * sizeof(float) + 16 * sizeof(int)));
  FCG_CUDA_TRY(c, cudaMemset(m->sfb.p, 0, nn * sizeof(float) + 16 * sizeof(int)));
  m->y32 = m->sfb.as<float>();
  m->ctl = (int *)(m->y32 + nn);
  m->sf_grid = c->num_sms * 2;
  {
    const char *e = std::getenv("FCG_SWEEP");
    m->sf_on = !(e && std::string(e) == "levels");
  }
  m->n = c->n;
  m->ns = ns;
  m->nnz = c->nnz;
  m->len = c->sell_len;
  m->bind_gen = c->bind_gen;
  return FCG_OK;
}

}  // namespace
}  // namespace fcg

using namespace fcg;

extern "C" int fcg_bicgstab_multi(fcg_context *c, int nsys, const double *a, const double *su,
                                  double *fi, double sor, int nsw, double *resor,
                                  fcg_solve_report *rep) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_bicgstab_multi before fcg_bind_mesh");
  if (c->mv.noc) return refuse_oc(c, "fcg_bicgstab_multi");
  if (nsys < 1 || nsys > kMaxSys) return set_error(c, FCG_ERR_ARG, "nsys must be 1..8");
  if (!a || !su || !fi || nsw < 0) return set_error(c, FCG_ERR_ARG, "bad argument");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = ensure_multi(c, nsys);
  if (rc) return rc;
  const size_t nb = sizeof(double) * (size_t)nsys * c->n;
  void *da, *dsu, *dfi;
  bool ha, hsu, hfi;
  if ((rc = stage_in(c, a, sizeof(double) * (size_t)nsys * c->nnz, 0, true, &da, &ha))) return rc;
  if ((rc = stage_in(c, su, nb, 1, true, &dsu, &hsu))) return rc;
  if ((rc = stage_in(c, fi, nb, 2, true, &dfi, &hfi))) return rc;
  const double *A = (const double *)da, *B = (const double *)dsu;
  double *X = (double *)dfi;
  switch (nsys) {
    case 1: rc = solve_multi<1>(c, A, B, X, sor, nsw, resor, rep); break;
    case 2: rc = solve_multi<2>(c, A, B, X, sor, nsw, resor, rep); break;
    case 3: rc = solve_multi<3>(c, A, B, X, sor, nsw, resor, rep); break;
    case 4: rc = solve_multi<4>(c, A, B, X, sor, nsw, resor, rep); break;
    case 5: rc = solve_multi<5>(c, A, B, X, sor, nsw, resor, rep); break;
    case 6: rc = solve_multi<6>(c, A, B, X, sor, nsw, resor, rep); break;
    case 7: rc = solve_multi<7>(c, A, B, X, sor, nsw, resor, rep); break;
    default: rc = solve_multi<8>(c, A, B, X, sor, nsw, resor, rep); break;
  }
  if (rc) return rc;
  if ((rc = stage_out(c, fi, dfi, nb, hfi))) return rc;
  if (hfi) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}
