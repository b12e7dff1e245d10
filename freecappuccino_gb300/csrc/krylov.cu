// Krylov solvers of the pressure-correction path: dpcg (src/dpcg.f90), iccg with the
// diagonal incomplete-Cholesky factor (src/iccg.f90) and bicgstab with the diagonal
// ILU factor (src/bicgstab.f90), plus the standalone SpMV.
//
// Design (one GPU, everything device-resident):
//  * The caller's CSR values are gathered once per solve into a sliced-ELL copy
//    (32-row slices, column-major inside a slice): a warp reads one entry of 32
//    consecutive rows per load, so the matrix streams from HBM fully coalesced.
//    Entries keep the CSR column order, so each row is summed in the reference's order.
//  * Every global sum (L1 norms, dot products) is a deterministic two-level reduction:
//    per-block partials, then the last block to finish (ticket counter) adds the
//    partials in index order and computes the solver scalars (alpha, beta, omega,
//    the stop test) on the device.  No host round trip per sweep.
//  * One sweep is a fixed chain of kernels captured once into the body of a CUDA-graph
//    WHILE node; the kernel that evaluates the stop test clears the node's condition.
//    A whole solve is one graph launch.
//  * The DIC/DILU triangular solves run level by level (rows of one level depend only
//    on rows of earlier levels), one kernel per level inside the same graph; each row
//    is computed with the reference's operand order, so the preconditioner is the
//    reference's M = (D+L) D^-1 (D+U) exactly.
// Deviations kept on purpose (FP64 division is slow on this part; each differs from the
// reference's division by at most one ulp per entry): DPCG's z = r / a(diag) is computed
// as r * (1/a(diag)), and the rescale zk/(d+small) between the DIC/DILU sweeps
// (iccg.f90:102) as zk * (1/(d+small)), the reciprocal formed once per solve with the
// factor.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fcg_internal.h"
#include "krylov_common.cuh"
#include "launch.h"

namespace fcg {

enum SolverKind { SK_DPCG = 0, SK_ICCG = 1, SK_BICG = 2, SK_MIXED = 3, SK_N = 4 };

// Device-resident solver scalars.  Written by the last block of a reduction kernel,
// read by the following kernels (stream order makes the writes visible).
struct Scal {
  double res0, resl, resor, rsm;
  double s0, sk, bet, pkapk, alf;  // CG; alf is also BiCGStab's alpha
  double gam, om, beto, bbet;      // BiCGStab
  double l2r, l2b;                 // final recomputed ||su - A x||^2 and ||su||^2
  double small, resmax, tol;
  int iter, nsw, done, converged, status, early, trace_cap, wait_fail;
  unsigned int ticket[8];
  unsigned int body_count;  // executions of the loop body, counted independently of iter
  // mixed precision (reliable updates)
  double rr, rr_old, maxr, l1ratio, delta;
  int ru, nupdates;
};

// Grid of each reduction kernel: one full wave of resident blocks on every SM (from the
// occupancy calculator), so no kernel runs a partial second wave.
struct Grids {
  int init, p, spmv, update, dot, bdot, bp, bspmv1, bupd1, bspmv2, bupd2, fin, plain;
  int mstart, mspmv, mupd, mru1, mru2, mp;
};

struct KrylovState {
  int n = 0, G = 0, nsw_cap = 0;
  Grids gr{};
  unsigned bind_gen = 0;
  long long nnz = 0, sell_len = 0;
  DBuf vec;  // all vectors
  double *x = nullptr, *res = nullptr, *su = nullptr, *pk = nullptr, *zk = nullptr,
         *qk = nullptr, *invd = nullptr, *d = nullptr, *reso = nullptr, *uk = nullptr,
         *vk = nullptr, *a = nullptr, *sval = nullptr, *partials = nullptr, *rtmp = nullptr;
  double *rdi = nullptr;  // 1/(d + small), the backward sweep's rescale (with the factor)
  // coefficient planes of the wavefront-tiled sweeps on a hex block: lower entries in
  // the order -nx ny, -nx, -1 and upper entries in the order +1, +nx, +nx ny, [3][n] each
  DBuf wcoef;
  double *wlo = nullptr, *wup = nullptr;
  DBuf trace;
  // mixed precision: FP32 copy of D^-1/2 A D^-1/2 in the sliced layout, the scaling
  // D^-1/2 in FP64 and the FP32 inner vectors (correction y, residual r, direction p, Ap)
  DBuf mixed;
  double *s64 = nullptr;
  float *sval32 = nullptr, *y32 = nullptr, *r32 = nullptr, *p32 = nullptr, *q32 = nullptr;
  bool mixed_ready = false;
  double ru_delta = 0.1;  // reliable update when ||r32|| drops below delta * its last true value
  Scal *S = nullptr;  // device
  Scal *hS = nullptr; // pinned host copy
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec[SK_N] = {};
  cudaGraph_t graph[SK_N] = {};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool matrix_loaded = false;
  int last_kind = -1;
  double small = (double)1e-20f;  // parameters::small (modules_allocatable.f90:27)
  int early_exit = 1;
  // sync-free triangular sweeps: the forward result and the control words
  // {forward claim counter, backward claim counter, -, error}
  DBuf sfb;
  double *sf_y = nullptr;
  int *sf_ctl = nullptr;
  int sf_grid = 0;
  bool sf_on = true;
  int sf_spin = 1 << 20;     // polls before a dependency wait gives up
  int sf_absent_row = -1;    // test hook: this row never publishes its flag
  bool wave_on = true;       // wavefront-tiled sweeps on lexicographic hex blocks
  bool wave_wide = true;     // tiles of 16 x 8 columns rather than 8 x 8
};

void destroy_krylov(KrylovState *k) {
  if (!k) return;
  for (int i = 0; i < SK_N; ++i) {
    if (k->exec[i]) cudaGraphExecDestroy(k->exec[i]);
    if (k->graph[i]) cudaGraphDestroy(k->graph[i]);
  }
  if (k->cap) cudaStreamDestroy(k->cap);
  if (k->ev0) cudaEventDestroy(k->ev0);
  if (k->ev1) cudaEventDestroy(k->ev1);
  if (k->hS) cudaFreeHost(k->hS);
  if (k->S) cudaFree(k->S);
  k->vec.release();
  k->wcoef.release();
  k->trace.release();
  k->mixed.release();
  k->sfb.release();
  delete k;
}

namespace {

__device__ __forceinline__ bool solve_done(const Scal *S) { return __ldcg(&S->done) != 0; }

// Records an error status unless one is already recorded: the first cause is reported
// (a failed wait, say, rather than the non-finite values it leads to).
__device__ __forceinline__ void fail_status(Scal *S, int code) {
  atomicCAS(&S->status, 0, code);
}

__device__ __forceinline__ void stop_loop(cudaGraphConditionalHandle h, int use_cond) {
  if (use_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(h, 0);
}

// Bound on the WHILE loop that does not depend on the reductions: the closing kernel of
// the body counts its executions and ends the loop after nsw + 2 of them whatever the
// solver scalars say (status FCG_ERR_TIMEOUT).
__device__ __forceinline__ void loop_guard(Scal *S, cudaGraphConditionalHandle h, int use_cond) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned int c = atomicAdd(&S->body_count, 1u) + 1u;
    if (c > (unsigned int)S->nsw + 2u) {
      fail_status(S, FCG_ERR_TIMEOUT);
      S->done = 1;
      if (use_cond) cudaGraphSetConditional(h, 0);
    }
  }
}

// ---------------------------------------------------------------------------
// Matrix preparation
// ---------------------------------------------------------------------------
// CSR values -> sliced ELL (one thread per row, writes coalesced along the slice);
// also 1/a(diag) for the Jacobi preconditioner.
__global__ void k_sell_fill(SellView s, int n, const int *__restrict__ diag,
                            const double *__restrict__ a, double *__restrict__ sval,
                            double *__restrict__ invd) {
  FCG_GRID_STRIDE(r, (long long)s.nslices * 32) {
    int slice = (int)(r >> 5), lane = (int)(r & 31);
    long long base = s.ptr[slice];
    int w = s.width[slice];
    int dpos = r < n ? diag[r] : -2;
    for (int j = 0; j < w; ++j) {
      long long p = base + (long long)j * 32 + lane;
      int src = s.src[p];
      double v = src >= 0 ? a[src] : 0.0;
      sval[p] = v;
      if (src == dpos && invd) invd[r] = 1.0 / v;
    }
  }
}

// Row r's O-C couplings in pair order, added to or subtracted from acc after the row's
// CSR terms, as the reference's loops over i = 1..noc follow its row loops
// (dpcg.f90:58-61 and 113-116).
__device__ __forceinline__ double oc_add(const OcView &o, int r, double acc,
                                         const double *__restrict__ x) {
  for (int e = o.ptr[r]; e < o.ptr[r + 1]; ++e) acc = acc + o.val[o.vix[e]] * x[o.col[e]];
  return acc;
}
__device__ __forceinline__ double oc_sub(const OcView &o, int r, double acc,
                                         const double *__restrict__ x) {
  for (int e = o.ptr[r]; e < o.ptr[r + 1]; ++e) acc = acc - o.val[o.vix[e]] * x[o.col[e]];
  return acc;
}

__global__ void __launch_bounds__(kTPB, 8) k_spmv(SellView s, int n, const double *__restrict__ val,
                       const double *__restrict__ x, double *__restrict__ y, OcView o) {
  FCG_SLICE_LOOP(slice, lane, s) {
    int r = slice * 32 + lane;
    double acc = sell_row(s, n, val, x, slice, lane);
    if (r < n) y[r] = o.ptr ? oc_add(o, r, acc, x) : acc;
  }
}

// ---------------------------------------------------------------------------
// Solver kernels
// ---------------------------------------------------------------------------
// res = su - A x, res0 = sum|res| (dpcg.f90:51-64); DPCG also sk = sum res^2/a(diag).
__global__ void __launch_bounds__(kTPB, 8) k_init(SellView s, int n, const double *__restrict__ val,
                       const double *__restrict__ su, const double *__restrict__ x,
                       double *__restrict__ res, const double *__restrict__ invd, Scal *S,
                       double *partials, int kind, OcView o) {
  double v[2] = {0.0, 0.0};
  FCG_SLICE_LOOP(slice, lane, s) {
    int r = slice * 32 + lane;
    double ax = sell_row(s, n, val, x, slice, lane);
    if (r < n) {
      double rr = su[r] - ax;
      if (o.ptr) rr = oc_sub(o, r, rr, x);  // every solver's residual (bicgstab.f90:49-52)
      res[r] = rr;
      v[0] += fabs(rr);
      if (kind == SK_DPCG) v[1] += rr * (rr * invd[r]);
    }
  }
  if (reduce_commit<2>(v, partials, &S->ticket[0]) && threadIdx.x == 0) {
    S->res0 = v[0];
    S->resl = v[0];
    S->iter = 0;
    S->converged = 0;
    S->status = 0;
    S->s0 = (double)1.e20f;  // dpcg.f90:76
    S->sk = v[1];
    S->bet = v[1] / S->s0;
    S->alf = 1.0;  // bicgstab.f90:90-92
    S->beto = 1.0;
    S->gam = 1.0;
    S->done = (S->nsw <= 0 || (S->early && v[0] < S->tol)) ? 1 : 0;  // dpcg.f90:66-70
    if (!isfinite(v[0])) {
      fail_status(S, FCG_ERR_NONFINITE);
      S->done = 1;
    }
  }
}

// Stop test shared by all solvers (dpcg.f90:130-142); thread 0 of the last block.
__device__ __noinline__ void finish_sweep(Scal *S, double resl, double *trace, cudaGraphConditionalHandle h,
                             int use_cond) {
  int it = S->iter + 1;
  S->iter = it;
  S->resl = resl;
  if (it == 1) S->resor = S->res0;
  double rsm = resl / (S->resor + S->small);
  S->rsm = rsm;
  if (trace && it <= S->trace_cap) {
    trace[2 * (it - 1)] = resl;
    trace[2 * (it - 1) + 1] = rsm;
  }
  if (rsm < S->resmax) S->converged = 1;
  if (!isfinite(resl)) fail_status(S, FCG_ERR_NONFINITE);
  if (S->converged || it >= S->nsw || S->status) {
    S->done = 1;
    if (use_cond) cudaGraphSetConditional(h, 0);
  }
}

// Scalar tail of k_cg_update, run by one thread: s0, sk, beta and the stop test.
__device__ __noinline__ void cg_close_sweep(Scal *S, double resl, double sk_new, double *trace,
                                            cudaGraphConditionalHandle h, int use_cond,
                                            int kind) {
  S->s0 = S->sk;  // dpcg.f90:132
  if (kind == SK_DPCG) {
    S->sk = sk_new;
    S->bet = sk_new / S->s0;  // next sweep's beta (dpcg.f90:95)
  }
  if (S->status) {
    S->done = 1;
    if (use_cond) cudaGraphSetConditional(h, 0);
    return;
  }
  finish_sweep(S, resl, trace, h, use_cond);
}

// pk = M^-1 res + bet*pk: Jacobi (dpcg.f90:85-100) or z from the sweeps (iccg.f90:278).
__global__ void __launch_bounds__(kTPB, 8) k_cg_p(int n, const double *__restrict__ res, const double *__restrict__ invd,
                       const double *__restrict__ z, double *__restrict__ pk, const Scal *S,
                       int kind) {
  if (solve_done(S)) return;
  const double bet = __ldcg(&S->bet);
  FCG_GRID_STRIDE(i, n) {
    double zi = kind == SK_DPCG ? res[i] * invd[i] : z[i];
    pk[i] = zi + bet * pk[i];
  }
}

// qk = A pk, pkapk = sum pk*qk, alf = sk/pkapk (dpcg.f90:105-121).
__global__ void __launch_bounds__(kTPB, 8) k_cg_spmv(SellView s, int n, const double *__restrict__ val,
                          const double *__restrict__ pk, double *__restrict__ qk, Scal *S,
                          double *partials, OcView o) {
  if (solve_done(S)) return;
  double v[1] = {0.0};
  FCG_SLICE_LOOP(slice, lane, s) {
    int r = slice * 32 + lane;
    double q = sell_row(s, n, val, pk, slice, lane);
    if (r < n) {
      if (o.ptr) q = oc_add(o, r, q, pk);  // block boundaries (dpcg.f90:113-116)
      qk[r] = q;
      v[0] += pk[r] * q;
    }
  }
  if (reduce_commit<1>(v, partials, &S->ticket[1]) && threadIdx.x == 0) {
    S->pkapk = v[0];
    S->alf = S->sk / v[0];
    if (!isfinite(S->alf)) fail_status(S, FCG_ERR_NONFINITE);
  }
}

// fi += alf*pk, res -= alf*qk, resl = sum|res| (dpcg.f90:124-142); DPCG also forms
// the next sk and beta in the same pass.
__global__ void __launch_bounds__(kTPB, 8) k_cg_update(int n, double *__restrict__ x, double *__restrict__ res,
                            const double *__restrict__ pk, const double *__restrict__ qk,
                            const double *__restrict__ invd, Scal *S, double *partials,
                            double *trace, cudaGraphConditionalHandle h, int use_cond, int kind) {
  if (solve_done(S)) {
    stop_loop(h, use_cond);
    return;
  }
  loop_guard(S, h, use_cond);
  const double alf = __ldcg(&S->alf);
  double v[2] = {0.0, 0.0};
  FCG_GRID_STRIDE(i, n) {
    x[i] = x[i] + alf * pk[i];
    double r = res[i] - alf * qk[i];
    res[i] = r;
    v[0] += fabs(r);
    if (kind == SK_DPCG) v[1] += r * (r * invd[i]);
  }
  if (reduce_commit<2>(v, partials, &S->ticket[2]) && threadIdx.x == 0)
    cg_close_sweep(S, v[0], v[1], trace, h, use_cond, kind);
}

// ICCG: sk = sum res*z, bet = sk/s0 (iccg.f90:268-273).
__global__ void __launch_bounds__(kTPB, 8) k_cg_dot(int n, const double *__restrict__ res, const double *__restrict__ z,
                         Scal *S, double *partials) {
  if (solve_done(S)) return;
  double v[1] = {0.0};
  FCG_GRID_STRIDE(i, n) v[0] += res[i] * z[i];
  if (reduce_commit<1>(v, partials, &S->ticket[3]) && threadIdx.x == 0) {
    S->sk = v[0];
    S->bet = v[0] / S->s0;
  }
}

// --- triangular sweeps, one launch per level -----------------------------------
// The row arithmetic of the sweeps and factors is written with __dmul_rn / __dsub_rn: a
// multiply and a subtract each rounded, as the reference's loops evaluate them, and the
// same bits whichever kernel form (per level or one launch) runs it.
// forward: z_i = (b_i - sum_{k<diag} a_k z_{ja_k}) * d_i        (iccg.f90:248-254)
__global__ void k_fwd_level(const int *__restrict__ rows, int count,
                            const int *__restrict__ ioffset, const int *__restrict__ ja,
                            const int *__restrict__ diag, const double *__restrict__ a,
                            const double *__restrict__ d, const double *__restrict__ b,
                            double *__restrict__ z, const Scal *S) {
  if (solve_done(S)) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  int i = rows[t];
  double zi = b[i];
  for (int k = ioffset[i]; k < diag[i]; ++k) zi = __dsub_rn(zi, __dmul_rn(a[k], z[ja[k]]));
  z[i] = zi * d[i];
}

// backward with the reference's rescale zk/(d+small) folded in (iccg.f90:256-265), as a
// product with rdi = 1/(d+small).
__global__ void k_bwd_level(const int *__restrict__ rows, int count,
                            const int *__restrict__ ioffset, const int *__restrict__ ja,
                            const int *__restrict__ diag, const double *__restrict__ a,
                            const double *__restrict__ d, const double *__restrict__ rdi,
                            double *__restrict__ z, const Scal *S) {
  if (solve_done(S)) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  int i = rows[t];
  double di = d[i];
  double zi = z[i] * rdi[i];
  for (int k = diag[i] + 1; k < ioffset[i + 1]; ++k) zi = __dsub_rn(zi, __dmul_rn(a[k], z[ja[k]]));
  z[i] = zi * di;
}

// --- sync-free triangular sweeps ---------------------------------------------------
// The same row arithmetic as the level kernels, in one launch: warps claim 32 entries of
// the level-ordered row list (levels padded to multiples of 32, so a warp's rows are
// independent) through an atomic counter, and each row waits for the values it reads.
// The output vector is filled with a sentinel before the sweep, a signalling-NaN bit
// pattern that arithmetic never produces; a row polls the 64-bit word it needs until the
// sentinel is gone and uses the value it read, so the value is its own ready flag (an
// aligned 64-bit access is single-copy atomic) and no fence is needed.  Claims are
// monotone and a row only reads rows of earlier levels, so every awaited row was claimed
// earlier by a warp that is running: the waits end.  Each wait is bounded; one that gives
// up records FCG_ERR_TIMEOUT, and every row still writes its result so no other wait is
// held up by it.  The backward sweep writes a second vector, so a forward result is
// never mistaken for a backward one.
constexpr unsigned long long kSentinel = 0x7ff0dead0badf00dULL;

__device__ __forceinline__ double ld_relaxed64(const double *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return __longlong_as_double((long long)v);
}

__device__ __forceinline__ void st_relaxed64(double *p, double x) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p),
               "l"((unsigned long long)__double_as_longlong(x))
               : "memory");
}

__device__ __forceinline__ bool is_sentinel(double v) {
  return (unsigned long long)__double_as_longlong(v) == kSentinel;
}

// The value at p once it is not the sentinel; gives up after `spin` polls (or when
// another wait has given up) and returns what it last read.
__device__ __forceinline__ double sf_value(const double *p, const int *err, int spin, bool *ok) {
  double v = ld_relaxed64(p);
  if (!is_sentinel(v)) return v;
  for (int it = 0; it < spin; ++it) {
    if (it >= 16) __nanosleep(32);
    v = ld_relaxed64(p);
    if (!is_sentinel(v)) return v;
    if ((it & 63) == 63 && *(volatile const int *)err) break;
  }
  *ok = false;
  return v;
}

__device__ __forceinline__ void sf_fail(int *err, Scal *S) {
  if (atomicExch(err, 1) == 0) {
    S->wait_fail = 1;
    fail_status(S, FCG_ERR_TIMEOUT);
  }
}

constexpr int kSfBatch = 8;  // dependencies of a row loaded and awaited together

// Sentinel into the sweep outputs; ctl = {forward counter, backward counter, -, error}.
__global__ void k_sf_fill(int n, double *__restrict__ o1, double *__restrict__ o2, int *ctl) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl[0] = 0;
    ctl[1] = 0;
    ctl[3] = 0;
  }
  const double s = __longlong_as_double((long long)kSentinel);
  FCG_GRID_STRIDE(i, n) {
    o1[i] = s;
    if (o2) o2[i] = s;
  }
}

// One row: acc - sum a_k v_{ja_k} over k in [k0, hi), the values awaited in batches.
__device__ __forceinline__ double sf_row(double acc, int k0, int hi, const int *__restrict__ ja,
                                         const double *__restrict__ a, const double *v, int *ctl,
                                         Scal *S, int spin) {
  for (; k0 < hi; k0 += kSfBatch) {
    int jj[kSfBatch];
    double aa[kSfBatch], vv[kSfBatch];
#pragma unroll
    for (int t = 0; t < kSfBatch; ++t)
      if (k0 + t < hi) {
        jj[t] = ja[k0 + t];
        aa[t] = a[k0 + t];
      }
    bool ok = true;
#pragma unroll
    for (int t = 0; t < kSfBatch; ++t)  // all first reads in flight together
      if (k0 + t < hi) vv[t] = ld_relaxed64(&v[jj[t]]);
#pragma unroll
    for (int t = 0; t < kSfBatch; ++t)
      if (k0 + t < hi && is_sentinel(vv[t])) vv[t] = sf_value(&v[jj[t]], &ctl[3], spin, &ok);
    if (!ok) sf_fail(&ctl[3], S);
#pragma unroll
    for (int t = 0; t < kSfBatch; ++t)
      if (k0 + t < hi) acc = __dsub_rn(acc, __dmul_rn(aa[t], vv[t]));
  }
  return acc;
}

// forward: y_i = (b_i - sum_{k<diag} a_k y_{ja_k}) * d_i        (iccg.f90:248-254)
__global__ void k_fwd_sf(const int *__restrict__ rows, int len, const int *__restrict__ ioffset,
                         const int *__restrict__ ja, const int *__restrict__ diag,
                         const double *__restrict__ a, const double *__restrict__ d,
                         const double *__restrict__ b, double *y, int *ctl, Scal *S, int spin,
                         int absent) {
  if (solve_done(S)) return;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&ctl[0], 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= len) break;
    const int i = rows[base + lane];
    if (i < 0 || i == absent) continue;
    const double zi = sf_row(b[i], ioffset[i], diag[i], ja, a, y, ctl, S, spin);
    st_relaxed64(&y[i], zi * d[i]);
  }
}

// backward from the forward result y with the reference's rescale zk/(d+small) folded
// in (iccg.f90:256-265): z_i = (y_i rdi_i - sum_{k>diag} a_k z_{ja_k}) * d_i,
// rdi = 1/(d+small)
__global__ void k_bwd_sf(const int *__restrict__ rows, int len, const int *__restrict__ ioffset,
                         const int *__restrict__ ja, const int *__restrict__ diag,
                         const double *__restrict__ a, const double *__restrict__ d,
                         const double *__restrict__ rdi, const double *__restrict__ y, double *z,
                         int *ctl, Scal *S, int spin) {
  if (solve_done(S)) return;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&ctl[1], 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= len) break;
    const int i = rows[base + lane];
    if (i < 0) continue;
    const double di = d[i];
    const double zi = sf_row(y[i] * rdi[i], diag[i] + 1, ioffset[i + 1], ja, a, z, ctl, S, spin);
    st_relaxed64(&z[i], zi * di);
  }
}

// DIC / DILU factor in one launch (iccg.f90:231-237, bicgstab.f90:68-79); d holds the
// sentinel on entry.
__global__ void k_factor_sf(const int *__restrict__ rows, int len, const int *__restrict__ ioffset,
                            const int *__restrict__ ja, const int *__restrict__ diag,
                            const int *__restrict__ tpos, const double *__restrict__ a, double *d,
                            double *__restrict__ rdi, int *ctl, Scal *S, int spin, int dilu) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&ctl[0], 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= len) break;
    const int i = rows[base + lane];
    if (i < 0) continue;
    double di = a[diag[i]];
    bool ok = true;
    for (int k = ioffset[i]; k < diag[i]; ++k) {
      const double dj = sf_value(&d[ja[k]], &ctl[3], spin, &ok);
      if (dilu)
        di = __dsub_rn(di, __dmul_rn(__dmul_rn(a[k], dj), a[tpos[k]]));
      else
        di = __dsub_rn(di, __dmul_rn(__dmul_rn(a[k], a[k]), dj));
    }
    if (!ok) sf_fail(&ctl[3], S);
    const double inv = 1.0 / di;
    st_relaxed64(&d[i], inv);
    rdi[i] = 1.0 / (inv + S->small);
    if (!isfinite(inv) || di == 0.0) fail_status(S, FCG_ERR_PIVOT);
  }
}

// Factor diagonals, level by level: DIC d_i = 1/(a_ii - sum a_ik^2 d_k) (iccg.f90:
// 231-237); DILU d_i = 1/(a_ii - sum a_ik d_k a_ki) (bicgstab.f90:68-79).
__global__ void k_factor_level(const int *__restrict__ rows, int count,
                               const int *__restrict__ ioffset, const int *__restrict__ ja,
                               const int *__restrict__ diag, const int *__restrict__ tpos,
                               const double *__restrict__ a, double *__restrict__ d,
                               double *__restrict__ rdi, Scal *S, int dilu) {
  if (solve_done(S)) return;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  int i = rows[t];
  double di = a[diag[i]];
  for (int k = ioffset[i]; k < diag[i]; ++k) {
    int j = ja[k];
    if (dilu)
      di = __dsub_rn(di, __dmul_rn(__dmul_rn(a[k], d[j]), a[tpos[k]]));
    else
      di = __dsub_rn(di, __dmul_rn(__dmul_rn(a[k], a[k]), d[j]));
  }
  double inv = 1.0 / di;
  d[i] = inv;
  rdi[i] = 1.0 / (inv + S->small);
  if (!isfinite(inv) || di == 0.0) fail_status(S, FCG_ERR_PIVOT);
}

// --- wavefront-tiled sweeps on a lexicographic hex block ---------------------------
// On a mesh whose cells form an nx x ny x nz block (c->hex), the lower entries of row r are
// (when present, in CSR order) r - nx ny, r - nx, r - 1 and the upper ones r + 1, r + nx,
// r + nx ny.  A block of TX x TY threads owns a tile of TX x TY (i, j) columns and walks
// the tile's cells in the order of their wavefront (i - i0) + (j - j0) + k: at local step
// L each thread computes the cell of its column with k = L - di - dj.  The cell's
// upstream neighbour in k is the thread's own previous cell (a register); those in i and
// j inside the tile were computed one step earlier by the neighbouring threads (shared
// memory, double buffered, one barrier per step).  Only the tile's first row and column
// read cells of another tile, from global memory through the value-as-flag wait of the
// one-launch sweeps.  The backward sweep walks from the opposite corner over the upper
// entries.  Tiles are claimed through an atomic counter in an order in which a tile's
// upstream tiles come first, so a block only waits for blocks that are running.  Each
// row uses the arithmetic of the level kernels with its entries in the same order: the
// same bits.
template <int TX, int TY>
struct WaveTile {
  int ntx, nty, di, dj, p, q;
  bool col_ok;
  long long col0, step_i, step_j;
};

// Claims a tile (thread 0, broadcast); false when every tile is taken.
template <int TX, int TY, bool BWD>
__device__ __forceinline__ bool wave_claim(int nx, int ny, int *counter, WaveTile<TX, TY> &t) {
  __shared__ int tile_sh;
  if (threadIdx.x == 0) tile_sh = atomicAdd(counter, 1);
  __syncthreads();
  t.ntx = (nx + TX - 1) / TX;
  t.nty = (ny + TY - 1) / TY;
  const int tile = tile_sh;
  if (tile >= t.ntx * t.nty) return false;
  t.di = threadIdx.x % TX;
  t.dj = threadIdx.x / TX;
  t.p = (tile % t.ntx) * TX + t.di;  // column, counted from the sweep's start corner
  t.q = (tile / t.ntx) * TY + t.dj;
  t.col_ok = t.p < nx && t.q < ny;
  const int i = BWD ? nx - 1 - t.p : t.p, j = BWD ? ny - 1 - t.q : t.q;
  t.col0 = i + (long long)nx * j;
  t.step_i = BWD ? 1 : -1;
  t.step_j = BWD ? nx : -nx;
  return true;
}

// DIC (DILU) factor d = 1/(a_ii - sum a_ik^2 d_k) (1/(a_ii - sum a_ik d_k a_ki)) in the
// forward wavefront, reading the CSR directly (once per solve); also rdi = 1/(d + small).
template <int TX, int TY, bool DILU>
__global__ void __launch_bounds__(TX * TY)
    k_wave_factor(int nx, int ny, int nz, const int *__restrict__ ioffset,
                  const int *__restrict__ diag, const int *__restrict__ tpos,
                  const double *__restrict__ a, double *d, double *__restrict__ rdi, int *ctl,
                  Scal *S, int spin) {
  __shared__ double sm[2][TY][TX];
  WaveTile<TX, TY> t;
  if (!wave_claim<TX, TY, false>(nx, ny, &ctl[0], t)) return;
  const long long nxy = (long long)nx * ny;
  const int nlev = TX + TY - 2 + nz;
  double prev = 0.0;
  for (int L = 0; L < nlev; ++L) {
    const int s = L - t.di - t.dj;
    double val = 0.0;
    if (t.col_ok && s >= 0 && s < nz) {
      const long long r = t.col0 + nxy * s;
      bool ok = true;
      double vq = 0.0, vp = 0.0;
      if (t.q > 0)
        vq = t.dj > 0 ? sm[(L - 1) & 1][t.dj - 1][t.di]
                      : sf_value(&d[r + t.step_j], &ctl[3], spin, &ok);
      if (t.p > 0)
        vp = t.di > 0 ? sm[(L - 1) & 1][t.dj][t.di - 1]
                      : sf_value(&d[r + t.step_i], &ctl[3], spin, &ok);
      if (!ok) sf_fail(&ctl[3], S);
      int e = ioffset[r];
      double dd = a[diag[r]];
      auto term = [&](double v) {
        if (DILU)
          dd = __dsub_rn(dd, __dmul_rn(__dmul_rn(a[e], v), a[tpos[e]]));
        else
          dd = __dsub_rn(dd, __dmul_rn(__dmul_rn(a[e], a[e]), v));
        ++e;
      };
      if (s > 0) term(prev);  // CSR order of the lower entries: k, j, i
      if (t.q > 0) term(vq);
      if (t.p > 0) term(vp);
      val = 1.0 / dd;
      st_relaxed64(&d[r], val);
      rdi[r] = 1.0 / (val + S->small);
      if (!isfinite(val) || dd == 0.0) fail_status(S, FCG_ERR_PIVOT);
      prev = val;
    }
    sm[L & 1][t.dj][t.di] = val;
    __syncthreads();
  }
}

// Coefficient planes of the sweeps from the CSR values: lo[t][r] for the lower entries in
// CSR order (-nx ny, -nx, -1) and up[t][r] for the upper ones (+1, +nx, +nx ny), 0 where the
// row has no such entry (the sweeps skip those terms).
__global__ void k_wave_coef(int nx, int ny, int nz, const int *__restrict__ ioffset,
                            const int *__restrict__ diag, const double *__restrict__ a,
                            double *__restrict__ lo, double *__restrict__ up) {
  const long long nxy = (long long)nx * ny, n = nxy * nz;
  FCG_GRID_STRIDE(r, n) {
    const int i = (int)(r % nx), j = (int)((r / nx) % ny), k = (int)(r / nxy);
    int e = ioffset[r];
    lo[r] = k > 0 ? a[e++] : 0.0;
    lo[n + r] = j > 0 ? a[e++] : 0.0;
    lo[2 * n + r] = i > 0 ? a[e++] : 0.0;
    e = diag[r] + 1;
    up[r] = i < nx - 1 ? a[e++] : 0.0;
    up[n + r] = j < ny - 1 ? a[e++] : 0.0;
    up[2 * n + r] = k < nz - 1 ? a[e++] : 0.0;
  }
}

// Forward sweep y = (b - L y) d (BWD false) or backward sweep z = (y rdi - U z) d (BWD
// true).  The inputs of a cell (its three coefficients, right-hand side, d, rdi, and for a
// column on the tile's first row or column the upstream value of the neighbouring tile)
// are loaded kRing steps ahead into a register ring whose slot is the step modulo kRing,
// so every slot index is a compile-time constant of the unrolled step loop.  An upstream
// value that was still the sentinel when loaded is then waited for.
//
// The step is branch-free: a neighbour outside the block has coefficient +0 (k_wave_coef)
// and value +0, and acc - (+0)(+0) is acc exactly, so every cell runs the same three
// terms in CSR order and gives the bits of the level kernels.  On this part a dependent
// FP64 operation takes about 64 cycles, so the step's length is its chain of FP64
// operations: the term of the cell's own column (the previous step of the same thread)
// is formed before the barrier, which leaves the two products and subtractions of the
// in-tile neighbours and the scaling after it.
template <int TX, int TY, bool BWD>
__global__ void __launch_bounds__(TX * TY)
    k_wave_sweep(int nx, int ny, int nz, const double *__restrict__ coef,
                 const double *__restrict__ in, const double *__restrict__ d,
                 const double *__restrict__ rdi, double *out, int *ctl, Scal *S, int spin) {
  constexpr int kRing = 4;
  if (solve_done(S)) return;
  __shared__ double sm[2][TY][TX];
  WaveTile<TX, TY> t;
  if (!wave_claim<TX, TY, BWD>(nx, ny, &ctl[BWD ? 1 : 0], t)) return;
  const long long nxy = (long long)nx * ny, n = nxy * nz;
  const bool edge_q = t.q > 0 && t.dj == 0, edge_p = t.p > 0 && t.di == 0;
  auto row_of = [&](int s) { return t.col0 + nxy * (BWD ? nz - 1 - s : s); };
  // Only loads here: an instruction that used a loaded value would hold the warp's
  // in-order issue until the load returned.
  struct Cell {
    double c0, c1, c2, x, dd, sc, eq, ep;
  };
  Cell ring[kRing];
  auto load = [&](int s, Cell &cl) {
    if (!t.col_ok || s < 0 || s >= nz) return;
    const long long r = row_of(s);
    cl.c0 = coef[r];
    cl.c1 = coef[n + r];
    cl.c2 = coef[2 * n + r];
    cl.x = in[r];
    cl.dd = d[r];
    if (BWD) cl.sc = rdi[r];
    if (edge_q) cl.eq = ld_relaxed64(&out[r + t.step_j]);
    if (edge_p) cl.ep = ld_relaxed64(&out[r + t.step_i]);
  };
  // The terms of the next step's cell that do not need the neighbours' values, formed
  // before the barrier: forward x - c0 prev (k first in CSR order); backward y rdi and the
  // product c2 prev (k last).
  double part = 0.0, part2 = 0.0;
  auto own = [&](const Cell &cl, double prev) {
    if (BWD) {
      part = cl.x * cl.sc;
      part2 = __dmul_rn(cl.c2, prev);
    } else {
      part = __dsub_rn(cl.x, __dmul_rn(cl.c0, prev));
    }
  };
#pragma unroll
  for (int u = 0; u < kRing; ++u) load(u - t.di - t.dj, ring[u]);
  const int nlev = TX + TY - 2 + nz;
  double prev = 0.0;  // +0: the first cell of a column has no own-column neighbour
  own(ring[0], prev);
  for (int L0 = 0; L0 < nlev; L0 += kRing) {
#pragma unroll
    for (int u = 0; u < kRing; ++u) {
      const int L = L0 + u;
      if (L < nlev) {  // the same for the whole block
        const int s = L - t.di - t.dj;
        double val = 0.0;
        if (t.col_ok && s >= 0 && s < nz) {
          const long long r = row_of(s);
          const Cell cl = ring[u];
          bool ok = true;
          const double sq = sm[(L - 1) & 1][t.dj > 0 ? t.dj - 1 : 0][t.di];
          const double sp = sm[(L - 1) & 1][t.dj][t.di > 0 ? t.di - 1 : 0];
          double vq = t.dj > 0 ? sq : (edge_q ? cl.eq : 0.0);
          double vp = t.di > 0 ? sp : (edge_p ? cl.ep : 0.0);
          if (edge_q && is_sentinel(vq)) vq = sf_value(&out[r + t.step_j], &ctl[3], spin, &ok);
          if (edge_p && is_sentinel(vp)) vp = sf_value(&out[r + t.step_i], &ctl[3], spin, &ok);
          if (!ok) sf_fail(&ctl[3], S);
          double acc;
          if (!BWD) {  // lower entries in CSR order: k, j, i
            acc = __dsub_rn(part, __dmul_rn(cl.c1, vq));
            acc = __dsub_rn(acc, __dmul_rn(cl.c2, vp));
          } else {  // upper entries in CSR order: i, j, k
            acc = __dsub_rn(part, __dmul_rn(cl.c0, vp));
            acc = __dsub_rn(acc, __dmul_rn(cl.c1, vq));
            acc = __dsub_rn(acc, part2);
          }
          val = acc * cl.dd;
          st_relaxed64(&out[r], val);
          prev = val;
        }
        load(s + kRing, ring[u]);
        sm[L & 1][t.dj][t.di] = val;
        own(ring[(u + 1) % kRing], prev);
        __syncthreads();
      }
    }
  }
}

// --- BiCGStab sweep (bicgstab.f90:99-224) -------------------------------------
// bet = sum res*reso; om = bet*gam/(alf*beto+small); beto = bet
__global__ void __launch_bounds__(kTPB, 8) k_bi_dot1(int n, const double *__restrict__ res, const double *__restrict__ reso,
                          Scal *S, double *partials) {
  if (solve_done(S)) return;
  double v[1] = {0.0};
  FCG_GRID_STRIDE(i, n) v[0] += res[i] * reso[i];
  if (reduce_commit<1>(v, partials, &S->ticket[3]) && threadIdx.x == 0) {
    double bet = v[0];
    S->bbet = bet;
    S->om = bet * S->gam / (S->alf * S->beto + S->small);
    S->beto = bet;
  }
}

// pk = res + om*(pk - alf*uk)
__global__ void __launch_bounds__(kTPB, 8) k_bi_p(int n, const double *__restrict__ res, const double *__restrict__ uk,
                       double *__restrict__ pk, const Scal *S) {
  if (solve_done(S)) return;
  const double om = __ldcg(&S->om), alf = __ldcg(&S->alf);
  FCG_GRID_STRIDE(i, n) pk[i] = res[i] + om * (pk[i] - alf * uk[i]);
}

// uk = A zk; gam = bet / sum uk*reso
__global__ void __launch_bounds__(kTPB, 8) k_bi_spmv1(SellView s, int n, const double *__restrict__ val,
                           const double *__restrict__ zk, const double *__restrict__ reso,
                           double *__restrict__ uk, Scal *S, double *partials) {
  if (solve_done(S)) return;
  double v[1] = {0.0};
  FCG_SLICE_LOOP(slice, lane, s) {
    int r = slice * 32 + lane;
    double u = sell_row(s, n, val, zk, slice, lane);
    if (r < n) {
      uk[r] = u;
      v[0] += u * reso[r];
    }
  }
  if (reduce_commit<1>(v, partials, &S->ticket[4]) && threadIdx.x == 0) {
    S->gam = S->bbet / v[0];
    if (!isfinite(S->gam)) fail_status(S, FCG_ERR_NONFINITE);
  }
}

// fi += gam*zk; res -= gam*uk
__global__ void __launch_bounds__(kTPB, 8) k_bi_upd1(int n, double *__restrict__ x, double *__restrict__ res,
                          const double *__restrict__ zk, const double *__restrict__ uk,
                          const Scal *S) {
  if (solve_done(S)) return;
  const double gam = __ldcg(&S->gam);
  FCG_GRID_STRIDE(i, n) {
    x[i] = x[i] + gam * zk[i];
    res[i] = res[i] - gam * uk[i];
  }
}

// vk = A zk; alf = sum vk*res / (sum vk*vk + small)
__global__ void __launch_bounds__(kTPB, 8) k_bi_spmv2(SellView s, int n, const double *__restrict__ val,
                           const double *__restrict__ zk, const double *__restrict__ res,
                           double *__restrict__ vk, Scal *S, double *partials) {
  if (solve_done(S)) return;
  double v[2] = {0.0, 0.0};
  FCG_SLICE_LOOP(slice, lane, s) {
    int r = slice * 32 + lane;
    double q = sell_row(s, n, val, zk, slice, lane);
    if (r < n) {
      vk[r] = q;
      v[0] += q * res[r];
      v[1] += q * q;
    }
  }
  if (reduce_commit<2>(v, partials, &S->ticket[5]) && threadIdx.x == 0) {
    S->alf = v[0] / (v[1] + S->small);
    if (!isfinite(S->alf)) fail_status(S, FCG_ERR_NONFINITE);
  }
}

__device__ __noinline__ void bi_close_sweep(Scal *S, double resl, double *trace,
                                            cudaGraphConditionalHandle h, int use_cond) {
  if (S->status) {
    S->done = 1;
    if (use_cond) cudaGraphSetConditional(h, 0);
    return;
  }
  finish_sweep(S, resl, trace, h, use_cond);
}

// fi += alf*zk; res -= alf*vk; resl = sum|res|; stop test
__global__ void __launch_bounds__(kTPB, 8) k_bi_upd2(int n, double *__restrict__ x, double *__restrict__ res,
                          const double *__restrict__ zk, const double *__restrict__ vk, Scal *S,
                          double *partials, double *trace, cudaGraphConditionalHandle h,
                          int use_cond) {
  if (solve_done(S)) {
    stop_loop(h, use_cond);
    return;
  }
  loop_guard(S, h, use_cond);
  const double alf = __ldcg(&S->alf);
  double v[1] = {0.0};
  FCG_GRID_STRIDE(i, n) {
    x[i] = x[i] + alf * zk[i];
    double r = res[i] - alf * vk[i];
    res[i] = r;
    v[0] += fabs(r);
  }
  if (reduce_commit<1>(v, partials, &S->ticket[6]) && threadIdx.x == 0)
    bi_close_sweep(S, v[0], trace, h, use_cond);
}

// ---------------------------------------------------------------------------
// Mixed precision: CG on D^-1/2 A D^-1/2 (Jacobi preconditioning folded into a
// symmetric scaling) in FP32, with reliable updates (Clark et al. 2010, "Solving lattice
// QCD systems of equations using mixed precision solvers on GPUs"): the FP32 recursion
// keeps its direction p, and whenever ||r32|| has dropped by `delta` since the last true
// residual, or the predicted L1 residual reaches the tolerance, the FP32 correction is
// added to the FP64 solution and the residual is recomputed in FP64, su - A x.  The stop
// test is the reference's L1-relative one, evaluated on that true residual only.
// Dot products: FP32 products summed per thread in FP32 (a few dozen terms), then in
// FP64 across threads, blocks and the grid.
// ---------------------------------------------------------------------------
__global__ void k_mx_scale(int n, const int *__restrict__ diag, const double *__restrict__ a,
                           double *__restrict__ s64) {
  FCG_GRID_STRIDE(i, n) s64[i] = 1.0 / sqrt(a[diag[i]]);
}

__global__ void k_mx_fill(SellView s, int n, const double *__restrict__ a,
                          const double *__restrict__ s64, float *__restrict__ sv32) {
  FCG_GRID_STRIDE(r, (long long)s.nslices * 32) {
    int slice = (int)(r >> 5), lane = (int)(r & 31);
    long long base = s.ptr[slice];
    int w = s.width[slice], op = s.offp[slice];
    double sr = r < n ? s64[r] : 0.0;
    for (int j = 0; j < w; ++j) {
      long long p = base + (long long)j * 32 + lane;
      int src = s.src[p];
      int c = s.kind[slice] == 0 ? (int)r + s.off[op + j] : s.off[op + 32 * j + lane];
      c = c < 0 ? 0 : (c >= n ? n - 1 : c);
      sv32[p] = src >= 0 ? (float)(a[src] * sr * s64[c]) : 0.0f;
    }
  }
}

// r32 = D^-1/2 res, y32 = 0, p32 = r32, rr = r32.r32
__global__ void __launch_bounds__(kTPB, 6)
    k_mx_start(int n, const double *__restrict__ res, const double *__restrict__ s64,
               float *__restrict__ r32, float *__restrict__ y32, float *__restrict__ p32, Scal *S,
               double *partials) {
  float t = 0.f;
  FCG_GRID_STRIDE(i, n) {
    float r = (float)(s64[i] * res[i]);
    r32[i] = r;
    p32[i] = r;
    y32[i] = 0.f;
    t += r * r;
  }
  double v[1] = {(double)t};
  if (reduce_commit<1>(v, partials, &S->ticket[3]) && threadIdx.x == 0) {
    S->rr = v[0];
    S->maxr = sqrt(v[0]);
    S->l1ratio = v[0] > 0 ? S->res0 / sqrt(v[0]) : 0.0;
    S->ru = 0;
    S->nupdates = 0;
  }
}

// q32 = Ahat p32, alf = rr / p.q.  Each block walks a contiguous run of slices, eight
// at a time (one per warp), so that the gathers of x at row, row+-1 and row+-N that one
// step makes are L1 hits of the steps just before and after it; only the +-N^2
// neighbours come from L2.
__global__ void __launch_bounds__(kTPB, 6)
    k_mx_spmv(SellView s, int n, const float *__restrict__ val, const float *__restrict__ p32,
              float *__restrict__ q32, Scal *S, double *partials) {
  if (solve_done(S)) return;
  float t = 0.f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int per = (s.nslices + gridDim.x - 1) / gridDim.x;
  const int sbeg = blockIdx.x * per, send = min(s.nslices, sbeg + per);
  for (int slice = sbeg + warp; slice < send; slice += kTPB / 32) {
    const float q = sell_row(s, n, val, p32, slice, lane);
    const int r = slice * 32 + lane;
    if (r < n) {
      q32[r] = q;
      t += p32[r] * q;
    }
  }
  double v[1] = {(double)t};
  if (reduce_commit<1>(v, partials, &S->ticket[1]) && threadIdx.x == 0) {
    S->alf = S->rr / v[0];
    if (!isfinite(S->alf)) fail_status(S, FCG_ERR_NONFINITE);
  }
}

__device__ __noinline__ void mx_decide(Scal *S, double rrn) {
  int it = S->iter + 1;
  S->iter = it;
  double nr = sqrt(rrn);
  double pred = S->l1ratio * nr;  // predicted L1 of the unscaled residual
  bool ru = nr < S->delta * S->maxr || pred < 0.9 * S->resmax * (S->res0 + S->small) ||
            it >= S->nsw || !isfinite(rrn);
  S->rr_old = S->rr;
  if (ru) {
    S->ru = 1;
  } else {
    S->bet = rrn / S->rr;
    S->rr = rrn;
  }
}

// y32 += alf p32, r32 -= alf q32, rr' = r32.r32; decides whether a reliable update
// follows and, inside the graph, arms the IF node that runs it.  float4 accesses.
__global__ void __launch_bounds__(kTPB, 6)
    k_mx_update(int n, float *__restrict__ y32, float *__restrict__ r32,
                const float *__restrict__ p32, const float *__restrict__ q32, Scal *S,
                double *partials, cudaGraphConditionalHandle hif, int use_cond) {
  if (solve_done(S)) return;
  const float alf = (float)__ldcg(&S->alf);
  float t = 0.f;
  const long long n4 = n >> 2;
  FCG_GRID_STRIDE(i, n4) {
    float4 y = reinterpret_cast<float4 *>(y32)[i], r = reinterpret_cast<float4 *>(r32)[i];
    const float4 p = reinterpret_cast<const float4 *>(p32)[i];
    const float4 q = reinterpret_cast<const float4 *>(q32)[i];
    y.x += alf * p.x; y.y += alf * p.y; y.z += alf * p.z; y.w += alf * p.w;
    r.x -= alf * q.x; r.y -= alf * q.y; r.z -= alf * q.z; r.w -= alf * q.w;
    reinterpret_cast<float4 *>(y32)[i] = y;
    reinterpret_cast<float4 *>(r32)[i] = r;
    t += r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w;
  }
  FCG_GRID_STRIDE(j, n - 4 * n4) {
    long long i = 4 * n4 + j;
    y32[i] = y32[i] + alf * p32[i];
    float r = r32[i] - alf * q32[i];
    r32[i] = r;
    t += r * r;
  }
  double v[1] = {(double)t};
  if (reduce_commit<1>(v, partials, &S->ticket[2]) && threadIdx.x == 0) {
    mx_decide(S, v[0]);
    if (use_cond) cudaGraphSetConditional(hif, S->ru ? 1u : 0u);
  }
}

// reliable update, part 1: x += D^-1/2 y32 in FP64, y32 = 0
__global__ void k_mx_ru1(int n, double *__restrict__ x, float *__restrict__ y32,
                         const double *__restrict__ s64, const Scal *S) {
  if (solve_done(S) || !__ldcg(&S->ru)) return;
  FCG_GRID_STRIDE(i, n) {
    x[i] = x[i] + s64[i] * (double)y32[i];
    y32[i] = 0.f;
  }
}

__device__ __noinline__ void mx_after_update(Scal *S, double l1, double rrn, double *trace,
                                             cudaGraphConditionalHandle h, int use_cond) {
  S->resl = l1;
  if (S->iter >= 1 && S->resor == 0.0) S->resor = S->res0;
  double rsm = l1 / (S->res0 + S->small);
  S->rsm = rsm;
  S->nupdates++;
  if (trace && S->nupdates <= S->trace_cap) {
    trace[2 * (S->nupdates - 1)] = l1;
    trace[2 * (S->nupdates - 1) + 1] = rsm;
  }
  if (rsm < S->resmax) S->converged = 1;
  if (!isfinite(l1)) fail_status(S, FCG_ERR_NONFINITE);
  if (S->converged || S->iter >= S->nsw || S->status) {
    S->done = 1;
    if (use_cond) cudaGraphSetConditional(h, 0);
    return;
  }
  S->bet = rrn / S->rr_old;  // continue the recursion with the true residual
  S->rr = rrn;
  S->maxr = sqrt(rrn);
  S->l1ratio = rrn > 0 ? l1 / sqrt(rrn) : 0.0;
  S->ru = 0;
}

// reliable update, part 2: res = su - A x (FP64), L1 of it, r32 = D^-1/2 res, rr
__global__ void __launch_bounds__(kTPB, 8)
    k_mx_ru2(SellView s, int n, const double *__restrict__ val, const double *__restrict__ su,
             const double *__restrict__ x, double *__restrict__ res,
             const double *__restrict__ s64, float *__restrict__ r32, Scal *S, double *partials,
             double *trace, cudaGraphConditionalHandle h, int use_cond) {
  if (solve_done(S) || !__ldcg(&S->ru)) return;
  double l1 = 0.0;
  float t = 0.f;
  FCG_SLICE_LOOP(slice, lane, s) {
    int r = slice * 32 + lane;
    double ax = sell_row(s, n, val, x, slice, lane);
    if (r < n) {
      double rr = su[r] - ax;
      res[r] = rr;
      l1 += fabs(rr);
      float r3 = (float)(s64[r] * rr);
      r32[r] = r3;
      t += r3 * r3;
    }
  }
  double v[2] = {l1, (double)t};
  if (reduce_commit<2>(v, partials, &S->ticket[4]) && threadIdx.x == 0)
    mx_after_update(S, v[0], v[1], trace, h, use_cond);
}

// p32 = r32 + bet p32; closes the loop body (float4 accesses)
__global__ void __launch_bounds__(kTPB, 6)
    k_mx_p(int n, const float *__restrict__ r32, float *__restrict__ p32, Scal *S,
           cudaGraphConditionalHandle h, int use_cond) {
  if (solve_done(S)) {
    stop_loop(h, use_cond);
    return;
  }
  loop_guard(S, h, use_cond);
  const float bet = (float)__ldcg(&S->bet);
  const long long n4 = n >> 2;
  FCG_GRID_STRIDE(i, n4) {
    const float4 r = reinterpret_cast<const float4 *>(r32)[i];
    float4 p = reinterpret_cast<float4 *>(p32)[i];
    p.x = r.x + bet * p.x; p.y = r.y + bet * p.y; p.z = r.z + bet * p.z; p.w = r.w + bet * p.w;
    reinterpret_cast<float4 *>(p32)[i] = p;
  }
  FCG_GRID_STRIDE(j, n - 4 * n4) {
    long long i = 4 * n4 + j;
    p32[i] = r32[i] + bet * p32[i];
  }
}

// Final FP64 check: ||su - A x||^2 and ||su||^2.
__global__ void __launch_bounds__(kTPB, 8) k_final(SellView s, int n, const double *__restrict__ val,
                        const double *__restrict__ su, const double *__restrict__ x, Scal *S,
                        double *partials, OcView o) {
  double v[2] = {0.0, 0.0};
  FCG_SLICE_LOOP(slice, lane, s) {
    int r = slice * 32 + lane;
    double ax = sell_row(s, n, val, x, slice, lane);
    if (r < n) {
      double rr = su[r] - ax;
      if (o.ptr) rr = oc_sub(o, r, rr, x);
      v[0] += rr * rr;
      v[1] += su[r] * su[r];
    }
  }
  if (reduce_commit<2>(v, partials, &S->ticket[7]) && threadIdx.x == 0) {
    S->l2r = v[0];
    S->l2b = v[1];
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int ensure_state(fcg_context *c, int nsw) {
  KrylovState *k = c->ks;
  if (!k) {
    k = c->ks = new KrylovState();
    FCG_CUDA_TRY(c, cudaMalloc(&k->S, sizeof(Scal)));
    FCG_CUDA_TRY(c, cudaMallocHost(&k->hS, sizeof(Scal)));
    FCG_CUDA_TRY(c, cudaMemset(k->S, 0, sizeof(Scal)));
    FCG_CUDA_TRY(c, cudaStreamCreateWithFlags(&k->cap, cudaStreamNonBlocking));
    FCG_CUDA_TRY(c, cudaEventCreate(&k->ev0));
    FCG_CUDA_TRY(c, cudaEventCreate(&k->ev1));
  }
  const int G = c->num_sms * 8;
  if (k->n != c->n || k->nnz != c->nnz || k->sell_len != c->sell_len || k->G != G ||
      k->bind_gen != c->bind_gen) {
    for (int i = 0; i < SK_N; ++i) {
      if (k->exec[i]) cudaGraphExecDestroy(k->exec[i]);
      if (k->graph[i]) cudaGraphDestroy(k->graph[i]);
      k->exec[i] = nullptr;
      k->graph[i] = nullptr;
    }
    const size_t n = c->n;
    size_t total = 14 * n + (size_t)a_len(c) + (size_t)c->sell_len + 8 * (size_t)G + 64;
    FCG_CUDA_TRY(c, k->vec.ensure(total * sizeof(double)));
    FCG_CUDA_TRY(c, cudaMemset(k->vec.p, 0, total * sizeof(double)));
    if (c->hex.ok) {
      FCG_CUDA_TRY(c, k->wcoef.ensure(6 * n * sizeof(double)));
      k->wlo = k->wcoef.as<double>();
      k->wup = k->wlo + 3 * n;
    } else {
      k->wcoef.release();
      k->wlo = k->wup = nullptr;
    }
    double *p = k->vec.as<double>();
    double **vecs[] = {&k->x, &k->res, &k->su, &k->pk, &k->zk, &k->qk, &k->invd,
                       &k->d, &k->reso, &k->uk, &k->vk, &k->rtmp, &k->rdi};
    for (double **v : vecs) {
      *v = p;
      p += n;
    }
    p += n;  // guard
    k->a = p;  // the CSR values, then the O-C pairs' ar and al
    p += a_len(c);
    k->sval = p;
    p += c->sell_len;
    k->partials = p;
    k->n = c->n;
    k->nnz = c->nnz;
    k->sell_len = c->sell_len;
    k->G = G;
    auto occ = [&](const void *fn) {
      int b = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, kTPB, 0) != cudaSuccess) {
        cudaGetLastError();
        b = 1;
      }
      return c->num_sms * std::max(1, std::min(b, 8));
    };
    Grids &g = k->gr;
    g.init = occ((const void *)k_init);
    g.p = occ((const void *)k_cg_p);
    g.spmv = occ((const void *)k_cg_spmv);
    g.update = occ((const void *)k_cg_update);
    g.dot = occ((const void *)k_cg_dot);
    g.bdot = occ((const void *)k_bi_dot1);
    g.bp = occ((const void *)k_bi_p);
    g.bspmv1 = occ((const void *)k_bi_spmv1);
    g.bupd1 = occ((const void *)k_bi_upd1);
    g.bspmv2 = occ((const void *)k_bi_spmv2);
    g.bupd2 = occ((const void *)k_bi_upd2);
    g.fin = occ((const void *)k_final);
    g.plain = occ((const void *)k_spmv);
    g.mstart = occ((const void *)k_mx_start);
    g.mspmv = occ((const void *)k_mx_spmv);
    g.mupd = occ((const void *)k_mx_update);
    g.mru1 = occ((const void *)k_mx_ru1);
    g.mru2 = occ((const void *)k_mx_ru2);
    g.mp = occ((const void *)k_mx_p);
    // sync-free sweeps: the forward result vector and the control words
    FCG_CUDA_TRY(c, k->sfb.ensure(sizeof(double) * (n + 4)));
    FCG_CUDA_TRY(c, cudaMemset(k->sfb.p, 0, sizeof(double) * (n + 4)));
    k->sf_y = k->sfb.as<double>();
    k->sf_ctl = (int *)(k->sf_y + n);
    k->sf_grid = std::min(occ((const void *)k_fwd_sf), occ((const void *)k_bwd_sf));
    {
      // FCG_SWEEP=levels: one launch per level; =rows: the row-claiming one-launch form
      // on every mesh; default: the wavefront-tiled form on hex blocks, rows elsewhere
      const char *e = std::getenv("FCG_SWEEP");
      k->sf_on = !(e && std::string(e) == "levels");
      k->wave_on = !(e && (std::string(e) == "levels" || std::string(e) == "rows"));
      // 16 x 8 tiles while 8 x 8 ones would number fewer than two per SM; FCG_WAVE_TILE
      // (8x8 or 16x8) overrides
      const char *wt = std::getenv("FCG_WAVE_TILE");
      const long long t88 = (long long)((c->hex.nx + 7) / 8) * ((c->hex.ny + 7) / 8);
      k->wave_wide = wt ? std::string(wt) == "16x8" : t88 < 2LL * c->num_sms;
      // two blocks per SM: more resident warps only poll further ahead (measured)
      k->sf_grid = std::min(k->sf_grid, c->num_sms * 2);
    }
    k->bind_gen = c->bind_gen;
    k->matrix_loaded = false;
    k->mixed_ready = false;
  }
  if (nsw > k->nsw_cap) {
    FCG_CUDA_TRY(c, k->trace.ensure(sizeof(double) * 2 * (size_t)nsw));
    k->nsw_cap = nsw;
    for (int i = 0; i < SK_N; ++i) {  // the trace pointer is baked into the graphs
      if (k->exec[i]) cudaGraphExecDestroy(k->exec[i]);
      if (k->graph[i]) cudaGraphDestroy(k->graph[i]);
      k->exec[i] = nullptr;
      k->graph[i] = nullptr;
    }
  }
  return FCG_OK;
}

// Loads CSR values a (device pointer) into the solver copies.
// The O-C couplings of the matrix load_matrix() placed in the state (none: ptr null).
static OcView oc_view(const fcg_context *c) {
  const MeshView &m = c->mv;
  if (!m.noc) return OcView{nullptr, nullptr, nullptr, nullptr};
  return OcView{m.oc_cptr, m.oc_col, m.oc_vix, c->ks->a + c->nnz};
}

static int load_matrix(fcg_context *c, const double *da) {
  KrylovState *k = c->ks;
  FCG_CUDA_TRY(c, cudaMemcpyAsync(k->a, da, sizeof(double) * a_len(c), cudaMemcpyDeviceToDevice,
                                  c->stream));
  k_sell_fill<<<grid_for((long long)c->sv.nslices * 32, c->num_sms), kTPB, 0, c->stream>>>(
      c->sv, c->n, c->mv.diag, k->a, k->sval, k->invd);
  FCG_CHECK_LAUNCH(c, "k_sell_fill");
  k->matrix_loaded = true;
  return FCG_OK;
}

// FP32 copy of D^-1/2 A D^-1/2 in the sliced layout and D^-1/2 in FP64, from the
// matrix load_matrix() placed in the state (used by the mixed and learned solvers).
int build_scaled32(fcg_context *c) {
  KrylovState *k = c->ks;
  if (!k->mixed_ready) {
    size_t n4 = ((size_t)c->n + 63) & ~(size_t)63;
    size_t bytes = sizeof(double) * n4 + sizeof(float) * (4 * n4 + (size_t)c->sell_len + 64);
    FCG_CUDA_TRY(c, k->mixed.ensure(bytes));
    k->s64 = k->mixed.as<double>();
    float *f = (float *)(k->s64 + n4);
    k->y32 = f;
    k->r32 = f + n4;
    k->p32 = f + 2 * n4;
    k->q32 = f + 3 * n4;
    k->sval32 = f + 4 * n4;
    k->mixed_ready = true;
    if (k->exec[SK_MIXED]) cudaGraphExecDestroy(k->exec[SK_MIXED]);  // buffers moved: recapture
    if (k->graph[SK_MIXED]) cudaGraphDestroy(k->graph[SK_MIXED]);
    k->exec[SK_MIXED] = nullptr;
    k->graph[SK_MIXED] = nullptr;
  }
  k_mx_scale<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(c->n, c->mv.diag, k->a, k->s64);
  k_mx_fill<<<grid_for((long long)c->sv.nslices * 32, c->num_sms), kTPB, 0, c->stream>>>(
      c->sv, c->n, k->a, k->s64, k->sval32);
  FCG_CHECK_LAUNCH(c, "scaled FP32 matrix");
  return FCG_OK;
}

int prepare_scaled32(fcg_context *c, const double *a_dev) {
  int rc = ensure_state(c, 1);
  if (rc) return rc;
  if ((rc = load_matrix(c, a_dev))) return rc;
  return build_scaled32(c);
}

int batch_load(fcg_context *c, const double *a_dev, const double *su_dev, const double *fi_dev,
               BatchVecs *out) {
  int rc = ensure_state(c, 1);
  if (rc) return rc;
  KrylovState *k = c->ks;
  if (a_dev) {
    if ((rc = load_matrix(c, a_dev))) return rc;
  } else if (!k->matrix_loaded) {
    return set_error(c, FCG_ERR_STATE, "batched solve with a == NULL before a matrix was loaded");
  }
  const size_t n1 = sizeof(double) * c->n;
  FCG_CUDA_TRY(c, cudaMemcpyAsync(k->su, su_dev, n1, cudaMemcpyDeviceToDevice, c->stream));
  FCG_CUDA_TRY(c, cudaMemcpyAsync(k->x, fi_dev, n1, cudaMemcpyDeviceToDevice, c->stream));
  FCG_CUDA_TRY(c, cudaMemsetAsync(k->pk, 0, n1, c->stream));
  out->val = k->sval;
  out->invd = k->invd;
  out->su = k->su;
  out->x = k->x;
  out->res = k->res;
  out->p = k->pk;
  out->q = k->qk;
  return FCG_OK;
}

const float *scaled32(const fcg_context *c) { return c->ks ? c->ks->sval32 : nullptr; }
const double *scale64(const fcg_context *c) { return c->ks ? c->ks->s64 : nullptr; }
const double *sliced64(const fcg_context *c) { return c->ks ? c->ks->sval : nullptr; }

// The wavefront-tiled form runs on hex blocks, unless a test hook asks for a row that
// never publishes (only the row-claiming form has one).
static bool wave_sweeps(const fcg_context *c) {
  const KrylovState *k = c->ks;
  return k->sf_on && k->wave_on && c->hex.ok && k->wlo && k->sf_absent_row < 0;
}

// Tiles of 16 x 8 or 8 x 8 columns (64 or 128 threads per block).  Measured on 20 ICCG
// sweeps: at 128^3 (256 tiles of 8 x 8) 16 x 8 tiles are 4% faster, at 256^3 (1024 tiles of
// 8 x 8) 8 x 8 tiles are 11% faster, where enough tiles are in flight to keep the SMs'
// FP64 units busy.
template <int TX, int TY>
static int wave_tiles(const fcg_context *c) {
  return ((c->hex.nx + TX - 1) / TX) * ((c->hex.ny + TY - 1) / TY);
}

template <int TX, int TY>
static void launch_wave_sweep(fcg_context *c, cudaStream_t st, bool forward, const double *b,
                              double *z) {
  KrylovState *k = c->ks;
  const HexBlock &h = c->hex;
  if (forward)
    k_wave_sweep<TX, TY, false><<<wave_tiles<TX, TY>(c), TX * TY, 0, st>>>(
        h.nx, h.ny, h.nz, k->wlo, b, k->d, k->rdi, k->sf_y, k->sf_ctl, k->S, k->sf_spin);
  else
    k_wave_sweep<TX, TY, true><<<wave_tiles<TX, TY>(c), TX * TY, 0, st>>>(
        h.nx, h.ny, h.nz, k->wup, k->sf_y, k->d, k->rdi, z, k->sf_ctl, k->S, k->sf_spin);
}

template <int TX, int TY>
static void launch_wave_factor(fcg_context *c, bool dilu) {
  KrylovState *k = c->ks;
  const HexBlock &h = c->hex;
  if (dilu)
    k_wave_factor<TX, TY, true><<<wave_tiles<TX, TY>(c), TX * TY, 0, c->stream>>>(
        h.nx, h.ny, h.nz, c->mv.ioffset, c->mv.diag, c->tpos, k->a, k->d, k->rdi, k->sf_ctl,
        k->S, k->sf_spin);
  else
    k_wave_factor<TX, TY, false><<<wave_tiles<TX, TY>(c), TX * TY, 0, c->stream>>>(
        h.nx, h.ny, h.nz, c->mv.ioffset, c->mv.diag, c->tpos, k->a, k->d, k->rdi, k->sf_ctl,
        k->S, k->sf_spin);
}

static void launch_sweeps(fcg_context *c, cudaStream_t st, const Level &lv, bool forward,
                          const double *b, double *z) {
  KrylovState *k = c->ks;
  if (k->sf_on) {
    const bool wave = wave_sweeps(c);
    auto wave_launch = [&](bool fwd) {
      if (k->wave_wide)
        launch_wave_sweep<16, 8>(c, st, fwd, b, z);
      else
        launch_wave_sweep<8, 8>(c, st, fwd, b, z);
    };
    if (forward) {  // b -> sf_y, after the sentinel fill of sf_y and z
      k_sf_fill<<<grid_for(c->n, c->num_sms), kTPB, 0, st>>>(c->n, k->sf_y, z, k->sf_ctl);
      if (wave)
        wave_launch(true);
      else
        k_fwd_sf<<<k->sf_grid, kTPB, 0, st>>>(lv.pad, lv.pad_len, c->mv.ioffset, c->mv.ja,
                                              c->mv.diag, k->a, k->d, b, k->sf_y, k->sf_ctl,
                                              k->S, k->sf_spin, k->sf_absent_row);
    } else {  // sf_y -> z
      if (wave)
        wave_launch(false);
      else
        k_bwd_sf<<<k->sf_grid, kTPB, 0, st>>>(lv.pad, lv.pad_len, c->mv.ioffset, c->mv.ja,
                                              c->mv.diag, k->a, k->d, k->rdi, k->sf_y, z,
                                              k->sf_ctl, k->S, k->sf_spin);
    }
    return;
  }
  for (int l = 0; l < lv.count; ++l) {
    int start = lv.ptr[l], cnt = lv.ptr[l + 1] - lv.ptr[l];
    int g = (cnt + kTPB - 1) / kTPB;
    if (forward)
      k_fwd_level<<<g, kTPB, 0, st>>>(lv.rows + start, cnt, c->mv.ioffset, c->mv.ja, c->mv.diag,
                                      k->a, k->d, b, z, k->S);
    else
      k_bwd_level<<<g, kTPB, 0, st>>>(lv.rows + start, cnt, c->mv.ioffset, c->mv.ja, c->mv.diag,
                                      k->a, k->d, k->rdi, z, k->S);
  }
}

// Kernels of one sweep, in order, as units (a unit of a DIC/DILU sweep is the whole
// chain of level launches).  Unit names are listed in sweep_unit_names().
static int sweep_units(int kind) {
  switch (kind) {
    case SK_DPCG: return 3;
    case SK_ICCG: return 6;
    case SK_BICG: return 10;
    case SK_MIXED: return 5;
  }
  return 0;
}

static const char *sweep_unit_name(int kind, int u) {
  static const char *dpcg[] = {"k_cg_p", "k_cg_spmv", "k_cg_update"};
  static const char *iccg[] = {"fwd_levels", "bwd_levels", "k_cg_dot", "k_cg_p", "k_cg_spmv",
                               "k_cg_update"};
  static const char *bicg[] = {"k_bi_dot1", "k_bi_p", "fwd_levels", "bwd_levels", "k_bi_spmv1",
                               "k_bi_upd1", "fwd_levels", "bwd_levels", "k_bi_spmv2", "k_bi_upd2"};
  static const char *mixed[] = {"k_mx_spmv", "k_mx_update", "k_mx_ru1", "k_mx_ru2", "k_mx_p"};
  if (u < 0 || u >= sweep_units(kind)) return "";
  switch (kind) {
    case SK_DPCG: return dpcg[u];
    case SK_ICCG: return iccg[u];
    case SK_BICG: return bicg[u];
    default: return mixed[u];
  }
}

// Enqueues unit u of one sweep of solver `kind` on stream st.
static void enqueue_unit(fcg_context *c, cudaStream_t st, int kind, int u,
                         cudaGraphConditionalHandle h, int use_cond,
                         cudaGraphConditionalHandle hif = 0) {
  KrylovState *k = c->ks;
  const int n = c->n;
  const SellView &s = c->sv;
  double *tr = k->trace.as<double>();
  if (kind == SK_DPCG || kind == SK_ICCG) {
    int v = kind == SK_DPCG ? u + 3 : u;
    switch (v) {
      case 0: launch_sweeps(c, st, c->lf, true, k->res, k->zk); break;
      case 1: launch_sweeps(c, st, c->lb, false, nullptr, k->zk); break;
      case 2: k_cg_dot<<<k->gr.dot, kTPB, 0, st>>>(n, k->res, k->zk, k->S, k->partials); break;
      case 3:
        k_cg_p<<<k->gr.p, kTPB, 0, st>>>(n, k->res, k->invd, k->zk, k->pk, k->S, kind);
        break;
      case 4:
        k_cg_spmv<<<k->gr.spmv, kTPB, 0, st>>>(s, n, k->sval, k->pk, k->qk, k->S, k->partials,
                                               oc_view(c));
        break;
      case 5:
        k_cg_update<<<k->gr.update, kTPB, 0, st>>>(n, k->x, k->res, k->pk, k->qk, k->invd, k->S,
                                                   k->partials, tr, h, use_cond, kind);
        break;
    }
  } else if (kind == SK_MIXED) {
    switch (u) {
      case 0:
        k_mx_spmv<<<k->gr.mspmv, kTPB, 0, st>>>(s, n, k->sval32, k->p32, k->q32, k->S,
                                                 k->partials);
        break;
      case 1:
        k_mx_update<<<k->gr.mupd, kTPB, 0, st>>>(n, k->y32, k->r32, k->p32, k->q32, k->S,
                                                 k->partials, hif, use_cond);
        break;
      case 2: k_mx_ru1<<<k->gr.mru1, kTPB, 0, st>>>(n, k->x, k->y32, k->s64, k->S); break;
      case 3:
        // sets only the stop flag: k_mx_p, after the IF node, ends the WHILE loop
        k_mx_ru2<<<k->gr.mru2, kTPB, 0, st>>>(s, n, k->sval, k->su, k->x, k->res, k->s64, k->r32,
                                              k->S, k->partials, tr, h, 0);
        break;
      case 4: k_mx_p<<<k->gr.mp, kTPB, 0, st>>>(n, k->r32, k->p32, k->S, h, use_cond); break;
    }
  } else {
    switch (u) {
      case 0: k_bi_dot1<<<k->gr.bdot, kTPB, 0, st>>>(n, k->res, k->reso, k->S, k->partials); break;
      case 1: k_bi_p<<<k->gr.bp, kTPB, 0, st>>>(n, k->res, k->uk, k->pk, k->S); break;
      case 2: launch_sweeps(c, st, c->lf, true, k->pk, k->zk); break;
      case 3: launch_sweeps(c, st, c->lb, false, nullptr, k->zk); break;
      case 4:
        k_bi_spmv1<<<k->gr.bspmv1, kTPB, 0, st>>>(s, n, k->sval, k->zk, k->reso, k->uk, k->S,
                                                   k->partials);
        break;
      case 5: k_bi_upd1<<<k->gr.bupd1, kTPB, 0, st>>>(n, k->x, k->res, k->zk, k->uk, k->S); break;
      case 6: launch_sweeps(c, st, c->lf, true, k->res, k->zk); break;
      case 7: launch_sweeps(c, st, c->lb, false, nullptr, k->zk); break;
      case 8:
        k_bi_spmv2<<<k->gr.bspmv2, kTPB, 0, st>>>(s, n, k->sval, k->zk, k->res, k->vk, k->S,
                                                   k->partials);
        break;
      case 9:
        k_bi_upd2<<<k->gr.bupd2, kTPB, 0, st>>>(n, k->x, k->res, k->zk, k->vk, k->S, k->partials,
                                                tr, h, use_cond);
        break;
    }
  }
}

// Enqueues one sweep of solver `kind` on stream st.
static void enqueue_sweep(fcg_context *c, cudaStream_t st, int kind, cudaGraphConditionalHandle h,
                          int use_cond) {
  for (int u = 0; u < sweep_units(kind); ++u) enqueue_unit(c, st, kind, u, h, use_cond);
}

static bool graphs_disabled() {
  const char *e = std::getenv("FCG_NO_GRAPH");
  return e && e[0] == '1';
}

// Captures the WHILE-node graph of one solver kind.
static int build_graph(fcg_context *c, int kind) {
  KrylovState *k = c->ks;
  if (k->exec[kind]) return FCG_OK;
  cudaGraph_t g;
  FCG_CUDA_TRY(c, cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  FCG_CUDA_TRY(c, cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};  // aggregate: rest zeroed
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  FCG_CUDA_TRY(c, cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  FCG_CUDA_TRY(c, cudaStreamBeginCaptureToGraph(k->cap, body, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal));
  cudaGraph_t captured = nullptr;
  cudaError_t e = cudaSuccess;
  if (kind == SK_MIXED) {
    // body: spmv -> update -> IF(reliable update){ ru1 -> ru2 } -> p
    cudaGraphConditionalHandle hif;
    FCG_CUDA_TRY(c, cudaGraphConditionalHandleCreate(&hif, body, 0, cudaGraphCondAssignDefault));
    enqueue_unit(c, k->cap, kind, 0, h, 1);
    enqueue_unit(c, k->cap, kind, 1, h, 1, hif);
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    FCG_CUDA_TRY(c, cudaStreamGetCaptureInfo(k->cap, &cs, nullptr, nullptr, &deps, nullptr, &nd));
    cudaGraphNodeParams ip = {cudaGraphNodeTypeConditional};
    ip.conditional.handle = hif;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t ifnode;
    FCG_CUDA_TRY(c, cudaGraphAddNode(&ifnode, body, deps, nullptr, nd, &ip));
    FCG_CUDA_TRY(c, cudaStreamUpdateCaptureDependencies(k->cap, &ifnode, nullptr, 1,
                                                        cudaStreamSetCaptureDependencies));
    enqueue_unit(c, k->cap, kind, 4, h, 1);
    e = cudaStreamEndCapture(k->cap, &captured);
    if (e == cudaSuccess) {
      FCG_CUDA_TRY(c, cudaStreamBeginCaptureToGraph(k->cap, ip.conditional.phGraph_out[0], nullptr,
                                                    nullptr, 0, cudaStreamCaptureModeThreadLocal));
      enqueue_unit(c, k->cap, kind, 2, h, 1);
      enqueue_unit(c, k->cap, kind, 3, h, 1);
      e = cudaStreamEndCapture(k->cap, &captured);
    }
  } else {
    enqueue_sweep(c, k->cap, kind, h, 1);
    e = cudaStreamEndCapture(k->cap, &captured);
  }
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(c, e, "capture of the solver sweep");
  }
  e = cudaGraphInstantiate(&k->exec[kind], g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(c, e, "cudaGraphInstantiate (solver)");
  }
  k->graph[kind] = g;
  return FCG_OK;
}

static int run_solver(fcg_context *c, int kind, const double *a, const double *su, double *fi,
                      double *res, double sor, int nsw, double *resor, fcg_solve_report *rep) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "solver called before fcg_bind_mesh");
  if (!a || !su || !fi) return set_error(c, FCG_ERR_ARG, "NULL a, su or fi");
  if (nsw < 0) return set_error(c, FCG_ERR_ARG, "nsw must be >= 0");
  if (kind == SK_MIXED && c->mv.noc) return refuse_oc(c, "fcg_dpcg_mixed");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = ensure_state(c, nsw > 0 ? nsw : 1);
  if (rc) return rc;
  KrylovState *k = c->ks;
  const size_t n1 = sizeof(double) * c->n;
  void *da, *dsu, *dfi;
  bool ha, hsu, hfi;
  if ((rc = stage_in(c, a, sizeof(double) * a_len(c), 0, true, &da, &ha))) return rc;
  if ((rc = stage_in(c, su, n1, 1, true, &dsu, &hsu))) return rc;
  if ((rc = stage_in(c, fi, n1, 2, true, &dfi, &hfi))) return rc;
  FCG_CUDA_TRY(c, cudaEventRecord(k->ev0, c->stream));
  if ((rc = load_matrix(c, (const double *)da))) return rc;
  FCG_CUDA_TRY(c, cudaMemcpyAsync(k->su, dsu, n1, cudaMemcpyDeviceToDevice, c->stream));
  FCG_CUDA_TRY(c, cudaMemcpyAsync(k->x, dfi, n1, cudaMemcpyDeviceToDevice, c->stream));
  FCG_CUDA_TRY(c, cudaMemsetAsync(k->pk, 0, n1, c->stream));
  FCG_CUDA_TRY(c, cudaMemsetAsync(k->uk, 0, n1, c->stream));
  // Scalars for this solve.
  Scal init;
  std::memset(&init, 0, sizeof init);
  init.nsw = nsw;
  init.small = k->small;
  init.early = k->early_exit;
  init.resmax = sor;
  init.tol = (double)1e-13f;  // dpcg.f90:37
  init.trace_cap = k->nsw_cap;
  init.delta = k->ru_delta;
  *k->hS = init;
  FCG_CUDA_TRY(c, cudaMemcpyAsync(k->S, k->hS, sizeof(Scal), cudaMemcpyHostToDevice, c->stream));
  k_init<<<k->gr.init, kTPB, 0, c->stream>>>(c->sv, c->n, k->sval, k->su, k->x, k->res, k->invd, k->S,
                                    k->partials, kind, oc_view(c));
  FCG_CHECK_LAUNCH(c, "k_init");
  if (kind == SK_BICG)
    FCG_CUDA_TRY(c, cudaMemcpyAsync(k->reso, k->res, n1, cudaMemcpyDeviceToDevice, c->stream));
  if (kind == SK_MIXED) {
    if ((rc = build_scaled32(c))) return rc;
    k_mx_start<<<k->gr.mstart, kTPB, 0, c->stream>>>(c->n, k->res, k->s64, k->r32, k->y32,
                                                     k->p32, k->S, k->partials);
    FCG_CHECK_LAUNCH(c, "mixed set-up");
  }
  if (kind != SK_DPCG && k->sf_on) {  // factor diagonal in one sync-free launch
    k_sf_fill<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(c->n, k->d, nullptr,
                                                                    k->sf_ctl);
    if (wave_sweeps(c)) {
      const HexBlock &h = c->hex;
      k_wave_coef<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(
          h.nx, h.ny, h.nz, c->mv.ioffset, c->mv.diag, k->a, k->wlo, k->wup);
      if (k->wave_wide)
        launch_wave_factor<16, 8>(c, kind == SK_BICG);
      else
        launch_wave_factor<8, 8>(c, kind == SK_BICG);
    } else {
      k_factor_sf<<<k->sf_grid, kTPB, 0, c->stream>>>(
          c->lf.pad, c->lf.pad_len, c->mv.ioffset, c->mv.ja, c->mv.diag, c->tpos, k->a, k->d,
          k->rdi, k->sf_ctl, k->S, k->sf_spin, kind == SK_BICG);
    }
    FCG_CHECK_LAUNCH(c, "factor");
  } else if (kind != SK_DPCG) {  // factor diagonal, level by level
    for (int l = 0; l < c->lf.count; ++l) {
      int start = c->lf.ptr[l], cnt = c->lf.ptr[l + 1] - c->lf.ptr[l];
      k_factor_level<<<(cnt + kTPB - 1) / kTPB, kTPB, 0, c->stream>>>(
          c->lf.rows + start, cnt, c->mv.ioffset, c->mv.ja, c->mv.diag, c->tpos, k->a, k->d,
          k->rdi, k->S,
          kind == SK_BICG);
    }
    FCG_CHECK_LAUNCH(c, "k_factor_level");
  }
  if (!graphs_disabled()) {
    if ((rc = build_graph(c, kind))) return rc;
    FCG_CUDA_TRY(c, cudaGraphLaunch(k->exec[kind], c->stream));
  } else {
    // Host-driven loop: chunks of sweeps, stop flag read back between chunks.
    for (int done = 0, it = 0; !done && it <= nsw; it += 16) {
      for (int j = 0; j < 16; ++j) enqueue_sweep(c, c->stream, kind, 0, 0);
      FCG_CHECK_LAUNCH(c, "solver sweep");
      FCG_CUDA_TRY(c, cudaMemcpyAsync(k->hS, k->S, sizeof(Scal), cudaMemcpyDeviceToHost, c->stream));
      FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      done = k->hS->done;
    }
  }
  k_final<<<k->gr.fin, kTPB, 0, c->stream>>>(c->sv, c->n, k->sval, k->su, k->x, k->S, k->partials,
                                             oc_view(c));
  FCG_CHECK_LAUNCH(c, "k_final");
  FCG_CUDA_TRY(c, cudaEventRecord(k->ev1, c->stream));
  FCG_CUDA_TRY(c, cudaMemcpyAsync(dfi, k->x, n1, cudaMemcpyDeviceToDevice, c->stream));
  if ((rc = stage_out(c, fi, dfi, n1, hfi))) return rc;
  if (res) {
    void *dres;
    bool hres;
    if ((rc = stage_in(c, res, n1, 3, false, &dres, &hres))) return rc;
    FCG_CUDA_TRY(c, cudaMemcpyAsync(dres, k->res, n1, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = stage_out(c, res, dres, n1, hres))) return rc;
  }
  FCG_CUDA_TRY(c, cudaMemcpyAsync(k->hS, k->S, sizeof(Scal), cudaMemcpyDeviceToHost, c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const Scal &S = *k->hS;
  k->last_kind = kind;
  if (resor && S.iter > 0) *resor = S.res0;  // dpcg.f90:139
  if (rep) {
    rep->res0 = S.res0;
    rep->resl = S.resl;
    rep->iters = S.iter;
    rep->converged = S.converged;
    rep->l2_rel = S.l2b > 0 ? std::sqrt(S.l2r / S.l2b) : std::sqrt(S.l2r);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, k->ev0, k->ev1);
    rep->seconds = ms * 1e-3;
  }
  if (S.status) {
    const char *what = S.status == FCG_ERR_PIVOT     ? "zero or non-finite pivot in the factor"
                       : S.status == FCG_ERR_TIMEOUT
                           ? (S.wait_fail ? "a triangular-sweep dependency wait gave up"
                                          : "solver loop exceeded nsw + 2 sweeps")
                                                     : "non-finite value in a reduction";
    return set_error(c, S.status, what);
  }
  return FCG_OK;
}

}  // namespace fcg

using namespace fcg;

extern "C" int fcg_dpcg(fcg_context *c, const double *a, const double *su, double *fi,
                        double *res, double sor, int nsw, double *resor, fcg_solve_report *rep) {
  return run_solver(c, SK_DPCG, a, su, fi, res, sor, nsw, resor, rep);
}

extern "C" int fcg_iccg(fcg_context *c, const double *a, const double *su, double *fi,
                        double *res, double sor, int nsw, double *resor, fcg_solve_report *rep) {
  return run_solver(c, SK_ICCG, a, su, fi, res, sor, nsw, resor, rep);
}

extern "C" int fcg_bicgstab(fcg_context *c, const double *a, const double *su, double *fi,
                            double *res, double sor, int nsw, double *resor,
                            fcg_solve_report *rep) {
  return run_solver(c, SK_BICG, a, su, fi, res, sor, nsw, resor, rep);
}

extern "C" int fcg_dpcg_mixed(fcg_context *c, const double *a, const double *su, double *fi,
                              double *res, double sor, int nsw, double *resor,
                              fcg_solve_report *rep) {
  return run_solver(c, SK_MIXED, a, su, fi, res, sor, nsw, resor, rep);
}

extern "C" int fcg_set_solver_options(fcg_context *c, double small, int early_exit) {
  if (!c) return FCG_ERR_ARG;
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = ensure_state(c, 1);
  if (rc) return rc;
  c->ks->small = small;
  c->ks->early_exit = early_exit ? 1 : 0;
  return FCG_OK;
}

extern "C" int fcg_set_sweep_wait_test(fcg_context *c, int polls, int absent_row) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_set_sweep_wait_test before fcg_bind_mesh");
  if (absent_row < 0 || absent_row > c->n) return set_error(c, FCG_ERR_INDEX, "absent_row out of range");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = ensure_state(c, 1);
  if (rc) return rc;
  KrylovState *k = c->ks;
  k->sf_spin = polls > 0 ? polls : (1 << 20);
  k->sf_absent_row = absent_row - 1;
  for (int i = 0; i < SK_N; ++i) {  // both values are kernel arguments of the graphs
    if (k->exec[i]) cudaGraphExecDestroy(k->exec[i]);
    if (k->graph[i]) cudaGraphDestroy(k->graph[i]);
    k->exec[i] = nullptr;
    k->graph[i] = nullptr;
  }
  return FCG_OK;
}

// Re-opens the last solve for profiling: clears the stop flag, the reliable-update
// flag and the sweep counters, and lifts the sweep cap.
__global__ void k_prof_reopen(Scal *S) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S->done = 0;
    S->ru = 0;
    S->status = 0;
    S->wait_fail = 0;
    S->converged = 0;
    S->iter = 0;
    S->body_count = 0;
    S->nsw = 0x3fffffff;
    S->resmax = 0.0;  // never converges: every profiled sweep does its full work
  }
}

extern "C" int fcg_profile_sweeps(fcg_context *c, int reps, double *ms, int max_units,
                                  int *units) {
  if (!c || reps < 1) return FCG_ERR_ARG;
  if (!c->ks || c->ks->last_kind < 0)
    return set_error(c, FCG_ERR_STATE, "fcg_profile_sweeps before any solve");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  KrylovState *k = c->ks;
  const int kind = k->last_kind, nu = sweep_units(kind);
  if (units) *units = nu;
  std::vector<cudaEvent_t> ev(2 * nu);
  for (auto &e : ev) FCG_CUDA_TRY(c, cudaEventCreate(&e));
  std::vector<double> acc(nu, 0.0);
  k_prof_reopen<<<1, 32, 0, c->stream>>>(k->S);
  for (int r = 0; r < reps; ++r) {
    for (int u = 0; u < nu; ++u) {
      cudaEventRecord(ev[2 * u], c->stream);
      enqueue_unit(c, c->stream, kind, u, 0, 0);
      cudaEventRecord(ev[2 * u + 1], c->stream);
    }
    FCG_CHECK_LAUNCH(c, "profiled sweep");
    FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    for (int u = 0; u < nu; ++u) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[2 * u], ev[2 * u + 1]);
      acc[u] += t;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  for (int u = 0; u < nu && u < max_units; ++u)
    if (ms) ms[u] = acc[u] / reps;
  return FCG_OK;
}

extern "C" const char *fcg_profile_unit_name(const fcg_context *c, int unit) {
  if (!c || !c->ks || c->ks->last_kind < 0) return "";
  return sweep_unit_name(c->ks->last_kind, unit);
}

extern "C" int fcg_get_solver_trace(fcg_context *c, double *out, int max_count, int *count) {
  if (!c || !c->ks) return FCG_ERR_STATE;
  // the mixed solver records one entry per FP64 reliable update, the others one per sweep
  const int written = c->ks->last_kind == SK_MIXED ? c->ks->hS->nupdates : c->ks->hS->iter;
  int avail = std::min(written, c->ks->nsw_cap);
  int m = std::min(avail, max_count);
  if (count) *count = avail;
  if (out && m > 0)
    FCG_CUDA_TRY(c, cudaMemcpy(out, c->ks->trace.p, sizeof(double) * 2 * m, cudaMemcpyDeviceToHost));
  return FCG_OK;
}

extern "C" int fcg_spmv(fcg_context *c, const double *a, const double *x, double *y) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_spmv before fcg_bind_mesh");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = ensure_state(c, 1);
  if (rc) return rc;
  KrylovState *k = c->ks;
  const size_t n1 = sizeof(double) * c->n;
  if (a) {
    void *da;
    bool ha;
    if ((rc = stage_in(c, a, sizeof(double) * a_len(c), 0, true, &da, &ha))) return rc;
    if ((rc = load_matrix(c, (const double *)da))) return rc;
  } else if (!k->matrix_loaded) {
    return set_error(c, FCG_ERR_STATE, "fcg_spmv with a == NULL before any matrix was loaded");
  }
  void *dx, *dy;
  bool hx, hy;
  if ((rc = stage_in(c, x, n1, 1, true, &dx, &hx))) return rc;
  if ((rc = stage_in(c, y, n1, 2, false, &dy, &hy))) return rc;
  k_spmv<<<k->gr.plain, kTPB, 0, c->stream>>>(c->sv, c->n, k->sval, (const double *)dx, (double *)dy,
                                              oc_view(c));
  FCG_CHECK_LAUNCH(c, "k_spmv");
  if ((rc = stage_out(c, y, dy, n1, hy))) return rc;
  if (hy) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}
