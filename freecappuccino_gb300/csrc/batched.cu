// Batched DPCG: several independent pressure solves of uneven sizes -- each bound to its
// own context (mesh, sliced matrix) -- in one persistent cooperative kernel, captured in
// a CUDA graph.  No reference counterpart as a batch: every system follows dpcg.f90:3-154
// exactly as fcg_dpcg does (same recurrence, constants and L1 stop test per system).
//
// Work is a list of items (system, run of 32-row slices).  The kernel walks all systems
// in lockstep phases -- initial residual; then per CG iteration p-update | SpMV | update
// -- separated by a grid-wide barrier; the items of a phase are spread over the CTAs, so
// a large system uses the whole GPU and small ones share it.  Each system's global sums
// are formed deterministically: every item stores its block partial, and the CTA that
// commits the system's last item (ticket counter) adds the partials in item order with a
// fixed block tree and updates that system's scalars.  A system that meets its stop test
// drops out (its items are skipped); the kernel ends when none is left.
//
// The grid barrier spins with a bounded number of polls; a CTA that gives up sets the
// error flag, which ends every CTA at its next barrier, and the call returns
// FCG_ERR_TIMEOUT.  The item size (slices per item) and the CTAs per SM are picked by
// fcg_batch_autotune, which times every candidate on the caller's systems.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "fcg_internal.h"
#include "krylov_common.cuh"
#include "launch.h"

namespace fcg {
namespace {

constexpr int kMaxBatch = 64;

// One system of the batch (device-resident; the host writes the inputs before a solve).
struct BSys {
  SellView sv;
  int n, item0, nitems, nsw;
  const double *val, *invd, *su;
  double *x, *res, *p, *q;
  double sor, small, tol;
  double res0, resl, sk, s0, bet, alf, l2r, l2b;
  int iter, active, converged, status, early, pad;
  unsigned int ticket, pad2;
};

struct BItem {
  int sys, s0, s1;  // slices [s0, s1) of system sys
};

struct BCtl {
  unsigned int count, gen;  // grid barrier
  int err;                  // 1: a barrier wait gave up, 2: loop bound exceeded
  int nactive;              // systems still iterating
};

// Grid-wide barrier with a bounded wait.  Returns false when any CTA has given up.
__device__ bool grid_sync(BCtl *ctl, long long limit) {
  __shared__ int ok_sh;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned int *vgen = &ctl->gen;
    volatile int *verr = &ctl->err;
    if (*verr) {
      ok = 0;
    } else {
      const unsigned int g = *vgen;
      __threadfence();
      const unsigned int arrived = atomicAdd(&ctl->count, 1u);
      if (arrived == gridDim.x - 1) {
        ctl->count = 0u;
        __threadfence();
        atomicAdd(&ctl->gen, 1u);
      } else {
        long long polls = 0;
        while (*vgen == g) {
          if (*verr) {
            ok = 0;
            break;
          }
          if (++polls > limit) {
            atomicExch(&ctl->err, 1);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
    }
    __threadfence();
    ok_sh = ok;
  }
  __syncthreads();
  __threadfence();
  return ok_sh != 0;
}

// Row sum of A x for lane `lane` of slice `slice` (FP64, slot order = CSR column order).
// x is written by other CTAs between phases, so it is read with plain coherent loads.
__device__ __forceinline__ double brow(const SellView &s, int n, const double *__restrict__ val,
                                       const double *x, int slice, int lane) {
  const long long base = __ldg(&s.ptr[slice]) + lane;
  const int w = __ldg(&s.width[slice]), op = __ldg(&s.offp[slice]);
  double acc = 0.0;
  if (__ldg(&s.kind[slice]) == 0) {
    const int row = slice * 32 + lane;
    for (int j = 0; j < w; ++j) {
      int c = row + __ldg(&s.off[op + j]);
      c = c < 0 ? 0 : (c >= n ? n - 1 : c);
      acc += __ldg(&val[base + (long long)j * 32]) * x[c];
    }
  } else {
    for (int j = 0; j < w; ++j)
      acc += __ldg(&val[base + (long long)j * 32]) * x[__ldg(&s.off[op + 32 * j + lane])];
  }
  return acc;
}

// Stores this item's block sums; in the CTA that commits the system's last item, returns
// true with the system's totals in v (all threads), summed over the items in order.
template <int NV>
__device__ bool item_commit(double (&v)[NV], double *part, int it, BSys &S,
                            double (*sh)[kWarps]) {
  __shared__ int last_sh;
  block_sum<NV>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) part[(long long)it * 2 + k] = v[k];
    __threadfence();
    const unsigned int t = atomicAdd(&S.ticket, 1u);
    last_sh = (t == (unsigned int)S.nitems - 1u);
  }
  __syncthreads();
  if (!last_sh) return false;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) s[k] = 0.0;
  for (int j = threadIdx.x; j < S.nitems; j += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] += __ldcg(&part[(long long)(S.item0 + j) * 2 + k]);
  block_sum<NV>(s, sh);
  if (threadIdx.x == 0) {
    S.ticket = 0u;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = s[k];
  }
  return true;
}

__device__ __noinline__ void fin_init(BSys &S, BCtl *ctl, double l1, double sk) {
  S.res0 = l1;
  S.resl = l1;
  S.iter = 0;
  S.s0 = (double)1.e20f;  // dpcg.f90:76
  S.sk = sk;
  S.bet = sk / S.s0;
  S.converged = 0;
  if (!isfinite(l1)) S.status = FCG_ERR_NONFINITE;
  S.active = !(S.nsw <= 0 || (S.early && l1 < S.tol) || S.status);  // dpcg.f90:66-70
  if (!S.active) atomicSub(&ctl->nactive, 1);
}

__device__ __noinline__ void fin_spmv(BSys &S, double pq) {
  S.alf = S.sk / pq;  // dpcg.f90:119-121
  if (!isfinite(S.alf)) {
    S.status = FCG_ERR_NONFINITE;
    S.alf = 0.0;
  }
}

__device__ __noinline__ void fin_update(BSys &S, BCtl *ctl, double resl, double sk_new) {
  const int it = S.iter + 1;
  S.iter = it;
  S.resl = resl;
  S.s0 = S.sk;  // dpcg.f90:132
  S.sk = sk_new;
  S.bet = sk_new / S.s0;
  if (resl / (S.res0 + S.small) < S.sor) S.converged = 1;  // dpcg.f90:139-142
  if (!isfinite(resl)) S.status = FCG_ERR_NONFINITE;
  if (S.converged || it >= S.nsw || S.status) {
    S.active = 0;
    atomicSub(&ctl->nactive, 1);
  }
}

__global__ void __launch_bounds__(kTPB)
    k_batch_dpcg(BSys *sys, const BItem *__restrict__ items, int nitems, double *part,
                 BCtl *ctl, int max_loops, long long spin_limit, int absent_block) {
  __shared__ double sh[2][kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // diagnostics only (fcg_batch_set_wait_test): one CTA never reaches a barrier, so the
  // others' bounded waits run out and the solve ends with FCG_ERR_TIMEOUT
  if ((int)blockIdx.x == absent_block) return;
  // initial residual res = su - A x, res0 = sum|res|, sk = sum res^2 / a_PP (dpcg.f90:51-90)
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const BItem I = items[it];
    BSys &S = sys[I.sys];
    double v[2] = {0.0, 0.0};
    for (int slice = I.s0 + warp; slice < I.s1; slice += kWarps) {
      const int r = slice * 32 + lane;
      const double ax = brow(S.sv, S.n, S.val, S.x, slice, lane);
      if (r < S.n) {
        const double rr = S.su[r] - ax;
        S.res[r] = rr;
        v[0] += fabs(rr);
        v[1] += rr * (rr * __ldg(&S.invd[r]));
      }
    }
    if (item_commit<2>(v, part, it, S, sh) && threadIdx.x == 0) fin_init(S, ctl, v[0], v[1]);
  }
  if (!grid_sync(ctl, spin_limit)) return;
  for (int loop = 0;; ++loop) {
    if (__ldcg(&ctl->nactive) <= 0) break;
    if (loop > max_loops) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(&ctl->err, 2);
      return;
    }
    // p = a_PP^-1 res + bet p (dpcg.f90:85-100)
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
      const BItem I = items[it];
      BSys &S = sys[I.sys];
      if (!__ldcg(&S.active)) continue;
      const double bet = __ldcg(&S.bet);
      const int r0 = I.s0 * 32, r1 = min(S.n, I.s1 * 32);
      for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x)
        S.p[r] = S.res[r] * __ldg(&S.invd[r]) + bet * S.p[r];
    }
    if (!grid_sync(ctl, spin_limit)) return;
    // q = A p, alf = sk / p.q (dpcg.f90:105-121)
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
      const BItem I = items[it];
      BSys &S = sys[I.sys];
      if (!__ldcg(&S.active)) continue;
      double v[2] = {0.0, 0.0};
      for (int slice = I.s0 + warp; slice < I.s1; slice += kWarps) {
        const int r = slice * 32 + lane;
        const double q = brow(S.sv, S.n, S.val, S.p, slice, lane);
        if (r < S.n) {
          S.q[r] = q;
          v[0] += S.p[r] * q;
        }
      }
      if (item_commit<2>(v, part, it, S, sh) && threadIdx.x == 0) fin_spmv(S, v[0]);
    }
    if (!grid_sync(ctl, spin_limit)) return;
    // x += alf p, res -= alf q, resl = sum|res|, next sk (dpcg.f90:124-142)
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
      const BItem I = items[it];
      BSys &S = sys[I.sys];
      if (!__ldcg(&S.active)) continue;
      const double alf = __ldcg(&S.alf);
      double v[2] = {0.0, 0.0};
      for (int slice = I.s0 + warp; slice < I.s1; slice += kWarps) {
        const int r = slice * 32 + lane;
        if (r < S.n) {
          S.x[r] = S.x[r] + alf * S.p[r];
          const double rr = S.res[r] - alf * S.q[r];
          S.res[r] = rr;
          v[0] += fabs(rr);
          v[1] += rr * (rr * __ldg(&S.invd[r]));
        }
      }
      if (item_commit<2>(v, part, it, S, sh) && threadIdx.x == 0)
        fin_update(S, ctl, v[0], v[1]);
    }
    if (!grid_sync(ctl, spin_limit)) return;
  }
  // final FP64 check of every system: ||su - A x||^2, ||su||^2
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const BItem I = items[it];
    BSys &S = sys[I.sys];
    double v[2] = {0.0, 0.0};
    for (int slice = I.s0 + warp; slice < I.s1; slice += kWarps) {
      const int r = slice * 32 + lane;
      const double ax = brow(S.sv, S.n, S.val, S.x, slice, lane);
      if (r < S.n) {
        const double rr = S.su[r] - ax;
        v[0] += rr * rr;
        v[1] += S.su[r] * S.su[r];
      }
    }
    if (item_commit<2>(v, part, it, S, sh) && threadIdx.x == 0) {
      S.l2r = v[0];
      S.l2b = v[1];
    }
  }
}

}  // namespace
}  // namespace fcg

using namespace fcg;

struct fcg_batch {
  std::vector<fcg_context *> ctx;
  int device = 0, num_sms = 0, occ = 1;
  cudaStream_t stream = nullptr;
  std::string err;
  int slices_per_item = 32, blocks_per_sm = 2;
  DBuf dsys, ditems, dpart, dctl;
  BSys *hsys = nullptr;  // pinned: the graph copies it to the device at every launch
  BCtl *hctl = nullptr;
  int nitems = 0, items_for = -1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_grid = 0, graph_loops = 0;
  long long spin_limit = 1LL << 22;  // polls of 64 ns sleeps per barrier wait: over 0.25 s
  int absent_block = -1;              // diagnostics: a CTA that skips the barriers
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

int bfail(fcg_batch *b, int status, const std::string &msg) {
  if (b) b->err = msg;
  return status;
}

#define B_TRY(b, expr)                                                                    \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess)                                                                \
      return bfail((b), FCG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

void drop_graph(fcg_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// Items of `slices_per_item` slices for every system, system after system.
int build_items(fcg_batch *b) {
  if (b->items_for == b->slices_per_item) return FCG_OK;
  std::vector<BItem> items;
  for (size_t k = 0; k < b->ctx.size(); ++k) {
    const int ns = b->ctx[k]->sv.nslices;
    b->hsys[k].item0 = (int)items.size();
    for (int s0 = 0; s0 < ns; s0 += b->slices_per_item)
      items.push_back({(int)k, s0, std::min(ns, s0 + b->slices_per_item)});
    b->hsys[k].nitems = (int)items.size() - b->hsys[k].item0;
  }
  b->nitems = (int)items.size();
  B_TRY(b, b->ditems.ensure(sizeof(BItem) * items.size()));
  B_TRY(b, b->dpart.ensure(sizeof(double) * 2 * items.size()));
  B_TRY(b, cudaMemcpy(b->ditems.p, items.data(), sizeof(BItem) * items.size(),
                      cudaMemcpyHostToDevice));
  b->items_for = b->slices_per_item;
  drop_graph(b);
  return FCG_OK;
}

int grid_size(const fcg_batch *b) { return b->num_sms * std::min(b->blocks_per_sm, b->occ); }

// Enqueues one batched solve on b->stream: inputs of hsys, control block, the kernel.
int enqueue(fcg_batch *b, cudaStream_t st, int grid, int max_loops) {
  const size_t ns = b->ctx.size();
  B_TRY(b, cudaMemcpyAsync(b->dsys.p, b->hsys, sizeof(BSys) * ns, cudaMemcpyHostToDevice, st));
  B_TRY(b, cudaMemcpyAsync(b->dctl.p, b->hctl, sizeof(BCtl), cudaMemcpyHostToDevice, st));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kTPB);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  B_TRY(b, cudaLaunchKernelEx(&cfg, k_batch_dpcg, b->dsys.as<BSys>(),
                              (const BItem *)b->ditems.as<BItem>(), b->nitems,
                              b->dpart.as<double>(), b->dctl.as<BCtl>(), max_loops,
                              b->spin_limit, b->absent_block));
  return FCG_OK;
}

bool graphs_off() {
  const char *e = std::getenv("FCG_NO_GRAPH");
  return e && e[0] == '1';
}

// Runs the batch on the systems already loaded (hsys filled); times it with events.
int run(fcg_batch *b, int max_loops, float *ms) {
  int rc = build_items(b);
  if (rc) return rc;
  const int grid = grid_size(b);
  b->hctl->count = 0;
  b->hctl->gen = 0;
  b->hctl->err = 0;
  b->hctl->nactive = (int)b->ctx.size();
  B_TRY(b, cudaEventRecord(b->ev0, b->stream));
  if (graphs_off()) {
    if ((rc = enqueue(b, b->stream, grid, max_loops))) return rc;
  } else {
    if (!b->exec || b->graph_grid != grid || b->graph_loops != max_loops) {
      drop_graph(b);
      cudaStream_t cap;
      B_TRY(b, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
      cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        rc = enqueue(b, cap, grid, max_loops);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(cap, &g);
        if (!rc && e == cudaSuccess) {
          e = cudaGraphInstantiate(&b->exec, g, 0);
          if (e == cudaSuccess) b->graph = g;
          else cudaGraphDestroy(g);
        } else if (g) {
          cudaGraphDestroy(g);
        }
      }
      cudaStreamDestroy(cap);
      if (rc) return rc;
      if (e != cudaSuccess)
        return bfail(b, FCG_ERR_CUDA, std::string("capture of the batched solve: ") +
                                          cudaGetErrorString(e));
      b->graph_grid = grid;
      b->graph_loops = max_loops;
    }
    B_TRY(b, cudaGraphLaunch(b->exec, b->stream));
  }
  B_TRY(b, cudaEventRecord(b->ev1, b->stream));
  B_TRY(b, cudaMemcpyAsync(b->hsys, b->dsys.p, sizeof(BSys) * b->ctx.size(),
                           cudaMemcpyDeviceToHost, b->stream));
  B_TRY(b, cudaMemcpyAsync(b->hctl, b->dctl.p, sizeof(BCtl), cudaMemcpyDeviceToHost, b->stream));
  B_TRY(b, cudaStreamSynchronize(b->stream));
  if (ms) B_TRY(b, cudaEventElapsedTime(ms, b->ev0, b->ev1));
  if (b->hctl->err == 1)
    return bfail(b, FCG_ERR_TIMEOUT, "a grid-barrier wait of the batched solve gave up");
  if (b->hctl->err == 2)
    return bfail(b, FCG_ERR_TIMEOUT, "batched solve exceeded its loop bound");
  return FCG_OK;
}

// Loads system k (host or device arrays) into its context and fills hsys[k].
int load_system(fcg_batch *b, int k, const double *a, const double *su, const double *fi,
                double sor, int nsw, void **dfi_out, bool *hfi_out) {
  fcg_context *c = b->ctx[k];
  const size_t n1 = sizeof(double) * c->n;
  void *da = nullptr, *dsu, *dfi;
  bool ha, hsu, hfi;
  int rc;
  if (a && (rc = stage_in(c, a, sizeof(double) * c->nnz, 0, true, &da, &ha)))
    return bfail(b, rc, fcg_last_error(c));
  if ((rc = stage_in(c, su, n1, 1, true, &dsu, &hsu))) return bfail(b, rc, fcg_last_error(c));
  if ((rc = stage_in(c, fi, n1, 2, true, &dfi, &hfi))) return bfail(b, rc, fcg_last_error(c));
  BatchVecs v;
  if ((rc = batch_load(c, (const double *)da, (const double *)dsu, (const double *)dfi, &v)))
    return bfail(b, rc, fcg_last_error(c));
  B_TRY(b, cudaStreamSynchronize(c->stream));
  BSys &S = b->hsys[k];
  const int item0 = S.item0, nitems = S.nitems;
  std::memset(&S, 0, sizeof S);
  S.item0 = item0;
  S.nitems = nitems;
  S.sv = c->sv;
  S.n = c->n;
  S.nsw = nsw;
  S.val = v.val;
  S.invd = v.invd;
  S.su = v.su;
  S.x = v.x;
  S.res = v.res;
  S.p = v.p;
  S.q = v.q;
  S.sor = sor;
  S.small = (double)1e-20f;  // modules_allocatable.f90:27
  S.tol = (double)1e-13f;    // dpcg.f90:37
  S.early = 1;
  if (dfi_out) *dfi_out = dfi;
  if (hfi_out) *hfi_out = hfi;
  return FCG_OK;
}

}  // namespace

extern "C" int fcg_batch_destroy(fcg_batch *b);

extern "C" int fcg_batch_create(fcg_context *const *ctxs, int nsys, fcg_batch **out) {
  if (!ctxs || !out || nsys < 1 || nsys > kMaxBatch) return FCG_ERR_ARG;
  *out = nullptr;
  std::set<fcg_context *> seen;
  for (int k = 0; k < nsys; ++k) {
    if (!ctxs[k] || !ctxs[k]->bound || ctxs[k]->device != ctxs[0]->device) return FCG_ERR_ARG;
    if (ctxs[k]->mv.noc) return FCG_ERR_UNSUPPORTED;  // O-C grid cuts: one system at a time
    if (!seen.insert(ctxs[k]).second) return FCG_ERR_ARG;  // systems share solver vectors
  }
  if (cudaSetDevice(ctxs[0]->device) != cudaSuccess) return FCG_ERR_CUDA;
  fcg_batch *b = new fcg_batch();
  b->ctx.assign(ctxs, ctxs + nsys);
  b->device = ctxs[0]->device;
  b->num_sms = ctxs[0]->num_sms;
  b->stream = ctxs[0]->stream;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_dpcg, kTPB, 0) != cudaSuccess ||
      occ < 1 || cudaMallocHost(&b->hsys, sizeof(BSys) * nsys) != cudaSuccess ||
      cudaMallocHost(&b->hctl, sizeof(BCtl)) != cudaSuccess ||
      b->dsys.ensure(sizeof(BSys) * nsys) != cudaSuccess ||
      b->dctl.ensure(sizeof(BCtl)) != cudaSuccess || cudaEventCreate(&b->ev0) != cudaSuccess ||
      cudaEventCreate(&b->ev1) != cudaSuccess) {
    cudaGetLastError();
    fcg_batch_destroy(b);
    return FCG_ERR_CUDA;
  }
  b->occ = occ;
  b->blocks_per_sm = std::min(2, occ);
  std::memset(b->hsys, 0, sizeof(BSys) * nsys);
  if (build_items(b)) {
    fcg_batch_destroy(b);
    return FCG_ERR_CUDA;
  }
  *out = b;
  return FCG_OK;
}

extern "C" int fcg_batch_destroy(fcg_batch *b) {
  if (!b) return FCG_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->hsys) cudaFreeHost(b->hsys);
  if (b->hctl) cudaFreeHost(b->hctl);
  b->dsys.release();
  b->ditems.release();
  b->dpart.release();
  b->dctl.release();
  delete b;
  return FCG_OK;
}

extern "C" const char *fcg_batch_last_error(const fcg_batch *b) {
  return b ? b->err.c_str() : "NULL batch";
}

extern "C" int fcg_batch_set_params(fcg_batch *b, int slices_per_item, int blocks_per_sm) {
  if (!b || slices_per_item < 1 || slices_per_item > 4096 || blocks_per_sm < 1) return FCG_ERR_ARG;
  if (blocks_per_sm > b->occ)
    return bfail(b, FCG_ERR_ARG, "more CTAs per SM than can be resident for a cooperative launch");
  if (b->blocks_per_sm != blocks_per_sm) drop_graph(b);
  b->slices_per_item = slices_per_item;
  b->blocks_per_sm = blocks_per_sm;
  B_TRY(b, cudaSetDevice(b->device));
  return build_items(b);
}

// Diagnostics for the timeout path: the poll limit of every grid-barrier wait and a CTA
// (absent_block >= 0) that returns before the first barrier.  (polls, -1) restores
// normal operation; polls <= 0 restores the default limit.
extern "C" int fcg_batch_set_wait_test(fcg_batch *b, long long polls, int absent_block) {
  if (!b || absent_block < -1) return FCG_ERR_ARG;
  b->spin_limit = polls > 0 ? polls : (1LL << 22);
  b->absent_block = absent_block;
  drop_graph(b);
  return FCG_OK;
}

extern "C" int fcg_batch_get_params(const fcg_batch *b, int *slices_per_item, int *blocks_per_sm,
                                    int *max_blocks_per_sm) {
  if (!b) return FCG_ERR_ARG;
  if (slices_per_item) *slices_per_item = b->slices_per_item;
  if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
  if (max_blocks_per_sm) *max_blocks_per_sm = b->occ;
  return FCG_OK;
}

extern "C" int fcg_batch_dpcg(fcg_batch *b, const double *const *a, const double *const *su,
                              double *const *fi, double sor, int nsw, double *resor,
                              fcg_solve_report *rep) {
  if (!b || !su || !fi || nsw < 0) return FCG_ERR_ARG;
  B_TRY(b, cudaSetDevice(b->device));
  const int ns = (int)b->ctx.size();
  int rc = build_items(b);
  if (rc) return rc;
  std::vector<void *> dfi(ns);
  std::vector<char> hfi(ns);
  for (int k = 0; k < ns; ++k) {
    if (!su[k] || !fi[k]) return bfail(b, FCG_ERR_ARG, "NULL su or fi");
    bool h = false;
    if ((rc = load_system(b, k, a ? a[k] : nullptr, su[k], fi[k], sor, nsw, &dfi[k], &h)))
      return rc;
    hfi[k] = h;
  }
  float ms = 0.f;
  rc = run(b, nsw + 2, &ms);
  if (rc && rc != FCG_ERR_TIMEOUT) return rc;
  const int timeout = rc;
  for (int k = 0; k < ns; ++k) {
    fcg_context *c = b->ctx[k];
    const BSys &S = b->hsys[k];
    const size_t n1 = sizeof(double) * c->n;
    B_TRY(b, cudaMemcpyAsync(dfi[k], S.x, n1, cudaMemcpyDeviceToDevice, c->stream));
    int r2 = stage_out(c, fi[k], dfi[k], n1, hfi[k] != 0);
    if (r2) return bfail(b, r2, fcg_last_error(c));
    B_TRY(b, cudaStreamSynchronize(c->stream));
    if (resor && S.iter > 0) resor[k] = S.res0;  // dpcg.f90:139
    if (rep) {
      rep[k].res0 = S.res0;
      rep[k].resl = S.resl;
      rep[k].iters = S.iter;
      rep[k].converged = S.converged;
      rep[k].l2_rel = S.l2b > 0 ? std::sqrt(S.l2r / S.l2b) : std::sqrt(S.l2r);
      rep[k].seconds = ms * 1e-3;
    }
  }
  if (timeout) return timeout;
  for (int k = 0; k < ns; ++k)
    if (b->hsys[k].status)
      return bfail(b, b->hsys[k].status, "non-finite value in a batched system");
  return FCG_OK;
}

// Times every (slices per item, CTAs per SM) candidate on `sweeps` fixed sweeps of the
// caller's systems (x = 0, sor = 0) and keeps the fastest.  a, su as in fcg_batch_dpcg.
extern "C" int fcg_batch_autotune(fcg_batch *b, const double *const *a, const double *const *su,
                                  int sweeps, double *best_ms) {
  if (!b || !su || sweeps < 1) return FCG_ERR_ARG;
  B_TRY(b, cudaSetDevice(b->device));
  const int ns = (int)b->ctx.size();
  std::vector<DBuf> zeros(ns);
  const int cand_items[] = {4, 8, 16, 32, 64, 128};
  int best_spi = b->slices_per_item, best_bps = b->blocks_per_sm;
  float best = 1e30f;
  int rc = FCG_OK;
  for (int k = 0; k < ns && !rc; ++k) {
    if (zeros[k].ensure(sizeof(double) * b->ctx[k]->n) != cudaSuccess)
      rc = bfail(b, FCG_ERR_NOMEM, "autotune scratch");
    else if (cudaMemset(zeros[k].p, 0, sizeof(double) * b->ctx[k]->n) != cudaSuccess)
      rc = bfail(b, FCG_ERR_CUDA, "autotune scratch");
  }
  bool loaded = false;
  for (int spi : cand_items) {
    for (int bps = 1; bps <= std::min(b->occ, 4) && !rc; bps *= 2) {
      if ((rc = fcg_batch_set_params(b, spi, bps))) break;
      float t = 0.f;
      for (int rep = 0; rep < 2 && !rc; ++rep) {  // first run warms up
        for (int k = 0; k < ns && !rc; ++k)
          rc = load_system(b, k, (a && !loaded) ? a[k] : nullptr, su[k],
                           zeros[k].as<double>(), 0.0, sweeps, nullptr, nullptr);
        loaded = true;
        if (!rc) rc = run(b, sweeps + 2, &t);
      }
      if (!rc && t < best) {
        best = t;
        best_spi = spi;
        best_bps = bps;
      }
    }
    if (rc) break;
  }
  for (DBuf &z : zeros) z.release();
  if (rc) return rc;
  if (best_ms) *best_ms = best;
  return fcg_batch_set_params(b, best_spi, best_bps);
}
