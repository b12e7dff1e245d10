// fcg_dpcg_noalloc: the Jacobi-preconditioned CG of fcg_dpcg for callers that cannot
// allocate device memory.
//
// Who needs it: a host code whose device memory is all owned by someone else -- e.g. a
// Fortran solver that reserves the whole GPU for its own pool at start-up, or a
// real-time loop whose rules forbid any allocation after initialisation.  Such a
// caller already holds its matrix and vectors in device memory and cannot let the
// library cudaMalloc workspaces.  This entry point therefore creates no context and
// allocates nothing: no cudaMalloc, no cudaFree, no allocating library routine.  Its
// work vectors live in one file-scope device array of fixed size, so the largest system
// it accepts is FCG_NOALLOC_MAX_CELLS cells (every GPU that loads the library keeps
// that array, about 6.4 MB, until the process exits).
//
// The array is shared by every call in the process: two calls that overlap on the GPU
// (on different streams, or from different host threads) race on it and give wrong
// results.  Each call clears what must start at zero (the solver scalars, counters and
// the search direction) before it uses the array, so a call never sees leftovers of
// the previous one.
//
// Set-up: the first call on a device, with that device current, looks up the array's
// device address with cudaGetSymbolAddress and caches it for that device.  Make that
// first call before any stream capture begins.  With CUDA's default lazy module loading
// that first call is also when this file's code and the array are loaded onto the
// device: it takes about 6.4 MB plus the code's size once, and later calls take
// nothing.  A caller that reserves the whole device for its own pool must make the first
// call before the pool takes its memory, or run with CUDA_MODULE_LOADING=EAGER, which
// loads the array when the library is loaded.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/fcgpu.h"

namespace {

constexpr int kMaxCells = FCG_NOALLOC_MAX_CELLS;
constexpr int kTPB = 256;
constexpr int kWarps = kTPB / 32;
constexpr int kMaxBlocks = 2048;
constexpr int kMaxDevices = 64;
constexpr int kSweepsPerCheck = 16;

struct NaScal {
  double res0, resl, resor, rsm, s0, sk, bet, alf, l2r, l2b, small, resmax, tol;
  int iter, nsw, done, converged, status, early, pad0, pad1;
  unsigned int ticket[4];
};

// Layout: pk[kMaxCells] | qk[kMaxCells] | invd[kMaxCells] | partials[2*kMaxBlocks] | NaScal
constexpr size_t kScalDoubles = (sizeof(NaScal) + sizeof(double) - 1) / sizeof(double);
constexpr size_t kScratchDoubles = 3 * (size_t)kMaxCells + 2 * (size_t)kMaxBlocks + kScalDoubles;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {nullptr};

// Deterministic block sum + last-block-done reduction (same scheme as the context
// solvers): thread 0 of the last block receives the grid-wide sums.
template <int NV>
__device__ bool na_reduce(double (&v)[NV], double *partials, unsigned int *ticket) {
  __shared__ double sh[NV][kWarps];
  __shared__ bool am_last;
  auto block_sum = [&](double(&x)[NV]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < NV; ++k) x[k] += __shfl_down_sync(0xffffffffu, x[k], o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) sh[k][w] = x[k];
    __syncthreads();
    if (w == 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) x[k] = lane < kWarps ? sh[k][lane] : 0.0;
#pragma unroll
      for (int o = kWarps / 2; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < NV; ++k) x[k] += __shfl_down_sync(0xffffffffu, x[k], o);
    }
    __syncthreads();
  };
  block_sum(v);
  const int G = gridDim.x;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * G + blockIdx.x] = v[k];
    __threadfence();
    am_last = atomicAdd(ticket, 1u) == (unsigned int)G - 1;
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
  block_sum(s);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = s[k];
    *ticket = 0u;
  }
  return true;
}

#define NA_ROWS(i, n) \
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// The caller's CSR is 1-based (sparse_matrix.f90); row i's entries are
// ioffset[i]-1 .. ioffset[i+1]-2, columns ja[k]-1.
__device__ __forceinline__ double csr_row(const int *__restrict__ io, const int *__restrict__ ja,
                                          const double *__restrict__ a,
                                          const double *__restrict__ x, int i) {
  double acc = 0.0;
  for (int k = io[i] - 1; k < io[i + 1] - 1; ++k) acc += a[k] * x[ja[k] - 1];
  return acc;
}

__global__ void k_na_reset(NaScal *S, int nsw, double sor, double small, double tol) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    memset(S, 0, sizeof(NaScal));
    S->nsw = nsw;
    S->resmax = sor;
    S->small = small;
    S->tol = tol;
    S->early = 1;
  }
}

// res = su - A fi, res0 = sum|res|, invd = 1/a(diag), pk = 0, sk = sum res^2/a(diag).
__global__ void k_na_init(int n, const int *io, const int *ja, const int *diag, const double *a,
                          const double *su, const double *fi, double *res, double *invd,
                          double *pk, double *partials, NaScal *S) {
  double v[2] = {0.0, 0.0};
  NA_ROWS(i, n) {
    double r = su[i] - csr_row(io, ja, a, fi, i);
    double dinv = 1.0 / a[diag[i] - 1];
    res[i] = r;
    invd[i] = dinv;
    pk[i] = 0.0;
    v[0] += fabs(r);
    v[1] += r * (r * dinv);
  }
  if (na_reduce<2>(v, partials, &S->ticket[0]) && threadIdx.x == 0) {
    S->res0 = v[0];
    S->resl = v[0];
    S->s0 = (double)1.e20f;  // dpcg.f90:76
    S->sk = v[1];
    S->bet = v[1] / S->s0;
    S->done = (S->nsw <= 0 || v[0] < S->tol) ? 1 : 0;  // dpcg.f90:66-70
    if (!isfinite(v[0])) {
      S->status = FCG_ERR_NONFINITE;
      S->done = 1;
    }
  }
}

__global__ void k_na_p(int n, const double *res, const double *invd, double *pk, const NaScal *S) {
  if (__ldcg(&S->done)) return;
  const double bet = __ldcg(&S->bet);
  NA_ROWS(i, n) pk[i] = res[i] * invd[i] + bet * pk[i];
}

__global__ void k_na_spmv(int n, const int *io, const int *ja, const double *a, const double *pk,
                          double *qk, double *partials, NaScal *S) {
  if (__ldcg(&S->done)) return;
  double v[1] = {0.0};
  NA_ROWS(i, n) {
    double q = csr_row(io, ja, a, pk, i);
    qk[i] = q;
    v[0] += pk[i] * q;
  }
  if (na_reduce<1>(v, partials, &S->ticket[1]) && threadIdx.x == 0) {
    S->alf = S->sk / v[0];
    if (!isfinite(S->alf)) S->status = FCG_ERR_NONFINITE;
  }
}

__global__ void k_na_update(int n, double *fi, double *res, const double *pk, const double *qk,
                            const double *invd, double *partials, NaScal *S) {
  if (__ldcg(&S->done)) return;
  const double alf = __ldcg(&S->alf);
  double v[2] = {0.0, 0.0};
  NA_ROWS(i, n) {
    fi[i] = fi[i] + alf * pk[i];
    double r = res[i] - alf * qk[i];
    res[i] = r;
    v[0] += fabs(r);
    v[1] += r * (r * invd[i]);
  }
  if (na_reduce<2>(v, partials, &S->ticket[2]) && threadIdx.x == 0) {
    S->s0 = S->sk;
    S->sk = v[1];
    S->bet = v[1] / S->s0;
    int it = S->iter + 1;
    S->iter = it;
    S->resl = v[0];
    if (it == 1) S->resor = S->res0;
    S->rsm = v[0] / (S->resor + S->small);
    if (S->rsm < S->resmax) S->converged = 1;
    if (!isfinite(v[0])) S->status = FCG_ERR_NONFINITE;
    if (S->converged || it >= S->nsw || S->status) S->done = 1;
  }
}

__global__ void k_na_final(int n, const int *io, const int *ja, const double *a, const double *su,
                           const double *fi, double *partials, NaScal *S) {
  double v[2] = {0.0, 0.0};
  NA_ROWS(i, n) {
    double r = su[i] - csr_row(io, ja, a, fi, i);
    v[0] += r * r;
    v[1] += su[i] * su[i];
  }
  if (na_reduce<2>(v, partials, &S->ticket[3]) && threadIdx.x == 0) {
    S->l2r = v[0];
    S->l2b = v[1];
  }
}

// Device memory of the current device `dev`, or managed memory: arrays of another GPU
// would be read over peer access, or fault without it.
bool on_device(const void *p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == dev;
}

// A launch that failed (no image for this GPU, bad configuration) leaves the solver
// scalars unwritten: report it instead of reading them.
bool launch_failed() {
  if (cudaPeekAtLastError() == cudaSuccess) return false;
  cudaGetLastError();
  return true;
}

}  // namespace

extern "C" int fcg_dpcg_noalloc(int numCells, const int *ioffset, const int *ja, const int *diag,
                                const double *a, const double *su, double *fi, double *res,
                                double sor, int nsw, double *resor, fcg_solve_report *rep,
                                void *stream) {
  if (numCells <= 0 || numCells > kMaxCells) return FCG_ERR_ARG;  // beyond the static array
  if (nsw < 0 || !ioffset || !ja || !diag || !a || !su || !fi || !res) return FCG_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FCG_ERR_CUDA;
  const void *arrays[] = {ioffset, ja, diag, a, su, fi, res};
  for (const void *p : arrays)
    if (!on_device(p, dev)) return FCG_ERR_ARG;  // host arrays would need staging memory
  double *base;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      void *ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
        cudaGetLastError();
        return FCG_ERR_CUDA;
      }
      g_scratch_addr[dev] = (double *)ptr;
    }
    base = g_scratch_addr[dev];
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return FCG_ERR_CUDA;
  const int need = (numCells + kTPB - 1) / kTPB;
  const int G = need < sms * 8 ? need : (sms * 8 < kMaxBlocks ? sms * 8 : kMaxBlocks);
  cudaStream_t st = (cudaStream_t)stream;
  double *pk = base, *qk = base + kMaxCells, *invd = base + 2 * (size_t)kMaxCells;
  double *partials = base + 3 * (size_t)kMaxCells;
  NaScal *S = (NaScal *)(partials + 2 * kMaxBlocks);
  const int n = numCells;
  const auto t0 = std::chrono::steady_clock::now();
  k_na_reset<<<1, 32, 0, st>>>(S, nsw, sor, (double)1e-20f, (double)1e-13f);
  k_na_init<<<G, kTPB, 0, st>>>(n, ioffset, ja, diag, a, su, fi, res, invd, pk, partials, S);
  if (launch_failed()) return FCG_ERR_CUDA;
  int done = 0;
  for (int swept = 0; !done && swept <= nsw; swept += kSweepsPerCheck) {
    for (int j = 0; j < kSweepsPerCheck; ++j) {
      k_na_p<<<G, kTPB, 0, st>>>(n, res, invd, pk, S);
      k_na_spmv<<<G, kTPB, 0, st>>>(n, ioffset, ja, a, pk, qk, partials, S);
      k_na_update<<<G, kTPB, 0, st>>>(n, fi, res, pk, qk, invd, partials, S);
    }
    if (launch_failed()) return FCG_ERR_CUDA;
    if (cudaMemcpyAsync(&done, &S->done, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaGetLastError();
      return FCG_ERR_CUDA;
    }
  }
  k_na_final<<<G, kTPB, 0, st>>>(n, ioffset, ja, a, su, fi, partials, S);
  if (launch_failed()) return FCG_ERR_CUDA;
  NaScal h;
  if (cudaMemcpyAsync(&h, S, sizeof(NaScal), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return FCG_ERR_CUDA;
  }
  if (resor && h.iter > 0) *resor = h.res0;  // dpcg.f90:139
  if (rep) {
    rep->res0 = h.res0;
    rep->resl = h.resl;
    rep->iters = h.iter;
    rep->converged = h.converged;
    rep->l2_rel = h.l2b > 0 ? std::sqrt(h.l2r / h.l2b) : std::sqrt(h.l2r);
    rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return h.status ? h.status : FCG_OK;
}
