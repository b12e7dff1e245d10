// Plane-staged form of one message-passing layer of the learned preconditioner, for
// meshes whose cells form a lexicographic nx x ny x nz hexahedral block (cell
// r = i + nx j + nx ny k, as the jittered hex meshes of the benchmark are numbered).
// No counterpart in the reference; the network and its sliced gather form are in
// learned.cu, and this kernel gives the same bits.
//
// On such a mesh every row of Ahat couples a cell to at most its six face neighbours,
// at column offsets -nx ny, -nx, -1, +1, +nx, +nx ny.  The gather form fetches each
// neighbour row from L2/HBM with a dependent chain of loads (slice metadata -> offset ->
// neighbour), which keeps it latency bound.  Here a block owns a 16 x 16 tile of (i, j)
// and marches along k over a chunk of planes:
//
//   - one producer warp streams the planes k-1 .. k_end of its tile, each with a
//     one-cell halo in i and j (18 x 18 cells x 32 BF16 channels = 20.7 KB), plus the
//     seven stencil value planes of the tile (7 x 16 x 16 FP32 = 7 KB), into a ring of
//     five shared-memory stages with TMA tensor copies (cp.async.bulk.tensor, 4-D
//     tensor maps over this GPU's memory, zero fill outside the block), each stage
//     signalled by an mbarrier with a transaction count;
//   - sixteen consumer warps compute plane k from stages k-1, k and k+1: per cell
//     m = sum over the seven directions of val[d] * h[neighbour], summed in the CSR column
//     order with the same fused multiply-adds as the gather form; then the per-warp
//     16-cell tile [h; m] goes through the shared mma.sync product and epilogue
//     (lp_tile.cuh) and h' leaves in 16-byte stores (16 consecutive cells = 1 KB);
//   - after plane k the consumers release the stage of plane k-1 to the producer.
//
// So each activation row and each stencil value is read from HBM once per layer (the
// halo rows of neighbouring tiles are L2 hits), and the loads are deep in flight without
// holding registers.  Every mbarrier wait is bounded: a wait that gives up stores
// FCG_ERR_TIMEOUT, the block waits (bounded) for its copies in flight and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "launch.h"
#include "lp_hex.h"
#include "lp_tile.cuh"

namespace fcg {
namespace lphex {
namespace {

constexpr int C = lp::kTileC;
constexpr int TS = lp::kTileStride;
constexpr int BX = 16, BY = 16;          // cells of a tile in i and j
constexpr int HX = BX + 2, HY = BY + 2;  // with the one-cell halo
constexpr int S = 5;                     // ring stages (planes)
constexpr int KC = 32;                   // planes computed by one block
constexpr int kCons = 16;                // consumer warps, one j row of the tile each
constexpr int kThreads = (kCons + 1) * 32;
constexpr unsigned kHBytes = HY * HX * C * 2;
constexpr unsigned kVBytes = 7 * BY * BX * 4;
constexpr unsigned long long kWaitNs = 1000000000ull;  // a wait gives up after 1 s
constexpr int kMaxDevices = 64;
static_assert(BY % kCons == 0, "each consumer warp owns whole j rows");
static_assert(kHBytes % 128 == 0 && kVBytes % 128 == 0, "TMA destinations stay 128-byte aligned");

struct __align__(128) Smem {
  __nv_bfloat16 h[S][HY][HX][C];
  float v[S][7][BY][BX];
  __nv_bfloat16 w[C * TS];
  float b[C];
  __nv_bfloat16 tile[kCons][16 * TS];
  unsigned long long full[S], empty[S];
  int abort, issued;
};
constexpr size_t kSmemBytes = sizeof(Smem) + 128;  // + alignment of the dynamic base

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait for the phase of parity `parity`; gives up after kWaitNs or when another
// warp has raised the abort flag.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity,
                                          const volatile int *abort) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned i = 1;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (abort && *abort) return false;
    if ((i & 255u) == 0 && global_ns() - t0 > kWaitNs) return false;
  }
}
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            int c2, int c3, unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
      "{%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(smem_u32(bar))
      : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    k_lp_layer_hex(const __grid_constant__ CUtensorMap tm_h, const __grid_constant__ CUtensorMap tm_v,
                   int nx, int ny, int nz, __nv_bfloat16 *__restrict__ hout,
                   const __nv_bfloat16 *__restrict__ wl, const float *__restrict__ bl,
                   const int *done, int *status) {
  if (done && __ldcg(done) != 0) return;
  extern __shared__ unsigned char smem_raw[];
  Smem &sm = *reinterpret_cast<Smem *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) &
                                       ~static_cast<uintptr_t>(127));
  const int ntx = (nx + BX - 1) / BX;
  const int i0 = (int)(blockIdx.x % ntx) * BX, j0 = (int)(blockIdx.x / ntx) * BY;
  const int k0 = (int)blockIdx.y * KC;
  const int k1 = min(k0 + KC, nz);
  const int np = k1 - k0 + 2;  // planes k0-1 .. k1
  for (int t = threadIdx.x; t < C * 2 * C; t += blockDim.x)
    sm.w[(t / (2 * C)) * TS + t % (2 * C)] = wl[t];
  if (threadIdx.x < C) sm.b[threadIdx.x] = bl[threadIdx.x];
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], kCons);
    }
    sm.abort = 0;
    sm.issued = 0;
    fence_mbar_init();
  }
  __syncthreads();
  volatile int *abort = &sm.abort;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == kCons) {
    // producer: one thread issues every copy of the block
    if (lane == 0) {
      for (int idx = 0; idx < np; ++idx) {
        const int s = idx % S;
        if (idx >= S && !mbar_wait(&sm.empty[s], ((idx / S) - 1) & 1, abort)) break;
        if (*abort) break;
        const int p = k0 - 1 + idx;
        const bool want_v = p >= k0 && p < k1;
        mbar_expect_tx(&sm.full[s], kHBytes + (want_v ? kVBytes : 0u));
        tma_load_4d(&sm.h[s][0][0][0], &tm_h, 0, i0 - 1, j0 - 1, p, &sm.full[s]);
        if (want_v) tma_load_4d(&sm.v[s][0][0][0], &tm_v, i0, j0, p, 0, &sm.full[s]);
        *(volatile int *)&sm.issued = idx + 1;
      }
    }
    __syncwarp();
  } else {
    const int g = lane >> 2, qc = 8 * (lane & 3);
    __nv_bfloat16 *tw = sm.tile[warp];
    // every decision to stop is taken by the whole warp (__all_sync / __any_sync), so
    // the warp never splits around its __syncwarp calls
    bool ok = __all_sync(0xffffffffu, mbar_wait(&sm.full[0], 0, abort) &&
                                          mbar_wait(&sm.full[1], 0, abort));
    for (int k = k0; ok && k < k1; ++k) {
      const int idx = k - k0 + 1;  // ring index of plane k
      if (!__all_sync(0xffffffffu, mbar_wait(&sm.full[(idx + 1) % S], ((idx + 1) / S) & 1, abort))) {
        ok = false;
        break;
      }
      const int sP = (idx - 1) % S, sC = idx % S, sN = (idx + 1) % S;
#pragma unroll 1
      for (int rr = 0; rr < BY / kCons; ++rr) {
        const int jr = warp + kCons * rr;
#pragma unroll 1
        for (int rd = 0; rd < 2; ++rd) {
          const int il = rd * 8 + g;
          const float *vv = &sm.v[sC][0][jr][il];
          float acc[8];
#pragma unroll
          for (int c = 0; c < 8; ++c) acc[c] = 0.f;
          // the seven terms in CSR column order: -nx ny, -nx, -1, 0, +1, +nx, +nx ny
          const uint4 hm2 = *reinterpret_cast<const uint4 *>(&sm.h[sP][jr + 1][il + 1][qc]);
          const uint4 hm1 = *reinterpret_cast<const uint4 *>(&sm.h[sC][jr][il + 1][qc]);
          const uint4 hm0 = *reinterpret_cast<const uint4 *>(&sm.h[sC][jr + 1][il][qc]);
          const uint4 own = *reinterpret_cast<const uint4 *>(&sm.h[sC][jr + 1][il + 1][qc]);
          const uint4 hp0 = *reinterpret_cast<const uint4 *>(&sm.h[sC][jr + 1][il + 2][qc]);
          const uint4 hp1 = *reinterpret_cast<const uint4 *>(&sm.h[sC][jr + 2][il + 1][qc]);
          const uint4 hp2 = *reinterpret_cast<const uint4 *>(&sm.h[sN][jr + 1][il + 1][qc]);
          lp::fma8(acc, vv[0 * BY * BX], hm2);
          lp::fma8(acc, vv[1 * BY * BX], hm1);
          lp::fma8(acc, vv[2 * BY * BX], hm0);
          lp::fma8(acc, vv[3 * BY * BX], own);
          lp::fma8(acc, vv[4 * BY * BX], hp0);
          lp::fma8(acc, vv[5 * BY * BX], hp1);
          lp::fma8(acc, vv[6 * BY * BX], hp2);
          __align__(16) __nv_bfloat16 mb[8];
          lp::tile_put_row(tw, il, qc, own, acc, mb);
        }
        __syncwarp();
        lp::tile_dense(tw, sm.w, sm.b, lane, lp::NoZ());
        const int jg = j0 + jr;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int e = lane + 32 * q, ri = e >> 2, part = e & 3;
          const int ig = i0 + ri;
          if (ig < nx && jg < ny)
            *reinterpret_cast<uint4 *>(
                hout + (((long long)k * ny + jg) * nx + ig) * C + 8 * part) =
                *reinterpret_cast<const uint4 *>(tw + ri * TS + 8 * part);
        }
        __syncwarp();
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.empty[sP]);  // plane k-1 is no longer read
      if (__any_sync(0xffffffffu, *abort != 0)) break;
    }
    if (!ok && lane == 0) {
      *abort = 1;
      if (status) atomicExch(status, FCG_ERR_TIMEOUT);
    }
  }
  __syncthreads();
  // After a wait that gave up, the copies still in flight must land before the block
  // leaves (their destination is this block's shared memory).
  if (threadIdx.x == 0 && *abort) {
    const int issued = *(volatile int *)&sm.issued;
    for (int idx = issued - S > 0 ? issued - S : 0; idx < issued; ++idx)
      mbar_wait(&sm.full[idx % S], (idx / S) & 1, nullptr);
  }
}

// Stencil value planes from the sliced FP32 matrix (real entries only: pads are skipped).
__global__ void k_hex_values(SellView s, int n, const float *__restrict__ aval, int nx, int ny,
                             int nz, int nxp, float *__restrict__ val) {
  const long long nxy = (long long)nx * ny;
  const long long plane = (long long)nz * ny * nxp;
  FCG_GRID_STRIDE(r, n) {
    const int i = (int)(r % nx), j = (int)((r / nx) % ny), k = (int)(r / nxy);
    const int slice = (int)(r >> 5), ln = (int)(r & 31);
    const long long base = s.ptr[slice] + ln;
    const int w = s.width[slice], op = s.offp[slice];
    const bool uni = s.kind[slice] == 0;
    float v[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) v[d] = 0.f;
    for (int q = 0; q < w; ++q) {
      const long long pos = base + 32LL * q;
      if (s.src[pos] < 0) continue;
      const long long col = uni ? r + s.off[op + q] : (long long)s.off[op + 32 * q + ln];
      const long long d = col - r;
      const int dir = d == -nxy ? 0 : d == -nx ? 1 : d == -1 ? 2 : d == 0 ? 3 : d == 1 ? 4
                    : d == nx ? 5 : d == nxy ? 6 : -1;
      const float x = aval[pos];
#pragma unroll
      for (int e = 0; e < 7; ++e)
        if (dir == e) v[e] = x;
    }
    const long long o = ((long long)k * ny + j) * nxp + i;
#pragma unroll
    for (int d = 0; d < 7; ++d) val[d * plane + o] = v[d];
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
std::mutex g_attr_mutex;
bool g_attr_set[kMaxDevices] = {false};

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  std::call_once(g_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    else
      cudaGetLastError();
  });
  return g_encode;
}

bool encode_maps(const HexGrid &g, const void *hin, const void *val, CUtensorMap *th,
                 CUtensorMap *tv) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
  if (!enc) return false;
  const cuuint64_t hdim[4] = {(cuuint64_t)C, (cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
  const cuuint64_t hstr[3] = {(cuuint64_t)C * 2, (cuuint64_t)C * 2 * g.nx,
                              (cuuint64_t)C * 2 * g.nx * g.ny};
  const cuuint32_t hbox[4] = {(cuuint32_t)C, HX, HY, 1};
  const cuuint64_t vdim[4] = {(cuuint64_t)g.nxp, (cuuint64_t)g.ny, (cuuint64_t)g.nz, 7};
  const cuuint64_t vstr[3] = {(cuuint64_t)4 * g.nxp, (cuuint64_t)4 * g.nxp * g.ny,
                              (cuuint64_t)4 * g.nxp * g.ny * g.nz};
  const cuuint32_t vbox[4] = {BX, BY, 1, 7};
  const cuuint32_t one[4] = {1, 1, 1, 1};
  if (enc(th, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(hin), hdim, hstr, hbox, one,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  if (enc(tv, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void *>(val), vdim, vstr, vbox, one,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  return true;
}

// The kernel's shared-memory opt-in, once per device (outside any stream capture).
cudaError_t set_attributes(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_attr_mutex);
  if (g_attr_set[dev]) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_lp_layer_hex, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kSmemBytes);
  if (e == cudaSuccess) g_attr_set[dev] = true;
  return e;
}

}  // namespace

int detect(fcg_context *c, HexGrid *g) {
  *g = HexGrid();
  if (!c->hex.ok || !encoder()) return FCG_OK;
  FCG_CUDA_TRY(c, set_attributes(c->device));
  HexGrid t;
  t.nx = c->hex.nx;
  t.ny = c->hex.ny;
  t.nz = c->hex.nz;
  t.nxp = (t.nx + 3) / 4 * 4;
  // a trial encoding on aligned placeholder addresses: maps that the driver refuses
  // (extents beyond its limits) leave the gather form in use
  CUtensorMap th, tv;
  t.ok = encode_maps(t, c->mv.xc, c->mv.xc, &th, &tv);
  *g = t;
  return FCG_OK;
}

cudaError_t values(const fcg_context *c, const HexGrid &g, const float *aval, float *val,
                   cudaStream_t st) {
  k_hex_values<<<grid_for(c->n, c->num_sms), kTPB, 0, st>>>(c->sv, c->n, aval, g.nx, g.ny, g.nz,
                                                             g.nxp, val);
  return cudaPeekAtLastError();
}

cudaError_t layer(const HexGrid &g, int num_sms, const __nv_bfloat16 *hin, __nv_bfloat16 *hout,
                  const float *val, const __nv_bfloat16 *wl, const float *bl, const int *done,
                  int *status, cudaStream_t st) {
  (void)num_sms;
  CUtensorMap th, tv;
  if (!encode_maps(g, hin, val, &th, &tv)) return cudaErrorInvalidValue;
  const int ntx = (g.nx + BX - 1) / BX, nty = (g.ny + BY - 1) / BY;
  const dim3 grid((unsigned)(ntx * nty), (unsigned)((g.nz + KC - 1) / KC));
  k_lp_layer_hex<<<grid, kThreads, kSmemBytes, st>>>(th, tv, g.nx, g.ny, g.nz, hout, wl, bl, done,
                                                     status);
  return cudaPeekAtLastError();  // left set for the caller's launch check
}

}  // namespace lphex
}  // namespace fcg
