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

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
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
  float wo[C + 4];  // w_out, b_out of a fused output (padded to 16 bytes)
  __nv_bfloat16 tile[kCons][16 * TS];
  unsigned long long full[S], empty[S];
  int abort, issued;
};
constexpr size_t kSmemBytes = sizeof(Smem) + 128;  // + alignment of the dynamic base
static_assert(offsetof(Smem, tile) % 16 == 0, "the tile rows take 16-byte accesses");

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
                   const int *done, int *status, OutFuse of) {
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
  if (of.z && threadIdx.x <= C) sm.wo[threadIdx.x] = of.wout[threadIdx.x];
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
    const float osc = of.z ? *of.rms : 0.f;
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
        if (of.z) {
          // the output instead of h': lane ri < 16 takes cell ri of the row, with the
          // operations of the output kernel on the stored h'
          const int ig = i0 + lane;
          if (lane < 16 && ig < nx && jg < ny) {
            const long long cell = ((long long)k * ny + jg) * nx + ig;
            const float acc = lp::out_dot_row(tw + lane * TS, sm.wo);
            of.z[cell] = of.r[cell] + osc * acc;
          }
        } else {
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const int e = lane + 32 * q, ri = e >> 2, part = e & 3;
            const int ig = i0 + ri;
            if (ig < nx && jg < ny)
              *reinterpret_cast<uint4 *>(
                  hout + (((long long)k * ny + jg) * nx + ig) * C + 8 * part) =
                  *reinterpret_cast<const uint4 *>(tw + ri * TS + 8 * part);
          }
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

// ---------------------------------------------------------------------------
// The same layer with the tile product on the fifth-generation tensor cores (selected by
// FCG_LP_HEX_MMA=tc; the mma.sync form above stays the default: this one measured 1.17
// against 0.94 ms per layer at 256^3 -- the per-plane barrier of all consumers and the
// bank conflicts of writing the canonical operand layout, whose K-chunks of a row share
// banks, cost more than the product it moves off the consumers).  The
// consumers write each plane's 256 rows [h; m] into a shared-memory operand in the
// canonical K-major layout without swizzle (8-row x 16-byte core matrices; 128 bytes
// between core matrices along K, 1024 between 8-row groups); after a barrier one thread
// issues two 128 x 32 x 64 products (four K = 16 steps each, `tcgen05.mma.kind::f16`,
// BF16 operands, FP32 accumulation in tensor memory) and commits them to an mbarrier.
// While they run, the consumers aggregate the next plane into the second operand buffer;
// then every warp reads its 32 rows x 16 columns of the accumulator (`tcgen05.ld`), adds
// the bias, applies the ReLU and the skip connection and stores h'.  Operands and
// accumulators are double buffered (2 x 32 KB of shared memory, 2 x 64 of the 128 tensor
// memory columns the block allocates).
constexpr int kTcRows = BX * BY;       // 256 rows of one plane
constexpr int kTcCols = 128;           // tensor-memory columns of the block
constexpr unsigned kTcABytes = kTcRows * 2 * C * 2;  // one [h; m] operand, 32 KB
constexpr uint32_t kTcIdesc = (1u << 4)              // FP32 accumulator
                              | (1u << 7) | (1u << 10)  // BF16 A and B
                              | ((uint32_t)(C >> 3) << 17)   // N = 32
                              | ((uint32_t)(128 >> 4) << 24);  // M = 128

struct __align__(1024) SmemTc {
  unsigned char a[2][kTcABytes];  // first: 1024-byte aligned operands
  __nv_bfloat16 h[S][HY][HX][C];
  float v[S][7][BY][BX];
  unsigned char wb[C * 2 * C * 2];  // W_l as the K-major B operand (32 x 64)
  float b[C];
  unsigned long long full[S], empty[S], mma_done[2];
  uint32_t tmem;
  int abort, issued;
};
constexpr size_t kSmemTcBytes = sizeof(SmemTc) + 1024;  // + alignment of the dynamic base

// Byte offset of 16-byte chunk `kc` (8 channels) of row `r` in a canonical operand.
__device__ __forceinline__ uint32_t tc_off(int r, int kc) {
  return (uint32_t)((r >> 3) * 1024 + kc * 128 + (r & 7) * 16);
}
// Shared-memory matrix descriptor: start address, 128-byte step between core matrices
// along K, 1024-byte step between 8-row groups, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) |
         ((uint64_t)(1024u >> 4) << 32) | (1ull << 46);
}
// OR of `v` over the consumer warps, which also wait for each other here (named barrier 1).
__device__ __forceinline__ bool cons_sync_or(bool v, int nthreads) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n barrier.cta.red.or.pred q, 1, %2, p;\n"
      " selp.u32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(nthreads)
      : "memory");
  return r != 0;
}

__global__ void __launch_bounds__(kThreads, 1)
    k_lp_layer_hex_tc(const __grid_constant__ CUtensorMap tm_h,
                      const __grid_constant__ CUtensorMap tm_v, int nx, int ny, int nz,
                      __nv_bfloat16 *__restrict__ hout, const __nv_bfloat16 *__restrict__ wl,
                      const float *__restrict__ bl, const int *done, int *status) {
  static_assert(kCons == 16 && BY == kCons, "one j row of the tile per consumer warp");
  if (done && __ldcg(done) != 0) return;
  extern __shared__ unsigned char smem_raw[];
  SmemTc &sm = *reinterpret_cast<SmemTc *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                           ~static_cast<uintptr_t>(1023));
  const int ntx = (nx + BX - 1) / BX;
  const int i0 = (int)(blockIdx.x % ntx) * BX, j0 = (int)(blockIdx.x / ntx) * BY;
  const int k0 = (int)blockIdx.y * KC;
  const int k1 = min(k0 + KC, nz);
  const int np = k1 - k0 + 2;  // planes k0-1 .. k1
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // W_l [out n][in k] is already K-major: chunk (n, kc) -> canonical position
  for (int t = threadIdx.x; t < C * 8; t += blockDim.x) {
    const int n = t >> 3, kc = t & 7;
    *reinterpret_cast<uint4 *>(sm.wb + tc_off(n, kc)) =
        *reinterpret_cast<const uint4 *>(wl + n * 2 * C + kc * 8);
  }
  if (threadIdx.x < C) sm.b[threadIdx.x] = bl[threadIdx.x];
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], kCons);
    }
    mbar_init(&sm.mma_done[0], 1);
    mbar_init(&sm.mma_done[1], 1);
    sm.abort = 0;
    sm.issued = 0;
    fence_mbar_init();
  }
  if (warp == 0) {  // tensor memory for the two accumulator buffers
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&sm.tmem)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B operand for the MMA
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = sm.tmem;
  volatile int *abort = &sm.abort;
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
    const int jr = warp;  // the consumer's j row in every plane
    // epilogue share: TMEM lane quarter, M tile and column half of this warp
    const int eq = warp & 3, et = (warp >> 2) & 1, ech = warp >> 3;
    const int erow = 128 * et + 32 * eq + lane;  // the operand row (cell) it finishes
    int ncommit[2] = {0, 0};                      // (issuing thread) commits per buffer
    bool bad = !(mbar_wait(&sm.full[0], 0, abort) && mbar_wait(&sm.full[1], 0, abort));
    // the epilogue of plane k: accumulator buffer `buf`, its commit phase `ph`, the ring
    // stage `st` that still holds the plane's activations (the skip connection)
    auto epilogue = [&](int k, int buf, int ph, int st) {
      bool ok = mbar_wait(&sm.mma_done[buf], ph & 1, abort);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t v[16];
      const uint32_t ta = tmem + ((uint32_t)(32 * eq) << 16) + (uint32_t)(64 * buf + 32 * et + 16 * ech);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
            "=r"(v[14]), "=r"(v[15])
          : "r"(ta)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int il = erow & 15, jrow = erow >> 4;
      __align__(16) __nv_bfloat16 o[16];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const uint4 hq =
            *reinterpret_cast<const uint4 *>(&sm.h[st][jrow + 1][il + 1][16 * ech + 8 * u]);
        const __nv_bfloat16 *hold = reinterpret_cast<const __nv_bfloat16 *>(&hq);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int col = 16 * ech + 8 * u + c;
          const float z = __uint_as_float(v[8 * u + c]) + sm.b[col];
          o[8 * u + c] = __float2bfloat16(lp::bf(hold[c]) + fmaxf(z, 0.f));
        }
      }
      const int ig = i0 + il, jg = j0 + jrow;
      if (ok && ig < nx && jg < ny) {
        uint4 *dst = reinterpret_cast<uint4 *>(
            hout + (((long long)k * ny + jg) * nx + ig) * C + 16 * ech);
        dst[0] = *reinterpret_cast<const uint4 *>(&o[0]);
        dst[1] = *reinterpret_cast<const uint4 *>(&o[8]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      return ok;
    };
    int k = k0;
    for (; k < k1; ++k) {
      const int idx = k - k0 + 1;  // ring index of plane k
      const int buf = (k - k0) & 1;
      bad = bad || !mbar_wait(&sm.full[(idx + 1) % S], ((idx + 1) / S) & 1, abort);
      if (!bad) {
        const int sP = (idx - 1) % S, sC = idx % S, sN = (idx + 1) % S;
        unsigned char *ab = sm.a[buf];
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
#pragma unroll
          for (int c = 0; c < 8; ++c) mb[c] = __float2bfloat16(acc[c]);
          const int row = jr * 16 + il;
          *reinterpret_cast<uint4 *>(ab + tc_off(row, qc >> 3)) = own;
          *reinterpret_cast<uint4 *>(ab + tc_off(row, 4 + (qc >> 3))) =
              *reinterpret_cast<const uint4 *>(mb);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      // every consumer has written its rows of the operand (and finished reading the
      // accumulator buffer the products are about to overwrite)
      if (cons_sync_or(bad || *abort, kCons * 32)) break;
      if (warp == 0 && lane == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a0 = smem_u32(sm.a[buf]), b0 = smem_u32(sm.wb);
#pragma unroll
        for (int t = 0; t < 2; ++t)
#pragma unroll
          for (int kb = 0; kb < 4; ++kb) {
            const uint64_t ad = tc_desc(a0 + t * (kTcABytes / 2) + kb * 256);
            const uint64_t bd = tc_desc(b0 + kb * 256);
            const uint32_t d = tmem + (uint32_t)(64 * buf + 32 * t);
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
                "l"(ad), "l"(bd), "r"(kTcIdesc), "r"((uint32_t)(kb > 0))
                : "memory");
          }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&sm.mma_done[buf]))
            : "memory");
        ++ncommit[buf];
      }
      // plane k-1: its products were issued one step ago; the stage that holds it is
      // released once the epilogue has read its activations
      if (k > k0 && !epilogue(k - 1, buf ^ 1, ((k - 1 - k0) >> 1), (idx - 1) % S)) bad = true;
      bad = __any_sync(0xffffffffu, bad);
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.empty[(idx - 1) % S]);
    }
    if (k == k1 && k1 > k0 && !bad) {  // the last plane's products
      if (!epilogue(k1 - 1, (k1 - 1 - k0) & 1, ((k1 - 1 - k0) >> 1), (k1 - k0) % S)) bad = true;
    }
    bad = __any_sync(0xffffffffu, bad);
    if (bad && lane == 0) {
      *abort = 1;
      if (status) atomicExch(status, FCG_ERR_TIMEOUT);
    }
    if (warp == 0 && lane == 0) {  // products still running write tensor memory: let them end
      for (int b = 0; b < 2; ++b)
        if (ncommit[b] > 0) mbar_wait(&sm.mma_done[b], (ncommit[b] - 1) & 1, nullptr);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols)
                 : "memory");
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
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_lp_layer_hex_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kSmemTcBytes);
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
                  int *status, cudaStream_t st, const OutFuse *out, bool *fused) {
  (void)num_sms;
  if (fused) *fused = false;
  CUtensorMap th, tv;
  if (!encode_maps(g, hin, val, &th, &tv)) return cudaErrorInvalidValue;
  const int ntx = (g.nx + BX - 1) / BX, nty = (g.ny + BY - 1) / BY;
  const dim3 grid((unsigned)(ntx * nty), (unsigned)((g.nz + KC - 1) / KC));
  // the tile product on mma.sync (default) or on tcgen05 (FCG_LP_HEX_MMA=tc: the same bits,
  // measured 1.17 against 0.94 ms per layer at 256^3)
  const char *mm = std::getenv("FCG_LP_HEX_MMA");
  if (mm && std::strcmp(mm, "tc") == 0)
    k_lp_layer_hex_tc<<<grid, kThreads, kSmemTcBytes, st>>>(th, tv, g.nx, g.ny, g.nz, hout, wl,
                                                            bl, done, status);
  else {
    k_lp_layer_hex<<<grid, kThreads, kSmemBytes, st>>>(th, tv, g.nx, g.ny, g.nz, hout, wl, bl,
                                                       done, status, out ? *out : OutFuse{});
    if (out && fused) *fused = true;
  }
  return cudaPeekAtLastError();  // left set for the caller's launch check
}

}  // namespace lphex
}  // namespace fcg
