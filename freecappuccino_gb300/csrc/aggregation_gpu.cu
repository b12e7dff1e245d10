// The aggregation hierarchy of aggregation.cpp built on the device, element for element
// the host construction: the same matching decisions, the same patterns and the same FP64
// values summed in the same order.  The levels, and every solve that uses them, do not
// depend on where they were built.
//
// Matching.  The host matches rows greedily in ascending order: row i, unless an earlier
// row took it, pairs with its untaken neighbour j > i of most negative coupling (the
// first in column order on ties).  Row i's decision depends only on the decisions of the
// earlier rows next to i or next to one of its candidates, so every row is decided in one
// launch: blocks claim 256 rows at a time in ascending order and each row waits for the
// decisions it reads (a value-as-flag wait with an iteration bound, as in the one-launch
// triangular sweeps), in shared memory for rows of its own block.  A row only waits for
// rows claimed before it, by blocks that are running, so the waits end.  The second loop
// (a row left single joins the pair it is most negatively coupled to, as matched, or the
// pair an earlier single joined) reads the earlier singles' joins the same way.  The
// pattern must be structurally symmetric, as a mesh's CSR and its Galerkin products are:
// who may take row i is read from row i.  That chained form serves the fine level, whose
// chains are short; the passes on a coarse level, where consecutive rows are neighbours
// and the chain runs through almost every row, walk the rows in order in one warp
// (k_pm_cands, k_pm_seq below).
//
// Galerkin products and the smoothed level.  One thread per output row enumerates the
// row's contributions in the host's order into an open-addressing table (its own slab of
// a scratch buffer): a column's first contribution is stored as is and the later ones
// added, as the host's RowSum does.  A count pass sizes the rows; the fill pass writes
// each row sorted by column.  A row with more distinct columns than the table holds
// restarts the pass with a larger table.
//
// Compiled with --fmad=false: the FP64 products and sums round as the host's do.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "coarse.h"
#include "fcg_internal.h"
#include "launch.h"

namespace fcg {
namespace ml {

namespace {

constexpr int kUndecided = -2;
constexpr int kAccThreads = 128;

__device__ __forceinline__ int ld_relaxed32(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed32(int *p, int v) {
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The decision at p once it is made; gives up after `spin` polls (or when another wait
// has given up), records the failure in *err and returns -1.  A decision changes once,
// from kUndecided to its value, so a plain (L1-cached) load that sees a value sees the
// final one; only kUndecided is polled again, at L2.  The polls back off up to about a
// microsecond apart, so that waiting blocks do not crowd the L2 (a quarter of a
// microsecond measured slower).
__device__ int wait_decided(const int *p, int *err, int spin) {
  int v = *p;
  if (v != kUndecided) return v;
  v = ld_relaxed32(p);
  if (v != kUndecided) return v;
  unsigned ns = 32;
  for (int it = 0; it < spin; ++it) {
    __nanosleep(ns);
    if (ns < 1024) ns <<= 1;
    v = ld_relaxed32(p);
    if (v != kUndecided) return v;
    if ((it & 15) == 15 && *(volatile const int *)err) break;
  }
  atomicExch(err, 1);
  return -1;
}

// The same for a decision of the calling block's own chunk, in shared memory.
__device__ int wait_shared(const volatile int *p, int *err, int spin) {
  int v = *p;
  for (int it = 0; v == kUndecided && it < spin; ++it) {
    if ((it & 1023) == 1023 && *(volatile const int *)err) break;
    v = *p;
  }
  if (v == kUndecided) {
    atomicExch(err, 1);
    return -1;
  }
  return v;
}

// Rows are claimed kTPB at a time by whole blocks in ascending order; a row's decision is
// published in global memory for later blocks and in shared memory for its own block.
struct Chunk {
  int base;
  volatile int *sh;  // decisions of rows base .. base + kTPB - 1
  const int *gl;     // decisions of every row
  int *err;
  int spin;
  __device__ int get(int r) const {
    return r >= base ? wait_shared(&sh[r - base], err, 16 * spin) : wait_decided(&gl[r], err, spin);
  }
  // the decision if it is made, else kUndecided (no wait)
  __device__ int peek(int r) const {
    if (r >= base) return sh[r - base];
    const int v = gl[r];
    return v != kUndecided ? v : ld_relaxed32(&gl[r]);
  }
};

// Claims the block's next chunk; all threads return the same base (kTPB threads).
__device__ __forceinline__ int claim_chunk(int *counter, int *s_base, volatile int *sh) {
  __syncthreads();  // the previous chunk's decisions are no longer read
  if (threadIdx.x == 0) *s_base = atomicAdd(counter, kTPB);
  sh[threadIdx.x] = kUndecided;
  __syncthreads();
  return *s_base;
}

__global__ void k_fill(int *__restrict__ a, long long n, int v) {
  FCG_GRID_STRIDE(i, n) a[i] = v;
}

__global__ void k_iota(int *__restrict__ a, int n) {
  FCG_GRID_STRIDE(i, n) a[i] = (int)i;
}

// --- fine matrix: CSR values of the scaled operator ------------------------------
__global__ void k_fine_scatter(long long len, const double *__restrict__ sval,
                               const int *__restrict__ src, double *__restrict__ val) {
  FCG_GRID_STRIDE(p, len) {
    const int k = src[p];
    if (k >= 0) val[k] = sval[p];
  }
}

// (a_ik s_i) s_k, as the host scales it
__global__ void k_fine_scale(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                             const double *__restrict__ s, double *__restrict__ val) {
  FCG_GRID_STRIDE(i, n) {
    const double si = s[i];
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) val[k] = (val[k] * si) * s[col[k]];
  }
}

// --- pair matching (aggregation.cpp pair_match) ------------------------------------
// pick[i]: the row leader i paired with, -1 for a row taken by an earlier leader or a
// leader left single; leader[i] = 1 for rows that start an aggregate.  ctl = {claim
// counter, error}.
constexpr int kTaken = -3;  // decide_blocking: an earlier row took row i

// Row i's decision by waiting in column order (the form for rows with more candidates or
// pending rows than the two-phase form holds): the row it pairs with, -1, or kTaken.
__device__ int decide_blocking(int i, const int *__restrict__ ptr, const int *__restrict__ col,
                               const double *__restrict__ val, const Chunk &ch) {
  const int k0 = ptr[i], k1 = ptr[i + 1];
  for (int k = k0; k < k1; ++k) {
    const int j = col[k];
    if (j < i && ch.get(j) == i) return kTaken;
  }
  int best = -1;
  double bv = 0.0;
  for (int k = k0; k < k1; ++k) {
    const int j = col[k];
    if (j <= i) continue;
    const double v = val[k];
    if (!(v < bv)) continue;
    bool jt = false;
    for (int q = ptr[j]; q < ptr[j + 1] && !jt; ++q) {
      const int r = col[q];
      if (r < i && ch.get(r) == j) jt = true;
    }
    if (!jt) {
      bv = v;
      best = j;
    }
  }
  return best;
}

constexpr int kMaxCand = 48;  // candidates of a row in the two-phase form
constexpr int kMaxPend = 96;  // earlier rows still undecided when the row starts

// The decisions form a chain (a row waits for its predecessor when they are neighbours),
// so a row first gathers everything already decided: whether an earlier row took it, and
// for every candidate (a later neighbour with a negative coupling) whether an earlier row
// took that.  It orders the candidates not known to be taken by coupling (the first in
// column order on ties, as the host's scan with a running minimum selects), then waits
// for the undecided rows that may have taken it and, while it is free, for those that may
// have taken its candidates in that order, stopping at the first candidate left free.
__global__ void __launch_bounds__(kTPB)
    k_pm_greedy(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                const double *__restrict__ val, int *pick, int *__restrict__ leader, int *ctl,
                int spin, int absent, bool count_full) {
  __shared__ int s_base;
  __shared__ int s_pick[kTPB];
  for (;;) {
    const int base = claim_chunk(&ctl[0], &s_base, s_pick);
    if (base >= n) return;
    const Chunk ch{base, s_pick, pick, &ctl[1], spin};
    const int i = base + threadIdx.x;
    if (i >= n) continue;
    const int k0 = ptr[i], k1 = ptr[i + 1];
    int prow[kMaxPend];                 // undecided earlier rows: first those that may have
    int cj[kMaxCand], cp0[kMaxCand], cp1[kMaxCand], ord[kMaxCand];  // taken i, then per
    double cv[kMaxCand];                // candidate the range [cp0, cp1) of its takers
    int np = 0, nc = 0, nt = 0;
    bool taken = false, full = false;
    for (int k = k0; k < k1 && !taken; ++k) {
      const int j = col[k];
      if (j >= i) continue;
      const int d = ch.peek(j);
      if (d == i) {
        taken = true;
      } else if (d == kUndecided) {
        if (np == kMaxPend) full = true;
        else prow[np++] = j;
      }
    }
    nt = np;
    if (!taken) {
      for (int k = k0; k < k1 && !full; ++k) {
        const int j = col[k];
        const double v = val[k];
        if (j <= i || !(v < 0.0)) continue;
        if (nc == kMaxCand) {
          full = true;
          break;
        }
        const int p0 = np;
        bool jt = false;
        for (int q = ptr[j]; q < ptr[j + 1]; ++q) {
          const int r = col[q];
          if (r >= i) continue;
          const int d = ch.peek(r);
          if (d == j) {
            jt = true;
            break;
          }
          if (d == kUndecided) {
            if (np == kMaxPend) {
              full = true;
              break;
            }
            prow[np++] = r;
          }
        }
        if (jt) {
          np = p0;  // known taken: its pending rows do not matter
          continue;
        }
        // insert in (coupling, column order)
        int at = nc++;
        while (at > 0 && cv[ord[at - 1]] > v) {
          ord[at] = ord[at - 1];
          --at;
        }
        cj[nc - 1] = j;
        cv[nc - 1] = v;
        cp0[nc - 1] = p0;
        cp1[nc - 1] = np;
        ord[at] = nc - 1;
      }
    }
    int d = -1;
    if (full) {
      if (count_full) atomicAdd(&ctl[2], 1);
      d = decide_blocking(i, ptr, col, val, ch);
      if (d == kTaken) d = -1, taken = true;
    } else {
      for (int q = 0; q < nt && !taken; ++q) taken = ch.get(prow[q]) == i;
      for (int o = 0; o < nc && !taken; ++o) {
        const int t = ord[o], j = cj[t];
        bool jt = false;
        for (int q = cp0[t]; q < cp1[t] && !jt; ++q) jt = ch.get(prow[q]) == j;
        if (!jt) {
          d = j;
          break;
        }
      }
    }
    leader[i] = taken ? 0 : 1;
    if (i == absent) continue;  // diagnostics: this decision is never announced
    ((volatile int *)s_pick)[threadIdx.x] = d;
    st_relaxed32(&pick[i], d);
  }
}

// --- pair matching in order, for the coarse levels ----------------------------------
// On a Galerkin level consecutive rows are neighbours, so the decisions above form one
// chain through almost every row and each row spends its turn rescanning its neighbours'
// decisions.  There the pass runs as the host's loop itself: k_pm_cands lists every
// row's candidates in the order the host prefers them (most negative coupling first, the
// lower column on ties), and k_pm_seq walks the rows in ascending order in one warp with
// the taken flags of the rows ahead in shared memory.  A row takes the first candidate
// of its list that no earlier row took, so the decisions are the host's.
constexpr int kSeqCand = 8;          // candidates of a row kept in order
constexpr int kSeqRing = 1 << 17;    // taken flags of the rows i .. i + kSeqRing - 1 (bytes)
constexpr int kSeqMargin = 8;        // candidates lie this far inside the ring
constexpr int kSeqBatch = 512;       // candidate lists staged per batch
constexpr int kSeqThreads = 128;     // warp 0 decides, warps 1-3 stage the next batch
constexpr size_t kSeqSmem = kSeqRing + 2 * kSeqBatch * (kSeqCand + 2) * sizeof(int);
constexpr int kNoCand = -2;          // an empty slot of a candidate list

// cand[8 i ..]: the first kSeqCand candidates of row i (j > i, a_ij < 0) in order of
// preference, kNoCand after the last; ncand[i] their number; ctl[3] = the largest j - i.
__global__ void k_pm_cands(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                           const double *__restrict__ val, int *__restrict__ cand,
                           int *__restrict__ ncand, int *ctl) {
  int far = 0;
  FCG_GRID_STRIDE(i, n) {
    double kv[kSeqCand];
    int kc[kSeqCand];
#pragma unroll
    for (int s = 0; s < kSeqCand; ++s) kv[s] = 0.0, kc[s] = kNoCand;
    int cnt = 0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      const double v = val[k];
      if (j <= (int)i || !(v < 0.0)) continue;
      ++cnt;
      far = max(far, j - (int)i);
      // insertion into the ordered list; an empty slot (value 0) never precedes an entry
      double cv = v;
      int cc = j;
#pragma unroll
      for (int s = 0; s < kSeqCand; ++s) {
        const bool first = kc[s] == kNoCand || cv < kv[s] || (cv == kv[s] && cc < kc[s]);
        const double tv = first ? kv[s] : cv;
        const int tc = first ? kc[s] : cc;
        kv[s] = first ? cv : kv[s];
        kc[s] = first ? cc : kc[s];
        cv = tv;
        cc = tc;
      }
    }
    int4 *o = reinterpret_cast<int4 *>(cand + (long long)kSeqCand * i);
    o[0] = make_int4(kc[0], kc[1], kc[2], kc[3]);
    o[1] = make_int4(kc[4], kc[5], kc[6], kc[7]);
    ncand[i] = cnt;
  }
  far = __reduce_max_sync(0xffffffffu, far);
  if ((threadIdx.x & 31) == 0 && far > 0) atomicMax(&ctl[3], far);
}

// Row i's choice when all of its first kSeqCand candidates are taken and it has more:
// the whole warp scans the row against the flags (every earlier decision is in them).
// Not inlined: its row loads must not be hoisted into the decision loop.
__device__ __noinline__ int seq_scan_row(int i, const int *__restrict__ ptr, const int *__restrict__ col,
                            const double *__restrict__ val, const unsigned char *ring,
                            int lane) {
  double bv = 0.0;
  int bj = -1;
  for (int k = ptr[i] + lane; k < ptr[i + 1]; k += 32) {
    const int j = col[k];
    const double v = val[k];
    if (j <= i || !(v < 0.0) || ring[j & (kSeqRing - 1)]) continue;
    if (bj < 0 || v < bv || (v == bv && j < bj)) bv = v, bj = j;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, bv, off);
    const int oj = __shfl_xor_sync(0xffffffffu, bj, off);
    if (oj >= 0 && (bj < 0 || ov < bv || (ov == bv && oj < bj))) bv = ov, bj = oj;
  }
  return bj;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned lds_u8(uint32_t a) {
  unsigned v;
  asm volatile("ld.shared.u8 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ int lds_s32(uint32_t a) {
  int v;
  asm volatile("ld.shared.s32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ int4 lds_v4(uint32_t a) {
  int4 v;
  asm volatile("ld.shared.v4.s32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"(a));
  return v;
}
__device__ __forceinline__ void sts_u8_if(bool p, uint32_t a, unsigned v) {
  asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %0, 0;\n @q st.shared.u8 [%1], %2;\n}" ::"r"(
                   (unsigned)p),
               "r"(a), "r"(v));
}
__device__ __forceinline__ void sts_s32_if(bool p, uint32_t a, int v) {
  asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %0, 0;\n @q st.shared.s32 [%1], %2;\n}" ::"r"(
                   (unsigned)p),
               "r"(a), "r"(v));
}

// One block.  Batches of kSeqBatch candidate lists are staged in shared memory by warps
// 1-3 while warp 0 decides the batch before; they also write out the decisions of the
// batch before that.  The decision loop touches shared memory only.  Warp 0 decides row i
// with lanes 0-7 on the
// row's candidate slots and lane 8 on the row itself: each lane reads its taken flag,
// one ballot gives which are free, and the first free candidate is chosen.  The flags
// of row i + 1 are read while row i is decided, so they miss only row i's decision,
// which is compared in.  ring[r mod kSeqRing] is the flag of row r; a decided row
// clears its own, which then stands for row r + kSeqRing (candidates lie less than
// kSeqRing - kSeqMargin rows ahead: k_pm_cands checks).  Nothing waits: each row is
// decided after the rows before it, by the same warp.
__global__ void __launch_bounds__(kSeqThreads, 1)
    k_pm_seq(int n, const int *__restrict__ cand, const int *__restrict__ ncand,
             const int *__restrict__ ptr, const int *__restrict__ col,
             const double *__restrict__ val, int *__restrict__ pick, int *__restrict__ leader) {
  extern __shared__ __align__(16) unsigned char seq_smem[];
  unsigned char *ring = seq_smem;
  int *buf = reinterpret_cast<int *>(seq_smem + kSeqRing);
  int *dec = buf + 2 * kSeqBatch * kSeqCand;  // decisions of two batches (kTaken: taken)
  int *cnb = dec + 2 * kSeqBatch;             // candidate counts of two batches
  constexpr int M = kSeqRing - 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int t = threadIdx.x; t < kSeqRing / 16; t += blockDim.x)
    reinterpret_cast<uint4 *>(ring)[t] = make_uint4(0, 0, 0, 0);
  const int nb = (n + kSeqBatch - 1) / kSeqBatch;
  auto stage = [&](int b, int t0, int nt) {
    const int r0 = b * kSeqBatch, rows = min(kSeqBatch, n - r0);
    const int4 *src = reinterpret_cast<const int4 *>(cand + (long long)kSeqCand * r0);
    int4 *dst = reinterpret_cast<int4 *>(buf + (b & 1) * kSeqBatch * kSeqCand);
    for (int t = t0; t < 2 * rows; t += nt) dst[t] = src[t];
    for (int t = t0; t < rows; t += nt) cnb[(b & 1) * kSeqBatch + t] = ncand[r0 + t];
  };
  auto flush = [&](int b, int t0, int nt) {
    const int r0 = b * kSeqBatch, rows = min(kSeqBatch, n - r0);
    const int *src = dec + (b & 1) * kSeqBatch;
    for (int t = t0; t < rows; t += nt) {
      const int v = src[t];
      pick[r0 + t] = v == kTaken ? -1 : v;
      leader[r0 + t] = v == kTaken ? 0 : 1;
    }
  };
  if (nb > 0) stage(0, threadIdx.x, blockDim.x);
  __syncthreads();
  for (int b = 0; b < nb; ++b) {
    if (warp != 0) {
      if (b + 1 < nb) stage(b + 1, threadIdx.x - 32, blockDim.x - 32);
      if (b > 0) flush(b - 1, threadIdx.x - 32, blockDim.x - 32);
    } else {
      const int r0 = b * kSeqBatch, r1 = min(n, r0 + kSeqBatch);
      const uint32_t ring_s = smem_u32(ring);
      // this lane's id in a row's list: its candidate slot (lanes 0-7), the row (lane 8);
      // the two rows after a batch read the staged words that follow it (in bounds of the
      // shared buffer; their flags are read but never used)
      const int *cb = buf + (b & 1) * kSeqBatch * kSeqCand;
      const uint32_t cb_s = smem_u32(cb + lane);
      const uint32_t db_s = smem_u32(dec + (b & 1) * kSeqBatch);
      const uint32_t nb_s = smem_u32(cnb + (b & 1) * kSeqBatch);
      const bool slot = lane < kSeqCand, self = lane == kSeqCand;
      auto id_of = [&](int r) -> int {
        return slot ? lds_s32(cb_s + 4u * (uint32_t)((r - r0) * kSeqCand)) : (self ? r : kNoCand);
      };
      auto flag_of = [&](int id) -> unsigned {
        return id >= 0 ? lds_u8(ring_s + ((uint32_t)id & M)) : 0u;
      };
      // a row's whole list in every lane
      const uint32_t cl_s = smem_u32(cb);
      auto list_of = [&](int r, int4 &lo, int4 &hi) {
        const uint32_t a = cl_s + 4u * (uint32_t)((r - r0) * kSeqCand);
        lo = lds_v4(a);
        hi = lds_v4(a + 16u);
      };
      // the slots of a list that hold id (bit k for slot k)
      auto eq_of = [](int id, const int4 &lo, const int4 &hi) -> unsigned {
        return (lo.x == id ? 1u : 0u) | (lo.y == id ? 2u : 0u) | (lo.z == id ? 4u : 0u) |
               (lo.w == id ? 8u : 0u) | (hi.x == id ? 16u : 0u) | (hi.y == id ? 32u : 0u) |
               (hi.z == id ? 64u : 0u) | (hi.w == id ? 128u : 0u);
      };
      int4 lo, hi;
      list_of(r0, lo, hi);
      int mine = id_of(r0);
      unsigned f = flag_of(mine);
      int mine1 = id_of(r0 + 1);
      unsigned eq = 0, selp = 0;  // row r0's flags miss no decision
      // Row i is decided from its flags, read after every decision up to row i - 2 was
      // stored, and from row i - 1's choice: a lane's id is taken if its flag is set or
      // if it is the candidate row i - 1 chose (its slot bit selp, against eq, the slots
      // of row i - 1 that hold the id).  The chosen slot's own lane then flags and
      // records it, so no lane waits for the choice to be broadcast.
#pragma unroll 2
      for (int i = r0; i < r1; ++i) {
        // flags of row i + 1 (every decision before row i is in the ring), its eq against
        // row i, the ids of row i + 2 and the list of row i + 1
        const unsigned f1 = flag_of(mine1);
        const unsigned eq1 = eq_of(mine1, lo, hi);
        const int mine2 = id_of(i + 2);
        int4 lo1, hi1;
        list_of(i + 1, lo1, hi1);
        const bool t = f != 0u || (eq & selp) != 0u;
        const unsigned bal = __ballot_sync(0xffffffffu, slot ? (mine >= 0 && !t) : (self && t));
        const unsigned fr = bal & 0xffu;
        const bool taken = (bal >> kSeqCand) & 1u;
        const unsigned sel = taken ? 0u : (fr & (0u - fr));
        // the chosen slot's lane flags its candidate and records it; the row's lane
        // clears the row's flag (it now stands for row i + kSeqRing) and records a row
        // left single or taken
        const bool chosen = slot && ((sel >> lane) & 1u);
        const uint32_t da = db_s + 4u * (uint32_t)(i - r0);
        sts_u8_if(chosen, ring_s + ((uint32_t)mine & M), 1u);
        sts_s32_if(chosen, da, mine);
        sts_s32_if(self && sel == 0u, da, taken ? kTaken : -1);
        sts_u8_if(self, ring_s + ((uint32_t)i & M), 0u);
        unsigned f1c = f1;
        if (!taken && fr == 0u && lds_s32(nb_s + 4u * (uint32_t)(i - r0)) > kSeqCand) {
          // every listed candidate taken: scan the row; row i + 1 then rereads its flags,
          // which hold every decision up to this one (selp stays 0)
          __syncwarp();
          const int d = seq_scan_row(i, ptr, col, val, ring, lane);
          sts_u8_if(lane == 0 && d >= 0, ring_s + ((uint32_t)d & M), 1u);
          sts_s32_if(lane == 0, da, d);
          __syncwarp();
          f1c = flag_of(mine1);
        }
        __syncwarp();
        lo = lo1, hi = hi1, mine = mine1, f = f1c, eq = eq1;
        mine1 = mine2;
        selp = sel;
      }
    }
    __syncthreads();
  }
  if (nb > 0) flush(nb - 1, threadIdx.x, blockDim.x);
}

// join[i] for a leader left single: the row whose aggregate it joins, or -1.  A neighbour
// j counts as paired when it is in a pair of the first loop, or is an earlier single that
// joined one.
__global__ void __launch_bounds__(kTPB)
    k_pm_join(int n, const int *__restrict__ ptr, const int *__restrict__ col,
              const double *__restrict__ val, const int *__restrict__ pick,
              const int *__restrict__ leader, int *join, int *ctl, int spin) {
  __shared__ int s_base;
  __shared__ int s_join[kTPB];
  for (;;) {
    const int base = claim_chunk(&ctl[0], &s_base, s_join);
    if (base >= n) return;
    const Chunk ch{base, s_join, join, &ctl[1], spin};
    const int i = base + threadIdx.x;
    if (i >= n) continue;
    if (!leader[i] || pick[i] >= 0) continue;  // join[] is read for singles only
    int best = -1;
    double bv = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      if (j == i) continue;
      bool pj;
      if (!leader[j] || pick[j] >= 0)
        pj = true;
      else if (j < i)
        pj = ch.get(j) >= 0;
      else
        pj = false;
      if (pj && val[k] < bv) {
        bv = val[k];
        best = j;
      }
    }
    st_relaxed32(&join[i], best);
    ((volatile int *)s_join)[threadIdx.x] = best;
  }
}

// picker[j] = the leader that paired with j
__global__ void k_pm_pickers(int n, const int *__restrict__ pick, const int *__restrict__ leader,
                             int *__restrict__ picker) {
  FCG_GRID_STRIDE(i, n) {
    if (leader[i] && pick[i] >= 0) picker[pick[i]] = (int)i;
  }
}

// First-loop aggregate of every row (the leader's rank among the leaders), then the joins
// followed to a row of a pair; used[] marks the aggregates that keep a row.
__global__ void k_pm_assign(int n, const int *__restrict__ pick, const int *__restrict__ leader,
                            const int *__restrict__ picker, const int *__restrict__ join,
                            const int *__restrict__ lrank, int *__restrict__ agg,
                            int *__restrict__ used) {
  FCG_GRID_STRIDE(i, n) {
    int r = (int)i;
    while (leader[r] && pick[r] < 0 && join[r] >= 0) r = join[r];  // joins lead to a pair
    const int a = leader[r] ? lrank[r] : lrank[picker[r]];
    agg[i] = a;
    used[a] = 1;
  }
}

__global__ void k_pm_renumber(int n, const int *__restrict__ id, int *__restrict__ agg) {
  FCG_GRID_STRIDE(i, n) agg[i] = id[agg[i]];
}

// --- members: rows of every aggregate, ascending --------------------------------------
__global__ void k_count(long long n, const int *__restrict__ key, int *__restrict__ cnt) {
  FCG_GRID_STRIDE(i, n) atomicAdd(&cnt[key[i]], 1);
}

__global__ void k_bucket(long long n, const int *__restrict__ key, int *__restrict__ cursor,
                         int *__restrict__ out) {
  FCG_GRID_STRIDE(i, n) out[atomicAdd(&cursor[key[i]], 1)] = (int)i;
}

// Sorts every segment [ptr[s], ptr[s+1]) of a ascending (and b along with it, if given).
__global__ void k_sort_segments(int ns, const int *__restrict__ ptr, int *__restrict__ a,
                                int *__restrict__ b) {
  FCG_GRID_STRIDE(s, ns) {
    const int lo = ptr[s], hi = ptr[s + 1];
    for (int k = lo + 1; k < hi; ++k) {
      const int v = a[k], w = b ? b[k] : 0;
      int j = k - 1;
      while (j >= lo && a[j] > v) {
        a[j + 1] = a[j];
        if (b) b[j + 1] = b[j];
        --j;
      }
      a[j + 1] = v;
      if (b) b[j + 1] = w;
    }
  }
}

__global__ void k_compose(int n, const int *__restrict__ agg, int *__restrict__ comp) {
  FCG_GRID_STRIDE(i, n) comp[i] = agg[comp[i]];
}

// --- rows accumulated in order: Galerkin, A P, P^T A P -----------------------------
__device__ __forceinline__ unsigned slot_of(int key, int cap) {
  return ((unsigned)key * 2654435761u) & (unsigned)(cap - 1);
}

// One thread's table: cap slots (keys -1 when empty), values, and the slots in use.
struct Table {
  int *key;
  double *val;
  int *used;
  int cap, m;
  bool over;
  template <bool VALS>
  __device__ void add(int J, double v) {
    if (over) return;
    unsigned h = slot_of(J, cap);
    for (;;) {
      const int k = key[h];
      if (k == J) {
        if (VALS) val[h] += v;
        return;
      }
      if (k < 0) {
        if (m >= (cap >> 1) + (cap >> 2)) {
          over = true;
          return;
        }
        key[h] = J;
        if (VALS) val[h] = v;  // the first contribution as is, as the host's RowSum
        used[m++] = (int)h;
        return;
      }
      h = (h + 1) & (unsigned)(cap - 1);
    }
  }
  __device__ void clear() {
    for (int q = 0; q < m; ++q) key[used[q]] = -1;
    m = 0;
    over = false;
  }
};

// Galerkin row I of the piecewise-constant P: member rows ascending, their entries in
// column order, each added to the slot of its aggregate.
struct GenGalerkin {
  const int *mptr, *mem, *ptr, *col, *agg;
  const double *val;
  template <class F>
  __device__ void operator()(int I, F &&f) const {
    for (int m = mptr[I]; m < mptr[I + 1]; ++m) {
      const int i = mem[m];
      for (int k = ptr[i]; k < ptr[i + 1]; ++k) f(agg[col[k]], val[k]);
    }
  }
};

// (A P) row i: the row's entries in column order, a_ik P_kJ in P_k's order.
struct GenAP {
  const int *ptr, *col, *p_ptr, *p_col;
  const double *val, *pv;
  template <class F>
  __device__ void operator()(int i, F &&f) const {
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      const double a = val[k];
      for (int p = p_ptr[j]; p < p_ptr[j + 1]; ++p) f(p_col[p], a * pv[p]);
    }
  }
};

// (P^T A P) row I: the rows whose P row holds I, ascending, P_iI (A P)_iJ in column order.
struct GenPtAP {
  const int *t_ptr, *t_row, *t_pos, *ap_ptr, *ap_col;
  const double *pv, *apv;
  template <class F>
  __device__ void operator()(int I, F &&f) const {
    for (int m = t_ptr[I]; m < t_ptr[I + 1]; ++m) {
      const int i = t_row[m];
      const double p = pv[t_pos[m]];
      for (int q = ap_ptr[i]; q < ap_ptr[i + 1]; ++q) f(ap_col[q], p * apv[q]);
    }
  }
};

// P's pattern row i: the row's own aggregate and its neighbours' aggregates.
struct GenPPattern {
  const int *ptr, *col, *agg;
  template <class F>
  __device__ void operator()(int i, F &&f) const {
    f(agg[i], 0.0);
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) f(agg[col[k]], 0.0);
  }
};

// Count pass (FILL false): cnt[r] = distinct columns of row r.  Fill pass: the row's
// columns ascending with their sums at optr[r].  ctl[0] is set when a row does not fit.
template <class Gen, bool FILL, bool VALS>
__global__ void __launch_bounds__(kAccThreads)
    k_acc_rows(int nrows, Gen gen, int cap, int *__restrict__ skey, double *__restrict__ sval,
               int *__restrict__ sused, int *__restrict__ cnt, const int *__restrict__ optr,
               int *__restrict__ ocol, double *__restrict__ oval, int *ctl) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Table t{skey + tid * cap, VALS ? sval + tid * cap : nullptr, sused + tid * cap, cap, 0, false};
  for (int q = 0; q < cap; ++q) t.key[q] = -1;
  for (long long r = tid; r < nrows; r += (long long)gridDim.x * blockDim.x) {
    gen((int)r, [&](int J, double v) { t.add<VALS>(J, v); });
    if (t.over) {
      atomicExch(&ctl[0], 1);
    } else if (!FILL) {
      cnt[r] = t.m;
    } else {
      const int b = optr[r];
      for (int q = 0; q < t.m; ++q) {  // insertion by column
        const int h = t.used[q], J = t.key[h];
        const double v = VALS ? t.val[h] : 0.0;
        int j = b + q - 1;
        while (j >= b && ocol[j] > J) {
          ocol[j + 1] = ocol[j];
          if (VALS) oval[j + 1] = oval[j];
          --j;
        }
        ocol[j + 1] = J;
        if (VALS) oval[j + 1] = v;
      }
    }
    t.clear();
  }
}

// P's values on its pattern: 1 at the own aggregate, then minus (omega / a_ii) a_ik for
// the row's entries in column order (aggregation.cpp smoothed_level).
__global__ void k_p_values(int n, const int *__restrict__ ptr, const int *__restrict__ col,
                           const double *__restrict__ val, const int *__restrict__ agg,
                           const int *__restrict__ p_ptr, const int *__restrict__ p_col,
                           double omega, double *__restrict__ pv) {
  FCG_GRID_STRIDE(i, n) {
    const int b = p_ptr[i], e = p_ptr[i + 1];
    double d = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
      if (col[k] == (int)i) d = val[k];
    const double w = d > 0.0 ? omega / d : 0.0;
    const int own = agg[i];
    for (int p = b; p < e; ++p) pv[p] = p_col[p] == own ? 1.0 : 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int J = agg[col[k]];
      int lo = b, hi = e - 1;  // the column is in the row
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (p_col[mid] < J) lo = mid + 1;
        else hi = mid;
      }
      pv[lo] -= w * val[k];
    }
  }
}

// t lists of P: for every aggregate the rows whose P row holds it with the positions.
__global__ void k_t_bucket(int n, const int *__restrict__ p_ptr, const int *__restrict__ p_col,
                           int *__restrict__ cursor, int *__restrict__ t_row,
                           int *__restrict__ t_pos) {
  FCG_GRID_STRIDE(i, n) {
    for (int p = p_ptr[i]; p < p_ptr[i + 1]; ++p) {
      const int f = atomicAdd(&cursor[p_col[p]], 1);
      t_row[f] = (int)i;
      t_pos[f] = p;
    }
  }
}

// --- host side -------------------------------------------------------------------
struct Ctx {
  fcg_context *c;
  std::string &err;
  bool trace = false;  // FCG_AGG_TRACE=1: seconds of every stage on stderr
  bool first_pass = true;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  void mark(const char *what, long long rows) {
    if (!trace) return;
    cudaStreamSynchronize(c->stream);
    const auto t = std::chrono::steady_clock::now();
    std::fprintf(stderr, "aggregation: %-10s %10lld rows %8.3f s\n", what, rows,
                 std::chrono::duration<double>(t - t0).count());
    t0 = t;
  }
  DBuf scan_tmp, ctl, cnt;
  DBuf skey, sval, sused;  // accumulation slabs
  DBuf m_pick, m_leader, m_join, m_picker, m_lrank, m_used, m_id;  // matching scratch
  DBuf m_cand, m_ncand;  // candidate lists of the in-order form
  bool seq_on = true;    // FCG_AGG_SEQ=0: the coarse levels match with the chained form too
  DBuf p_agg, p_mptr, p_mem;  // one pass's aggregates and members
  int cap = 64;
  long long slab_threads = 0;
  void release() {
    for (DBuf *b : {&scan_tmp, &ctl, &cnt, &skey, &sval, &sused, &m_pick, &m_leader, &m_join,
                    &m_picker, &m_lrank, &m_used, &m_id, &m_cand, &m_ncand, &p_agg, &p_mptr,
                    &p_mem})
      b->release();
  }
};

int cuda_fail(Ctx &x, cudaError_t e, const char *what) {
  x.err = std::string(what) + ": " + cudaGetErrorString(e);
  return FCG_ERR_CUDA;
}

#define AG_TRY(call, what)                                \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(x, e_, what); \
  } while (0)

int read_int(Ctx &x, const int *dptr, int *out) {
  AG_TRY(cudaMemcpyAsync(out, dptr, sizeof(int), cudaMemcpyDeviceToHost, x.c->stream), "read");
  AG_TRY(cudaStreamSynchronize(x.c->stream), "read");
  return FCG_OK;
}

int ints(Ctx &x, DBuf &b, long long n) {
  AG_TRY(b.ensure(sizeof(int) * (size_t)(n > 0 ? n : 1)), "hierarchy allocation");
  return FCG_OK;
}

int dbls(Ctx &x, DBuf &b, long long n) {
  AG_TRY(b.ensure(sizeof(double) * (size_t)(n > 0 ? n : 1)), "hierarchy allocation");
  return FCG_OK;
}

// Exclusive scan of n counts into out (n + 1 entries); *total = out[n].
int scan(Ctx &x, const int *in, DBuf &out, int n, int *total) {
  int rc;
  if ((rc = ints(x, out, (long long)n + 1))) return rc;
  if ((rc = scan_ints(x.c, in, out.as<int>(), n, x.scan_tmp))) return rc;
  return read_int(x, out.as<int>() + n, total);
}

// Rows of every aggregate in ascending order (aggregation.cpp members).
int members(Ctx &x, int n, int m, const int *agg, DBuf &mptr, DBuf &mem) {
  fcg_context *c = x.c;
  int rc, total;
  if ((rc = ints(x, x.cnt, m)) || (rc = ints(x, mem, n))) return rc;
  AG_TRY(cudaMemsetAsync(x.cnt.p, 0, sizeof(int) * (size_t)(m > 0 ? m : 1), c->stream), "members");
  k_count<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, agg, x.cnt.as<int>());
  if ((rc = scan(x, x.cnt.as<int>(), mptr, m, &total))) return rc;
  AG_TRY(cudaMemcpyAsync(x.cnt.p, mptr.p, sizeof(int) * (size_t)m, cudaMemcpyDeviceToDevice,
                         c->stream), "members");
  k_bucket<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, agg, x.cnt.as<int>(), mem.as<int>());
  k_sort_segments<<<grid_for(m, c->num_sms), kTPB, 0, c->stream>>>(m, mptr.as<int>(), mem.as<int>(),
                                                                   nullptr);
  AG_TRY(cudaGetLastError(), "members");
  return FCG_OK;
}

// The in-order form of one pass (pick, leader as k_pm_greedy gives them); *done = false
// when a candidate lies beyond the flag ring (the caller then runs the chained form).
int match_in_order(Ctx &x, const DevCsr &a, int *pick, int *leader, bool *done) {
  fcg_context *c = x.c;
  const int n = a.n;
  int *ctl = x.ctl.as<int>();
  int rc, far = 0;
  *done = false;
  if ((rc = ints(x, x.m_cand, (long long)kSeqCand * n)) || (rc = ints(x, x.m_ncand, n))) return rc;
  AG_TRY(cudaMemsetAsync(ctl + 3, 0, sizeof(int), c->stream), "matching");
  k_pm_cands<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(
      n, a.ptr, a.col, a.val, x.m_cand.as<int>(), x.m_ncand.as<int>(), ctl);
  AG_TRY(cudaGetLastError(), "matching");
  if ((rc = read_int(x, ctl + 3, &far))) return rc;
  if (far >= kSeqRing - kSeqMargin) return FCG_OK;
  AG_TRY(cudaFuncSetAttribute(k_pm_seq, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kSeqSmem), "matching");
  k_pm_seq<<<1, kSeqThreads, kSeqSmem, c->stream>>>(n, x.m_cand.as<int>(), x.m_ncand.as<int>(),
                                                   a.ptr, a.col, a.val, pick, leader);
  AG_TRY(cudaGetLastError(), "matching");
  *done = true;
  return FCG_OK;
}

// One pass of pairwise matching on a; agg (a.n) gets the aggregates, *m their count.
// in_order: decide the pairs with the in-order form (coarse levels), else the chained one.
int match(Ctx &x, const DevCsr &a, DBuf &agg, int *m, bool in_order) {
  fcg_context *c = x.c;
  const int n = a.n;
  // scratch kept across passes (the first pass is the largest)
  DBuf &pick = x.m_pick, &leader = x.m_leader, &join = x.m_join, &picker = x.m_picker,
       &lrank = x.m_lrank, &used = x.m_used, &id = x.m_id;
  int rc;
  if ((rc = ints(x, pick, n)) || (rc = ints(x, leader, n)) || (rc = ints(x, join, n)) ||
      (rc = ints(x, picker, n)) || (rc = ints(x, agg, n)))
    return rc;
  int *ctl = x.ctl.as<int>();
  const int g = grid_for(n, c->num_sms);
  const int gw = std::max(1, std::min((n + kTPB - 1) / kTPB, c->num_sms * 8));
  const int spin = c->agg_test_polls > 0 ? c->agg_test_polls : 1 << 22;
  const int absent = x.first_pass ? c->agg_test_row : -1;
  x.first_pass = false;
  int fail = 0;
  bool done = false;
  k_fill<<<g, kTPB, 0, c->stream>>>(join.as<int>(), n, kUndecided);
  if (in_order && absent < 0 && x.seq_on &&
      (rc = match_in_order(x, a, pick.as<int>(), leader.as<int>(), &done)))
    return rc;
  if (done) {
    if (x.trace) std::fprintf(stderr, "aggregation: %d rows decided in order\n", n);
  } else {
    k_fill<<<g, kTPB, 0, c->stream>>>(pick.as<int>(), n, kUndecided);
    AG_TRY(cudaMemsetAsync(ctl, 0, 2 * sizeof(int), c->stream), "matching");
    AG_TRY(cudaMemsetAsync(ctl + 2, 0, sizeof(int), c->stream), "matching");
    k_pm_greedy<<<gw, kTPB, 0, c->stream>>>(n, a.ptr, a.col, a.val, pick.as<int>(),
                                           leader.as<int>(), ctl, spin, absent, x.trace);
    AG_TRY(cudaGetLastError(), "matching");
    if ((rc = read_int(x, ctl + 1, &fail))) return rc;
    if (fail) {
      x.err = "aggregation: a matching wait gave up";
      return FCG_ERR_TIMEOUT;
    }
    if (x.trace) {
      int nfull = 0;
      if ((rc = read_int(x, ctl + 2, &nfull))) return rc;
      std::fprintf(stderr, "aggregation: %d of %d rows decided by the blocking form\n", nfull, n);
    }
  }
  AG_TRY(cudaMemsetAsync(ctl, 0, 2 * sizeof(int), c->stream), "matching");
  k_pm_join<<<gw, kTPB, 0, c->stream>>>(n, a.ptr, a.col, a.val, pick.as<int>(), leader.as<int>(),
                                       join.as<int>(), ctl, spin);
  AG_TRY(cudaGetLastError(), "matching");
  if ((rc = read_int(x, ctl + 1, &fail))) return rc;
  if (fail) {
    x.err = "aggregation: a joining wait gave up";
    return FCG_ERR_TIMEOUT;
  }
  k_pm_pickers<<<g, kTPB, 0, c->stream>>>(n, pick.as<int>(), leader.as<int>(), picker.as<int>());
  int nc1 = 0;
  if ((rc = scan(x, leader.as<int>(), lrank, n, &nc1)) || (rc = ints(x, used, nc1))) return rc;
  AG_TRY(cudaMemsetAsync(used.p, 0, sizeof(int) * (size_t)(nc1 > 0 ? nc1 : 1), c->stream),
         "matching");
  k_pm_assign<<<g, kTPB, 0, c->stream>>>(n, pick.as<int>(), leader.as<int>(), picker.as<int>(),
                                        join.as<int>(), lrank.as<int>(), agg.as<int>(),
                                        used.as<int>());
  if ((rc = scan(x, used.as<int>(), id, nc1, m))) return rc;
  if (*m < nc1)  // aggregates a single left: renumber in order
    k_pm_renumber<<<g, kTPB, 0, c->stream>>>(n, id.as<int>(), agg.as<int>());
  AG_TRY(cudaGetLastError(), "matching");
  return FCG_OK;
}

// Rows of nrows accumulated by gen into (ptr, col[, val]), each row sorted by column.
template <class Gen, bool VALS>
int acc_rows(Ctx &x, int nrows, const Gen &gen, DBuf &ptr, DBuf &col, DBuf *val,
             long long *nnz) {
  fcg_context *c = x.c;
  int rc;
  int *ctl = x.ctl.as<int>();
  if ((rc = ints(x, x.cnt, nrows))) return rc;
  for (;;) {
    // threads: enough for the rows, at most 256 MB of slabs (more threads measured slower:
    // the tables then spill out of L1)
    const long long budget = (256LL << 20) / (16LL * x.cap);
    long long thr = std::min<long long>({(long long)nrows, (long long)c->num_sms * 512, budget});
    thr = std::max<long long>(kAccThreads, (thr + kAccThreads - 1) / kAccThreads * kAccThreads);
    if ((rc = ints(x, x.skey, thr * x.cap)) || (rc = dbls(x, x.sval, thr * x.cap)) ||
        (rc = ints(x, x.sused, thr * x.cap)))
      return rc;
    x.slab_threads = thr;
    AG_TRY(cudaMemsetAsync(ctl, 0, sizeof(int), c->stream), "accumulation");
    k_acc_rows<Gen, false, false><<<(int)(thr / kAccThreads), kAccThreads, 0, c->stream>>>(
        nrows, gen, x.cap, x.skey.as<int>(), x.sval.as<double>(), x.sused.as<int>(),
        x.cnt.as<int>(), nullptr, nullptr, nullptr, ctl);
    AG_TRY(cudaGetLastError(), "accumulation");
    int over = 0;
    if ((rc = read_int(x, ctl, &over))) return rc;
    if (!over) break;
    if (x.cap >= 8192) {
      x.err = "aggregation: a coarse row has more than 6144 columns";
      return FCG_ERR_UNSUPPORTED;
    }
    x.cap *= 2;
  }
  int total = 0;
  if ((rc = scan(x, x.cnt.as<int>(), ptr, nrows, &total)) || (rc = ints(x, col, total)) ||
      (val && (rc = dbls(x, *val, total))))
    return rc;
  const long long thr = x.slab_threads;
  k_acc_rows<Gen, true, VALS><<<(int)(thr / kAccThreads), kAccThreads, 0, c->stream>>>(
      nrows, gen, x.cap, x.skey.as<int>(), x.sval.as<double>(), x.sused.as<int>(), nullptr,
      ptr.as<int>(), col.as<int>(), val ? val->as<double>() : nullptr, ctl);
  AG_TRY(cudaGetLastError(), "accumulation");
  *nnz = total;
  return FCG_OK;
}

int galerkin(Ctx &x, const DevCsr &a, const int *agg, int m, const int *mptr, const int *mem,
             DevMat &dst) {
  GenGalerkin gen{mptr, mem, a.ptr, a.col, agg, a.val};
  dst.n = m;
  return acc_rows<GenGalerkin, true>(x, m, gen, dst.ptr, dst.col, &dst.val, &dst.nnz);
}

// aggregation.cpp smoothed_level: P, its transpose lists, A P and P^T A P of level lv
// below A.
int smoothed(Ctx &x, const DevCsr &A, double omega, DevBuiltLevel &lv) {
  fcg_context *c = x.c;
  const int n = A.n, nc = lv.n;
  const int *agg = lv.agg.as<int>();
  DBuf pv, apv;
  struct Rel {
    DBuf *b[2];
    ~Rel() {
      for (DBuf *p : b) p->release();
    }
  } rel{{&pv, &apv}};
  int rc, total;
  GenPPattern gp{A.ptr, A.col, agg};
  if ((rc = acc_rows<GenPPattern, false>(x, n, gp, lv.p_ptr, lv.p_col, nullptr, &lv.p_nnz)) ||
      (rc = dbls(x, pv, lv.p_nnz)))
    return rc;
  k_p_values<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(
      n, A.ptr, A.col, A.val, agg, lv.p_ptr.as<int>(), lv.p_col.as<int>(), omega, pv.as<double>());
  // transpose lists, rows ascending within every aggregate
  if ((rc = ints(x, x.cnt, nc)) || (rc = ints(x, lv.t_row, lv.p_nnz)) ||
      (rc = ints(x, lv.t_pos, lv.p_nnz)))
    return rc;
  AG_TRY(cudaMemsetAsync(x.cnt.p, 0, sizeof(int) * (size_t)nc, c->stream), "smoothed level");
  k_count<<<grid_for(lv.p_nnz, c->num_sms), kTPB, 0, c->stream>>>(lv.p_nnz, lv.p_col.as<int>(),
                                                                   x.cnt.as<int>());
  if ((rc = scan(x, x.cnt.as<int>(), lv.t_ptr, nc, &total))) return rc;
  AG_TRY(cudaMemcpyAsync(x.cnt.p, lv.t_ptr.p, sizeof(int) * (size_t)nc, cudaMemcpyDeviceToDevice,
                         c->stream), "smoothed level");
  k_t_bucket<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(
      n, lv.p_ptr.as<int>(), lv.p_col.as<int>(), x.cnt.as<int>(), lv.t_row.as<int>(),
      lv.t_pos.as<int>());
  k_sort_segments<<<grid_for(nc, c->num_sms), kTPB, 0, c->stream>>>(
      nc, lv.t_ptr.as<int>(), lv.t_row.as<int>(), lv.t_pos.as<int>());
  AG_TRY(cudaGetLastError(), "smoothed level");
  GenAP ga{A.ptr, A.col, lv.p_ptr.as<int>(), lv.p_col.as<int>(), A.val, pv.as<double>()};
  if ((rc = acc_rows<GenAP, true>(x, n, ga, lv.ap_ptr, lv.ap_col, &apv, &lv.ap_nnz))) return rc;
  GenPtAP gc{lv.t_ptr.as<int>(), lv.t_row.as<int>(), lv.t_pos.as<int>(), lv.ap_ptr.as<int>(),
             lv.ap_col.as<int>(), pv.as<double>(), apv.as<double>()};
  x.cap = std::max(x.cap, 128);  // P^T A P rows hold about 45 columns on hex meshes
  lv.A.n = nc;
  if ((rc = acc_rows<GenPtAP, true>(x, nc, gc, lv.A.ptr, lv.A.col, &lv.A.val, &lv.A.nnz)))
    return rc;
  AG_TRY(cudaStreamSynchronize(c->stream), "smoothed level");
  return FCG_OK;
}

int copy_mat(Ctx &x, const DevCsr &a, DevMat &dst) {
  int rc;
  dst.n = a.n;
  dst.nnz = a.nnz;
  if ((rc = ints(x, dst.ptr, (long long)a.n + 1)) || (rc = ints(x, dst.col, a.nnz)) ||
      (rc = dbls(x, dst.val, a.nnz)))
    return rc;
  cudaStream_t st = x.c->stream;
  AG_TRY(cudaMemcpyAsync(dst.ptr.p, a.ptr, sizeof(int) * ((size_t)a.n + 1),
                         cudaMemcpyDeviceToDevice, st), "level copy");
  AG_TRY(cudaMemcpyAsync(dst.col.p, a.col, sizeof(int) * (size_t)a.nnz, cudaMemcpyDeviceToDevice,
                         st), "level copy");
  AG_TRY(cudaMemcpyAsync(dst.val.p, a.val, sizeof(double) * (size_t)a.nnz,
                         cudaMemcpyDeviceToDevice, st), "level copy");
  return FCG_OK;
}

int levels_impl(Ctx &x, const DevCsr &fine, int max_levels, int dense_max, int passes,
                double sa_omega, std::vector<DevBuiltLevel> &levels) {
  fcg_context *c = x.c;
  int rc;
  if ((rc = ints(x, x.ctl, 16))) return rc;
  DevMat work[2];
  struct Rel {
    DevMat *w;
    ~Rel() {
      w[0].release();
      w[1].release();
    }
  } rel{work};
  int wi = 0;
  DevCsr cur = fine;
  while ((int)levels.size() + 1 < max_levels) {
    const int n0 = cur.n;
    if (n0 < 2) break;
    DevBuiltLevel lv;
    if ((rc = ints(x, lv.agg, n0))) {
      lv.release();
      return rc;
    }
    k_iota<<<grid_for(n0, c->num_sms), kTPB, 0, c->stream>>>(lv.agg.as<int>(), n0);
    DevCsr a = cur;
    int nc = n0;
    for (int p = 0; p < passes; ++p) {
      DBuf &agg = x.p_agg, &mptr = x.p_mptr, &mem = x.p_mem;
      int m = 0;
      rc = match(x, a, agg, &m, !levels.empty());
      if (!rc && m == a.n) break;  // no pair formed: this matrix does not coarsen
      x.mark("matching", a.n);
      // the last pass of a smoothed first level needs no Galerkin product: that level's
      // matrix is P^T A P
      const bool last = p == passes - 1 || m <= dense_max;
      const bool need_a = !(levels.empty() && sa_omega > 0.0 && last);
      DevMat &dst = work[wi];
      if (need_a) {
        wi ^= 1;
        if (!rc) rc = members(x, a.n, m, agg.as<int>(), mptr, mem);
        if (!rc) rc = galerkin(x, a, agg.as<int>(), m, mptr.as<int>(), mem.as<int>(), dst);
        x.mark("galerkin", m);
      }
      if (!rc) k_compose<<<grid_for(n0, c->num_sms), kTPB, 0, c->stream>>>(n0, agg.as<int>(),
                                                                          lv.agg.as<int>());
      if (!rc) rc = cudaStreamSynchronize(c->stream) == cudaSuccess ? FCG_OK : FCG_ERR_CUDA;
      if (rc) {
        lv.release();
        return rc;
      }
      if (need_a) a = dst.view();
      nc = m;
      if (nc <= dense_max) break;
    }
    if (nc == n0 || 10LL * nc > 9LL * n0) {  // less than 10% fewer rows: stop
      lv.release();
      break;
    }
    lv.n = nc;
    lv.np = n0;
    rc = members(x, n0, nc, lv.agg.as<int>(), lv.mptr, lv.mem);
    if (!rc) {
      if (levels.empty() && sa_omega > 0.0)
        rc = smoothed(x, cur, sa_omega, lv);
      else
        rc = copy_mat(x, a, lv.A);
    }
    if (!rc) rc = cudaStreamSynchronize(c->stream) == cudaSuccess ? FCG_OK : FCG_ERR_CUDA;
    x.mark(levels.empty() && sa_omega > 0.0 ? "smoothed" : "level", nc);
    if (rc) {
      lv.release();
      return rc;
    }
    levels.push_back(lv);
    cur = levels.back().A.view();
    if (nc <= dense_max) break;
  }
  return FCG_OK;
}

}  // namespace

void DevBuiltLevel::release() {
  for (DBuf *b : {&agg, &mptr, &mem, &p_ptr, &p_col, &t_ptr, &t_row, &t_pos, &ap_ptr, &ap_col})
    b->release();
  A.release();
}

void fine_values(fcg_context *c, const double *sval, const int *src, long long len,
                 const double *s, double *val) {
  k_fine_scatter<<<grid_for(len, c->num_sms), kTPB, 0, c->stream>>>(len, sval, src, val);
  k_fine_scale<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(c->n, c->mv.ioffset,
                                                                   c->mv.ja, s, val);
}

int build_levels_device(fcg_context *c, const DevCsr &fine, int max_levels, int dense_max,
                        int passes, double sa_omega, std::vector<DevBuiltLevel> &levels,
                        std::string &err) {
  Ctx x{c, err};
  const char *tr = std::getenv("FCG_AGG_TRACE");
  x.trace = tr && tr[0] == '1';
  const char *sq = std::getenv("FCG_AGG_SEQ");
  x.seq_on = !(sq && sq[0] == '0');
  levels.clear();
  const int rc = levels_impl(x, fine, max_levels, dense_max, passes, sa_omega, levels);
  x.release();
  if (rc) {
    for (auto &l : levels) l.release();
    levels.clear();
  }
  return rc;
}

}  // namespace ml
}  // namespace fcg

extern "C" int fcg_set_aggregation_wait_test(fcg_context *c, int polls, int absent_row) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound)
    return fcg::set_error(c, FCG_ERR_STATE, "fcg_set_aggregation_wait_test before fcg_bind_mesh");
  if (absent_row < 0 || absent_row > c->n)
    return fcg::set_error(c, FCG_ERR_INDEX, "absent_row out of range");
  c->agg_test_polls = polls > 0 ? polls : 0;
  c->agg_test_row = absent_row - 1;
  return FCG_OK;
}
