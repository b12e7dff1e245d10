// Mesh setup on the GPU: the geometry pass of mesh_geometry
// (mesh_geometry_and_topology.f90:859-1079) and the CSR construction of
// create_CSR_matrix_from_mesh_data (sparse_matrix.f90:42-172), with the results of the
// host forms (fcg_mesh_geometry, fcg_csr_build) bit for bit.
//
// Integer work (incidence lists, CSR rows) is filled with atomic cursors and then each
// row is sorted by a unique key, so the result does not depend on the order in which
// the atomics land.  The floating-point passes evaluate the host form's expressions in
// the same order; this file is compiled with --fmad=false.  Every input index is checked
// by a validation kernel before any kernel gathers through it.
#include <algorithm>
#include <climits>
#include <string>
#include <vector>

#include "fcg_internal.h"
#include "launch.h"

using namespace fcg;

namespace {

enum SetupFlag { BAD_FACEPTR = 1, BAD_OWNER = 2, BAD_NEIGHBOUR = 4, BAD_NODE = 8, DUP_PAIR = 16 };

// ---------------------------------------------------------------------------
// exclusive scan of int counts: out[0..n] with out[n] the total
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024, kScanItems = 4, kScanChunk = kScanThreads * kScanItems;

// Exclusive scan of one value per thread over the block; *total gets the block sum.
__device__ int block_exclusive(int v, int *sh, int *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) sh[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = sh[lane];  // kScanThreads / 32 == 32 warps
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    sh[lane] = w;
  }
  __syncthreads();
  const int prefix = warp > 0 ? sh[warp - 1] : 0;
  *total = sh[31];
  __syncthreads();  // sh is reused by the caller's next round
  return prefix + incl - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_local(const int *__restrict__ in,
                                                             int *__restrict__ out, int n,
                                                             int *__restrict__ bsum) {
  __shared__ int sh[32];
  const long long base = (long long)blockIdx.x * kScanChunk + (long long)threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  int total;
  int run = block_exclusive(s, sh, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// One block scans the block sums in place (exclusive), carrying across chunks.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int *__restrict__ bsum, int nb) {
  __shared__ int sh[32];
  int carry = 0;
  for (int c0 = 0; c0 < nb; c0 += kScanChunk) {
    const int base = c0 + threadIdx.x * kScanItems;
    int v[kScanItems], s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      v[k] = base + k < nb ? bsum[base + k] : 0;
      s += v[k];
    }
    int total;
    int run = carry + block_exclusive(s, sh, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      if (base + k < nb) bsum[base + k] = run;
      run += v[k];
    }
    carry += total;
  }
}

__global__ void k_scan_add(int *__restrict__ out, const int *__restrict__ in, int n,
                           const int *__restrict__ bsum) {
  FCG_GRID_STRIDE(i, n) {
    out[i] += bsum[i / kScanChunk];
    if (i == n - 1) out[n] = out[i] + in[i];
  }
}

// RAII device scratch for one setup call.
struct Tmp {
  DBuf b;
  ~Tmp() { b.release(); }
};

int scan_into(fcg_context *c, const int *in, int *out, int n, DBuf &tmp) {
  const int nb = (n + kScanChunk - 1) / kScanChunk;
  FCG_CUDA_TRY(c, tmp.ensure(sizeof(int) * (nb > 0 ? nb : 1)));
  if (n == 0) {
    FCG_CUDA_TRY(c, cudaMemsetAsync(out, 0, sizeof(int), c->stream));
    return FCG_OK;
  }
  k_scan_local<<<nb, kScanThreads, 0, c->stream>>>(in, out, n, tmp.as<int>());
  k_scan_sums<<<1, kScanThreads, 0, c->stream>>>(tmp.as<int>(), nb);
  k_scan_add<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(out, in, n, tmp.as<int>());
  FCG_CHECK_LAUNCH(c, "scan_exclusive");
  return FCG_OK;
}

int scan_exclusive(fcg_context *c, const int *in, int *out, int n, Tmp &tmp) {
  return scan_into(c, in, out, n, tmp.b);
}

__global__ void k_fill_int(int *__restrict__ a, long long n, int v) {
  FCG_GRID_STRIDE(i, n) a[i] = v;
}

// Sorts a[lo..hi) ascending by key(a[k]) in place (insertion sort: the rows are short).
template <class Key>
__device__ void sort_row(int *a, int lo, int hi, Key key) {
  for (int k = lo + 1; k < hi; ++k) {
    const int v = a[k];
    const long long kv = key(v);
    int j = k - 1;
    while (j >= lo && key(a[j]) > kv) {
      a[j + 1] = a[j];
      --j;
    }
    a[j + 1] = v;
  }
}

// ---------------------------------------------------------------------------
// CSR (sparse_matrix.f90:42-172)
// ---------------------------------------------------------------------------
__global__ void k_csr_check(int n, int nin, const int *__restrict__ owner,
                            const int *__restrict__ neighbour, int *__restrict__ flag) {
  FCG_GRID_STRIDE(f, nin) {
    const int o = owner[f], q = neighbour[f];
    int bad = 0;
    if (o < 1 || o > n) bad |= BAD_OWNER;
    if (q < 1 || q > n || q == o) bad |= BAD_NEIGHBOUR;
    if (bad) atomicOr(flag, bad);
  }
}

// row counts: 1 (the diagonal) + one per inner face the row's cell is on
// (owner and neighbour indices are `base`-based: 1 for the reference's arrays, 0 for the
// bound copies)
__global__ void k_csr_count(int nin, const int *__restrict__ owner,
                            const int *__restrict__ neighbour, int base, int *__restrict__ cnt) {
  FCG_GRID_STRIDE(f, nin) {
    atomicAdd(&cnt[owner[f] - base], 1);
    atomicAdd(&cnt[neighbour[f] - base], 1);
  }
}

__global__ void k_csr_fill_diag(int n, const int *__restrict__ off, int *__restrict__ ja,
                                int *__restrict__ cursor) {
  FCG_GRID_STRIDE(i, n) {
    ja[off[i]] = (int)i + 1;
    cursor[i] = 1;
  }
}

// (owner, neighbour) and (neighbour, owner) of every inner face (sparse_matrix.f90:60-71)
__global__ void k_csr_fill_faces(int nin, const int *__restrict__ owner,
                                 const int *__restrict__ neighbour, int base,
                                 const int *__restrict__ off, int *__restrict__ cursor,
                                 int *__restrict__ ja) {
  FCG_GRID_STRIDE(f, nin) {
    const int o = owner[f] - base, q = neighbour[f] - base;
    ja[off[o] + atomicAdd(&cursor[o], 1)] = q + 1;
    ja[off[q] + atomicAdd(&cursor[q], 1)] = o + 1;
  }
}

// Sorted rows (the lexical order of the reference's heap sort, :77), a duplicate pair
// check, and diag = position of (i,i) (:87), 1-based.
__global__ void k_csr_sort(int n, const int *__restrict__ off, int *__restrict__ ja,
                           int *__restrict__ diag, int *__restrict__ flag) {
  FCG_GRID_STRIDE(i, n) {
    const int lo = off[i], hi = off[i + 1];
    sort_row(ja, lo, hi, [](int v) { return (long long)v; });
    int d = 0;
    for (int k = lo; k < hi; ++k) {
      if (k > lo && ja[k] == ja[k - 1]) atomicOr(flag, DUP_PAIR);
      if (ja[k] == (int)i + 1) d = k + 1;
    }
    diag[i] = d;
  }
}

__device__ __forceinline__ int find_col(const int *__restrict__ ja, int lo, int hi, int col) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (ja[mid] < col)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// icell_jcell / jcell_icell slot maps (sparse_matrix.f90:153-167), 1-based
__global__ void k_csr_slots(int nin, const int *__restrict__ owner,
                            const int *__restrict__ neighbour, int base,
                            const int *__restrict__ off, const int *__restrict__ ja,
                            int *__restrict__ slot_pn, int *__restrict__ slot_np) {
  FCG_GRID_STRIDE(f, nin) {
    const int o = owner[f] - base, q = neighbour[f] - base;
    slot_pn[f] = find_col(ja, off[o], off[o + 1], q + 1) + 1;
    slot_np[f] = find_col(ja, off[q], off[q + 1], o + 1) + 1;
  }
}

__global__ void k_csr_ioffset(int n1, const int *__restrict__ off, int *__restrict__ ioffset) {
  FCG_GRID_STRIDE(i, n1) ioffset[i] = off[i] + 1;
}

// ---------------------------------------------------------------------------
// geometry (mesh_geometry_and_topology.f90:859-1079)
// ---------------------------------------------------------------------------
struct Nodes {
  const double *x, *y, *z;
};

__global__ void k_geo_check(int nf, int nin, int n, int nnodes, long long total,
                            const int *__restrict__ fp, const int *__restrict__ fn,
                            const int *__restrict__ owner, const int *__restrict__ neighbour,
                            int *__restrict__ flag) {
  FCG_GRID_STRIDE(f, nf) {
    int bad = 0;
    const long long a = fp[f], b = fp[f + 1];
    if (a < 0 || b > total || b - a < 3) {
      bad |= BAD_FACEPTR;
    } else {
      for (long long q = a; q < b; ++q)
        if (fn[q] < 1 || fn[q] > nnodes) bad |= BAD_NODE;
    }
    const int o = owner[f];
    if (o < 1 || o > n) bad |= BAD_OWNER;
    if (f < nin) {
      const int q = neighbour[f];
      if (q < 1 || q > n) bad |= BAD_NEIGHBOUR;
    }
    if (bad) atomicOr(flag, bad);
  }
}

// face area vectors by the triangle fan from node 1 and arithmetic-mean centres (:866-948)
__global__ void k_geo_faces(int nf, Nodes P, const int *__restrict__ fp,
                            const int *__restrict__ fn, double *__restrict__ arx,
                            double *__restrict__ ary, double *__restrict__ arz,
                            double *__restrict__ xf, double *__restrict__ yf,
                            double *__restrict__ zf) {
  const double half = 0.5;
  FCG_GRID_STRIDE(f, nf) {
    const int *nd = fn + fp[f];
    const int nnod = fp[f + 1] - fp[f];
    const int n0 = nd[0] - 1;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int i = 1; i <= nnod - 2; ++i) {
      const int a = nd[i] - 1, b = nd[i + 1] - 1;
      const double px = P.x[a] - P.x[n0], py = P.y[a] - P.y[n0], pz = P.z[a] - P.z[n0];
      const double qx = P.x[b] - P.x[n0], qy = P.y[b] - P.y[n0], qz = P.z[b] - P.z[n0];
      ax = ax + half * (py * qz - pz * qy);
      ay = ay + half * (pz * qx - px * qz);
      az = az + half * (px * qy - py * qx);
    }
    arx[f] = ax;
    ary[f] = ay;
    arz[f] = az;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int q = 0; q < nnod; ++q) {
      sx = sx + P.x[nd[q] - 1];
      sy = sy + P.y[nd[q] - 1];
      sz = sz + P.z[nd[q] - 1];
    }
    xf[f] = sx / (double)nnod;
    yf[f] = sy / (double)nnod;
    zf[f] = sz / (double)nnod;
  }
}

// cell -> face incidence: counts, then entries f+1 (owner) / -(f+1) (neighbour)
__global__ void k_inc_count(int nf, int nin, const int *__restrict__ owner,
                            const int *__restrict__ neighbour, int *__restrict__ cnt) {
  FCG_GRID_STRIDE(f, nf) {
    atomicAdd(&cnt[owner[f] - 1], 1);
    if (f < nin) atomicAdd(&cnt[neighbour[f] - 1], 1);
  }
}

__global__ void k_inc_fill(int nf, int nin, const int *__restrict__ owner,
                           const int *__restrict__ neighbour, const int *__restrict__ ptr,
                           int *__restrict__ cursor, int *__restrict__ list) {
  FCG_GRID_STRIDE(f, nf) {
    const int o = owner[f] - 1;
    list[ptr[o] + atomicAdd(&cursor[o], 1)] = (int)f + 1;
    if (f < nin) {
      const int q = neighbour[f] - 1;
      list[ptr[q] + atomicAdd(&cursor[q], 1)] = -((int)f + 1);
    }
  }
}

// ascending face order, the owner role first where a face is listed twice
__global__ void k_inc_sort(int n, const int *__restrict__ ptr, int *__restrict__ list) {
  FCG_GRID_STRIDE(c, n) {
    sort_row(list, ptr[c], ptr[c + 1], [](int e) {
      return 2LL * (e > 0 ? e : -e) + (e < 0 ? 1 : 0);
    });
  }
}

struct Tri {
  double x1, y1, z1, x2, y2, z2, x3, y3, z3, nx, ny, nz;
};

__device__ __forceinline__ Tri tri(const Nodes &P, int a, int b, int cc) {
  Tri t;
  t.x1 = P.x[a];
  t.y1 = P.y[a];
  t.z1 = P.z[a];
  t.x2 = P.x[b];
  t.y2 = P.y[b];
  t.z2 = P.z[b];
  t.x3 = P.x[cc];
  t.y3 = P.y[cc];
  t.z3 = P.z[cc];
  const double px = t.x2 - t.x1, py = t.y2 - t.y1, pz = t.z2 - t.z1;
  const double qx = t.x3 - t.x1, qy = t.y3 - t.y1, qz = t.z3 - t.z1;
  t.nx = py * qz - pz * qy;
  t.ny = pz * qx - px * qz;
  t.nz = px * qy - py * qx;
  return t;
}

// divergence-theorem volumes (:915-921), per cell in face order, triangles in order
__global__ void k_geo_vol(int n, Nodes P, const int *__restrict__ fp, const int *__restrict__ fn,
                          const int *__restrict__ ptr, const int *__restrict__ list,
                          double *__restrict__ vol) {
  const double one_third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  FCG_GRID_STRIDE(c, n) {
    double v = 0.0;
    for (int e = ptr[c]; e < ptr[c + 1]; ++e) {
      const int ent = list[e];
      const int f = (ent > 0 ? ent : -ent) - 1;
      const int *nd = fn + fp[f];
      const int nnod = fp[f + 1] - fp[f];
      for (int i = 1; i <= nnod - 2; ++i) {
        const Tri t = tri(P, nd[0] - 1, nd[i] - 1, nd[i + 1] - 1);
        const double cx = one_third * (t.x3 + t.x2 + t.x1), cy = one_third * (t.y3 + t.y2 + t.y1),
                     cz = one_third * (t.z3 + t.z2 + t.z1);
        if (ent > 0)
          v = v + sixth * (cx * t.nx + cy * t.ny + cz * t.nz);
        else
          v = v + sixth * (cx * -t.nx + cy * -t.ny + cz * -t.nz);
      }
    }
    vol[c] = v;
  }
}

// centroid_component_part_polymesh (:162-183), evaluated left to right
__device__ __forceinline__ double cc_part(double a, double b, double c, double nx, double vol) {
  double t = 1.0 / (2.0 * vol);
  t = t * 1.0;
  t = t / 24.0;
  t = t * nx;
  return t * ((a + b) * (a + b) + (b + c) * (b + c) + (c + a) * (c + a));
}

// Nurnberg centroids (:972-1008)
__global__ void k_geo_centroid(int n, Nodes P, const int *__restrict__ fp,
                               const int *__restrict__ fn, const int *__restrict__ ptr,
                               const int *__restrict__ list, const double *__restrict__ vol,
                               double *__restrict__ xc, double *__restrict__ yc,
                               double *__restrict__ zc) {
  FCG_GRID_STRIDE(c, n) {
    double sx = 0.0, sy = 0.0, sz = 0.0;
    const double vc = vol[c];
    for (int e = ptr[c]; e < ptr[c + 1]; ++e) {
      const int ent = list[e];
      const int f = (ent > 0 ? ent : -ent) - 1;
      const int *nd = fn + fp[f];
      const int nnod = fp[f + 1] - fp[f];
      for (int i = 1; i <= nnod - 2; ++i) {
        const Tri t = tri(P, nd[0] - 1, nd[i] - 1, nd[i + 1] - 1);
        if (ent > 0) {
          sx = sx + cc_part(t.x1, t.x2, t.x3, t.nx, vc);
          sy = sy + cc_part(t.y1, t.y2, t.y3, t.ny, vc);
          sz = sz + cc_part(t.z1, t.z2, t.z3, t.nz, vc);
        } else {
          sx = sx + cc_part(t.x1, t.x3, t.x2, -t.nx, vc);
          sy = sy + cc_part(t.y1, t.y3, t.y2, -t.ny, vc);
          sz = sz + cc_part(t.z1, t.z3, t.z2, -t.nz, vc);
        }
      }
    }
    xc[c] = sx;
    yc[c] = sy;
    zc[c] = sz;
  }
}

// interpolation factor through the plane of the first three face nodes (:1030-1079),
// find_intersection_point (:201-274) term for term
__global__ void k_geo_facint(int nin, Nodes P, const int *__restrict__ fp,
                             const int *__restrict__ fn, const int *__restrict__ owner,
                             const int *__restrict__ neighbour, const double *__restrict__ xc,
                             const double *__restrict__ yc, const double *__restrict__ zc,
                             double *__restrict__ facint) {
  const double tiny = (double)1e-30f;
  FCG_GRID_STRIDE(f, nin) {
    const int *nd = fn + fp[f];
    const int inp = owner[f] - 1, inn = neighbour[f] - 1;
    double xpn = xc[inn] - xc[inp], ypn = yc[inn] - yc[inp], zpn = zc[inn] - zc[inp];
    const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    const double x1 = P.x[nd[0] - 1], y1 = P.y[nd[0] - 1], z1 = P.z[nd[0] - 1];
    const double x2 = P.x[nd[1] - 1], y2 = P.y[nd[1] - 1], z2 = P.z[nd[1] - 1];
    const double x3 = P.x[nd[2] - 1], y3 = P.y[nd[2] - 1], z3 = P.z[nd[2] - 1];
    const double x4 = xc[inp], y4 = yc[inp], z4 = zc[inp];
    const double x5 = xc[inn], y5 = yc[inn], z5 = zc[inn];
    const double num =
        x2 * (y3 * z4 - y4 * z3) - x1 * (y3 * z4 - y4 * z3) - x3 * (y2 * z4 - y4 * z2) +
        x1 * (y2 * z4 - y4 * z2) + x3 * (y1 * z4 - y4 * z1) - x2 * (y1 * z4 - y4 * z1) +
        x4 * (y2 * z3 - y3 * z2) - x1 * (y2 * z3 - y3 * z2) - x4 * (y1 * z3 - y3 * z1) +
        x2 * (y1 * z3 - y3 * z1) + x4 * (y1 * z2 - y2 * z1) - x3 * (y1 * z2 - y2 * z1);
    const double den =
        x2 * (y3 * (z5 - z4) - (y5 - y4) * z3) - x1 * (y3 * (z5 - z4) - (y5 - y4) * z3) -
        x3 * (y2 * (z5 - z4) - (y5 - y4) * z2) + x1 * (y2 * (z5 - z4) - (y5 - y4) * z2) +
        x3 * (y1 * (z5 - z4) - (y5 - y4) * z1) - x2 * (y1 * (z5 - z4) - (y5 - y4) * z1) +
        (x5 - x4) * (y2 * z3 - y3 * z2) - (x5 - x4) * (y1 * z3 - y3 * z1) +
        (x5 - x4) * (y1 * z2 - y2 * z1) + tiny;
    const double t = -num / den;
    const double xj = x4 + (x5 - x4) * t, yj = y4 + (y5 - y4) * t, zj = z4 + (z5 - z4) * t;
    xpn = xj - x4;
    ypn = yj - y4;
    zpn = zj - z4;
    const double djn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    facint[f] = djn / dpn;
  }
}

const char *flag_text(int flag) {
  if (flag & BAD_FACEPTR) return "face_ptr is not increasing or a face has fewer than 3 nodes";
  if (flag & BAD_NODE) return "a face node index is out of 1..numNodes";
  if (flag & BAD_OWNER) return "an owner index is out of 1..numCells";
  if (flag & BAD_NEIGHBOUR) return "a neighbour index is out of 1..numCells or equals the owner";
  return "two faces connect the same pair of cells";
}

// Reads the validation flag (one word) after the stream's work so far.
int read_flag(fcg_context *c, const int *dflag, int *out) {
  FCG_CUDA_TRY(c, cudaMemcpyAsync(out, dflag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

}  // namespace

int fcg::scan_ints(fcg_context *c, const int *in, int *out, int n, DBuf &tmp) {
  return scan_into(c, in, out, n, tmp);
}

extern "C" int fcg_csr_build_gpu(fcg_context *c, int numCells, int numInnerFaces,
                                 const int *owner, const int *neighbour, int *ioffset, int *ja,
                                 int *diag, int *slot_pn, int *slot_np) {
  if (!c) return FCG_ERR_ARG;
  const int n = numCells, nin = numInnerFaces;
  if (n <= 0 || nin < 0 || (nin > 0 && (!owner || !neighbour)) || !ioffset || !ja || !diag ||
      (nin > 0 && (!slot_pn || !slot_np)))
    return set_error(c, FCG_ERR_ARG, "fcg_csr_build_gpu: bad size or NULL array");
  const long long nnz = (long long)n + 2LL * nin;
  if (nnz > INT_MAX) return set_error(c, FCG_ERR_ARG, "nnz does not fit a 32-bit CSR index");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  int rc;
  void *dow = nullptr, *dnb = nullptr, *dio, *dja, *ddg, *dpn = nullptr, *dnp = nullptr;
  bool h0 = false, h1 = false, hio, hja, hdg, hpn = false, hnp = false;
  const size_t fb = sizeof(int) * (size_t)nin;
  if (nin > 0) {
    if ((rc = stage_in(c, owner, fb, 0, true, &dow, &h0))) return rc;
    if ((rc = stage_in(c, neighbour, fb, 1, true, &dnb, &h1))) return rc;
    if ((rc = stage_in(c, slot_pn, fb, 5, false, &dpn, &hpn))) return rc;
    if ((rc = stage_in(c, slot_np, fb, 6, false, &dnp, &hnp))) return rc;
  }
  if ((rc = stage_in(c, ioffset, sizeof(int) * (size_t)(n + 1), 2, false, &dio, &hio))) return rc;
  if ((rc = stage_in(c, ja, sizeof(int) * (size_t)nnz, 3, false, &dja, &hja))) return rc;
  if ((rc = stage_in(c, diag, sizeof(int) * (size_t)n, 4, false, &ddg, &hdg))) return rc;
  Tmp work, scan;
  // [flag][cnt: n][off: n+1][cursor: n]
  FCG_CUDA_TRY(c, work.b.ensure(sizeof(int) * (4 + 3 * (size_t)n + 1)));
  int *flag = work.b.as<int>(), *cnt = flag + 4, *off = cnt + n, *cursor = off + n + 1;
  FCG_CUDA_TRY(c, cudaMemsetAsync(flag, 0, sizeof(int), c->stream));
  const int *ow = (const int *)dow, *nb = (const int *)dnb;
  int hflag = 0;
  if (nin > 0) {
    k_csr_check<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(n, nin, ow, nb, flag);
    FCG_CHECK_LAUNCH(c, "k_csr_check");
    if ((rc = read_flag(c, flag, &hflag))) return rc;
    if (hflag) return set_error(c, FCG_ERR_INDEX, flag_text(hflag));
  }
  k_fill_int<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(cnt, n, 1);
  if (nin > 0)
    k_csr_count<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, ow, nb, 1, cnt);
  FCG_CHECK_LAUNCH(c, "k_csr_count");
  if ((rc = scan_exclusive(c, cnt, off, n, scan))) return rc;
  int *dj = (int *)dja;
  k_csr_fill_diag<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, off, dj, cursor);
  if (nin > 0)
    k_csr_fill_faces<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, ow, nb, 1, off, cursor,
                                                                         dj);
  k_csr_sort<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, off, dj, (int *)ddg, flag);
  if (nin > 0)
    k_csr_slots<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, ow, nb, 1, off, dj,
                                                                    (int *)dpn, (int *)dnp);
  k_csr_ioffset<<<grid_for(n + 1, c->num_sms), kTPB, 0, c->stream>>>(n + 1, off, (int *)dio);
  FCG_CHECK_LAUNCH(c, "fcg_csr_build_gpu");
  if ((rc = read_flag(c, flag, &hflag))) return rc;
  if (hflag) return set_error(c, FCG_ERR_INDEX, flag_text(hflag));
  if ((rc = stage_out(c, ioffset, dio, sizeof(int) * (size_t)(n + 1), hio)) ||
      (rc = stage_out(c, ja, dja, sizeof(int) * (size_t)nnz, hja)) ||
      (rc = stage_out(c, diag, ddg, sizeof(int) * (size_t)n, hdg)))
    return rc;
  if (nin > 0 && ((rc = stage_out(c, slot_pn, dpn, fb, hpn)) ||
                  (rc = stage_out(c, slot_np, dnp, fb, hnp))))
    return rc;
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_mesh_geometry_gpu(fcg_context *c, int numNodes, const double *x,
                                     const double *y, const double *z, int numCells,
                                     int numFaces, int numInnerFaces, const int *face_ptr,
                                     const int *face_nodes, const int *owner,
                                     const int *neighbour, double *arx, double *ary, double *arz,
                                     double *xf, double *yf, double *zf, double *xc, double *yc,
                                     double *zc, double *vol, double *facint) {
  if (!c) return FCG_ERR_ARG;
  const int n = numCells, nf = numFaces, nin = numInnerFaces;
  if (n <= 0 || nf <= 0 || nin < 0 || nin > nf || numNodes <= 0 || !x || !y || !z || !face_ptr ||
      !face_nodes || !owner || !arx || !ary || !arz || !xf || !yf || !zf || !xc || !yc || !zc ||
      !vol || (nin > 0 && (!neighbour || !facint)))
    return set_error(c, FCG_ERR_ARG, "fcg_mesh_geometry_gpu: bad size or NULL array");
  if ((long long)nf + nin > INT_MAX)
    return set_error(c, FCG_ERR_ARG, "the cell-face incidence does not fit 32-bit offsets");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  int rc;
  void *dfp;
  bool hfp;
  if ((rc = stage_in(c, face_ptr, sizeof(int) * ((size_t)nf + 1), 0, true, &dfp, &hfp))) return rc;
  // the length of face_nodes is face_ptr[nf]; face_ptr[0] must be 0
  int ends[2];
  if (hfp) {
    ends[0] = face_ptr[0];
    ends[1] = face_ptr[nf];
  } else {
    FCG_CUDA_TRY(c, cudaMemcpyAsync(&ends[0], face_ptr, sizeof(int), cudaMemcpyDeviceToHost,
                                    c->stream));
    FCG_CUDA_TRY(c, cudaMemcpyAsync(&ends[1], face_ptr + nf, sizeof(int),
                                    cudaMemcpyDeviceToHost, c->stream));
    FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  if (ends[0] != 0 || ends[1] < 3 * nf)
    return set_error(c, FCG_ERR_INDEX, "face_ptr must start at 0 and hold at least 3 nodes a face");
  const long long total = ends[1];
  const size_t nb = sizeof(double) * (size_t)numNodes, fb8 = sizeof(double) * (size_t)nf,
               cb8 = sizeof(double) * (size_t)n;
  void *dx, *dy, *dz, *dfn, *dow, *dnb = nullptr;
  bool hx, hy, hz, hfn, how, hnb = false;
  if ((rc = stage_in(c, x, nb, 1, true, &dx, &hx)) || (rc = stage_in(c, y, nb, 2, true, &dy, &hy)) ||
      (rc = stage_in(c, z, nb, 3, true, &dz, &hz)) ||
      (rc = stage_in(c, face_nodes, sizeof(int) * (size_t)total, 4, true, &dfn, &hfn)) ||
      (rc = stage_in(c, owner, sizeof(int) * (size_t)nf, 5, true, &dow, &how)))
    return rc;
  if (nin > 0 && (rc = stage_in(c, neighbour, sizeof(int) * (size_t)nin, 6, true, &dnb, &hnb)))
    return rc;
  double *outs[11] = {arx, ary, arz, xf, yf, zf, xc, yc, zc, vol, facint};
  const size_t ob[11] = {fb8, fb8, fb8, fb8, fb8, fb8, cb8, cb8, cb8, cb8,
                         sizeof(double) * (size_t)(nin > 0 ? nin : 1)};
  void *dout[11] = {};
  bool hout[11] = {};
  for (int k = 0; k < 11; ++k) {
    if (k == 10 && nin == 0) continue;
    if ((rc = stage_in(c, outs[k], ob[k], 7 + k, false, &dout[k], &hout[k]))) return rc;
  }
  Tmp work, scan;
  // [flag][cnt: n][ptr: n+1][cursor: n][list: nf+nin]
  FCG_CUDA_TRY(c, work.b.ensure(sizeof(int) * (4 + 3 * (size_t)n + 1 + (size_t)nf + nin)));
  int *flag = work.b.as<int>(), *cnt = flag + 4, *ptr = cnt + n, *cursor = ptr + n + 1,
      *list = cursor + n;
  FCG_CUDA_TRY(c, cudaMemsetAsync(flag, 0, sizeof(int), c->stream));
  const int *fp = (const int *)dfp, *fn = (const int *)dfn, *ow = (const int *)dow,
            *nbr = (const int *)dnb;
  k_geo_check<<<grid_for(nf, c->num_sms), kTPB, 0, c->stream>>>(nf, nin, n, numNodes, total, fp,
                                                                  fn, ow, nbr, flag);
  FCG_CHECK_LAUNCH(c, "k_geo_check");
  int hflag = 0;
  if ((rc = read_flag(c, flag, &hflag))) return rc;
  if (hflag) return set_error(c, FCG_ERR_INDEX, flag_text(hflag));
  const Nodes P{(const double *)dx, (const double *)dy, (const double *)dz};
  double *d[11];
  for (int k = 0; k < 11; ++k) d[k] = (double *)dout[k];
  k_geo_faces<<<grid_for(nf, c->num_sms), kTPB, 0, c->stream>>>(nf, P, fp, fn, d[0], d[1], d[2],
                                                                  d[3], d[4], d[5]);
  FCG_CUDA_TRY(c, cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)n, c->stream));
  FCG_CUDA_TRY(c, cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)n, c->stream));
  k_inc_count<<<grid_for(nf, c->num_sms), kTPB, 0, c->stream>>>(nf, nin, ow, nbr, cnt);
  FCG_CHECK_LAUNCH(c, "k_inc_count");
  if ((rc = scan_exclusive(c, cnt, ptr, n, scan))) return rc;
  k_inc_fill<<<grid_for(nf, c->num_sms), kTPB, 0, c->stream>>>(nf, nin, ow, nbr, ptr, cursor,
                                                                 list);
  k_inc_sort<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, ptr, list);
  k_geo_vol<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, P, fp, fn, ptr, list, d[9]);
  k_geo_centroid<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, P, fp, fn, ptr, list, d[9],
                                                                    d[6], d[7], d[8]);
  if (nin > 0)
    k_geo_facint<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, P, fp, fn, ow, nbr, d[6],
                                                                      d[7], d[8], d[10]);
  FCG_CHECK_LAUNCH(c, "fcg_mesh_geometry_gpu");
  for (int k = 0; k < 11; ++k) {
    if (k == 10 && nin == 0) continue;
    if ((rc = stage_out(c, outs[k], dout[k], ob[k], hout[k]))) return rc;
  }
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

// ---------------------------------------------------------------------------
// The topology of fcg_bind_mesh on the device, 0-based, element for element the host
// construction (topology.cpp): the CSR and slot maps (the kernels above), transpose
// positions, inner-face incidence lists, the sliced ELL copy and the level values of the
// sweeps.  The boundary lists (a pass over the boundary faces), the prefix sums over
// slices and the grouping of rows by level run on the host.
// ---------------------------------------------------------------------------
namespace {

__global__ void k_minus1(long long n, int *__restrict__ a) {
  FCG_GRID_STRIDE(i, n) a[i] -= 1;
}

// 0-based position of column col in row `row`, -1 when absent (rows sorted)
__device__ __forceinline__ int find0(const int *__restrict__ io, const int *__restrict__ ja,
                                     int row, int col) {
  int lo = io[row], hi = io[row + 1];
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (ja[mid] < col)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < io[row + 1] && ja[lo] == col) ? lo : -1;
}

__global__ void k_tpos0(int n, const int *__restrict__ io, const int *__restrict__ ja,
                        int *__restrict__ tpos) {
  FCG_GRID_STRIDE(i, n) {
    for (int k = io[i]; k < io[i + 1]; ++k) tpos[k] = find0(io, ja, ja[k], (int)i);
  }
}

__global__ void k_cf_ptr0(int n, const int *__restrict__ io, int *__restrict__ cf_ptr) {
  FCG_GRID_STRIDE(i, n + 1) cf_ptr[i] = io[i] - (int)i;
}

__global__ void k_face_at0(int nin, const int *__restrict__ spn, const int *__restrict__ snp,
                           int *__restrict__ face_at) {
  FCG_GRID_STRIDE(f, nin) {
    face_at[spn[f]] = (int)f;
    face_at[snp[f]] = (int)f;
  }
}

// inner faces of cell i in ascending face order: ent = f+1 (owner) / -(f+1), slot = the
// CSR position of the entry in row i (the inverse of the slot maps, sorted by face)
__global__ void k_cf_lists0(int n, const int *__restrict__ io, const int *__restrict__ dg,
                            const int *__restrict__ owner0, const int *__restrict__ face_at,
                            int *__restrict__ ent, int *__restrict__ slot) {
  FCG_GRID_STRIDE(i, n) {
    const int p0 = io[i] - (int)i;
    int e = p0;
    for (int k = io[i]; k < io[i + 1]; ++k) {
      if (k == dg[i]) continue;
      const int f = face_at[k];
      int j = e++;
      while (j > p0 && abs(ent[j - 1]) > f + 1) {
        ent[j] = ent[j - 1];
        slot[j] = slot[j - 1];
        --j;
      }
      ent[j] = owner0[f] == (int)i ? f + 1 : -(f + 1);
      slot[j] = k;
    }
  }
}

__global__ void k_maxrow(int n, const int *__restrict__ io, int *out) {
  int m = 0;
  FCG_GRID_STRIDE(i, n) m = max(m, io[i + 1] - io[i]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// One warp per slice of 32 rows: the longest row, and the sorted distinct column offsets
// (column - row) as long as a uniform slice stays cheaper than an explicit one
// (2*|u| < 3*wexp); kind 0 with the offsets in u, or kind 1.
__global__ void k_sell_shape0(int n, int ns, const int *__restrict__ io, const int *__restrict__ ja,
                              int ucap, int *__restrict__ width, int *__restrict__ kind,
                              int *__restrict__ u) {
  const int lane = threadIdx.x & 31;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long sl = warp0; sl < ns; sl += nwarps) {
    const long long r = 32 * sl + lane;
    const int b = r < n ? io[r] : 0, e = r < n ? io[r + 1] : 0;
    int wexp = e - b;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wexp = max(wexp, __shfl_xor_sync(0xffffffffu, wexp, o));
    int k = b, cnt = 0;
    bool uniform = wexp > 0;
    while (true) {
      const int mine = k < e ? ja[k] - (int)r : INT_MAX;
      const int m = __reduce_min_sync(0xffffffffu, mine);
      if (m == INT_MAX) break;
      if (2 * (cnt + 1) >= 3 * wexp) {  // one more distinct offset makes uniform dearer
        uniform = false;
        break;
      }
      if (lane == 0) u[sl * (long long)ucap + cnt] = m;
      ++cnt;
      if (mine == m) ++k;
    }
    if (lane == 0) {
      kind[sl] = uniform ? 0 : 1;
      width[sl] = uniform ? cnt : wexp;
    }
  }
}

// Offset table (uniform) or column block (explicit) of every slice and src = CSR
// position of each value slot (-1: none).
__global__ void k_sell_fill0(int n, int ns, const int *__restrict__ io, const int *__restrict__ ja,
                             int ucap, const int *__restrict__ u, const int *__restrict__ width,
                             const int *__restrict__ kind, const long long *__restrict__ ptr,
                             const int *__restrict__ offp, int *__restrict__ off,
                             int *__restrict__ src) {
  const int lane = threadIdx.x & 31;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long sl = warp0; sl < ns; sl += nwarps) {
    const long long r = 32 * sl + lane;
    const int b = r < n ? io[r] : 0, e = r < n ? io[r + 1] : 0;
    const int w = width[sl];
    if (kind[sl] == 0) {
      const int *us = u + sl * (long long)ucap;
      for (int j = lane; j < w; j += 32) off[offp[sl] + j] = us[j];
      for (int j = 0; j < w; ++j) {
        int sidx = -1;
        const int want = (int)r + us[j];
        for (int k = b; k < e; ++k)
          if (ja[k] == want) sidx = k;
        src[ptr[sl] + (long long)j * 32 + lane] = sidx;
      }
    } else {
      for (int j = 0; j < w; ++j) {
        const long long pos = ptr[sl] + (long long)j * 32 + lane;
        const long long cpos = offp[sl] + (long long)j * 32 + lane;
        if (j < e - b) {
          off[cpos] = ja[b + j];
          src[pos] = b + j;
        } else {
          off[cpos] = (int)(r < n - 1 ? r : n - 1);
          src[pos] = -1;
        }
      }
    }
  }
}

// Level of every row in one launch, rows taken in sweep order: lane 0 of a warp claims
// 32 consecutive rows through a counter and does them in order; level = 1 + the largest
// level of the rows it reads, 0 without any.  lev holds -1 until a row's level is
// written; a row only reads rows earlier in the sweep order -- earlier in its own chunk
// (done by this thread) or in a chunk claimed earlier by a running warp -- so every wait
// ends; each is bounded, and one that gives up sets err.
__global__ void k_levels0(int n, const int *__restrict__ io, const int *__restrict__ ja,
                          const int *__restrict__ dg, int upper, int *lev, int *ctr, int *err,
                          int spin) {
  if ((threadIdx.x & 31) != 0) return;
  for (;;) {
    const int t0 = atomicAdd(ctr, 32);
    if (t0 >= n) break;
    const int t1 = min(n, t0 + 32);
    for (int t = t0; t < t1; ++t) {
      const int i = upper ? n - 1 - t : t;
      const int k0 = upper ? dg[i] + 1 : io[i];
      const int k1 = upper ? io[i + 1] : dg[i];
      int l = 0;
      for (int k = k0; k < k1; ++k) {
        const int j = ja[k];
        int v;
        int it = 0;
        while (true) {
          asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(lev + j) : "memory");
          if (v >= 0) break;
          if (++it > spin || *(volatile int *)err) {
            atomicExch(err, 1);
            v = 0;
            break;
          }
          if (it > 16) __nanosleep(64);
        }
        l = max(l, v + 1);
      }
      asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(lev + i), "r"(l) : "memory");
    }
  }
}

// A device array owned by the bound mesh.
template <class T>
T *bound_alloc(fcg_context *c, size_t count) {
  c->bound_allocs.emplace_back();
  DBuf &b = c->bound_allocs.back();
  if (b.ensure(count * sizeof(T)) != cudaSuccess) return nullptr;
  return (T *)b.p;
}

template <class T>
int bound_upload(fcg_context *c, const std::vector<T> &h, const T **out) {
  T *d = bound_alloc<T>(c, h.size());
  if (!d) return set_error(c, FCG_ERR_NOMEM, "device allocation for the mesh topology failed");
  if (!h.empty())
    FCG_CUDA_TRY(c, cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice,
                                    c->stream));
  *out = d;
  return FCG_OK;
}

// rows grouped by level, ascending inside a level (a counting sort)
void group_levels(const std::vector<int> &lev, std::vector<int> &ptr, std::vector<int> &rows) {
  int nlev = 0;
  for (int l : lev) nlev = std::max(nlev, l + 1);
  ptr.assign(nlev + 1, 0);
  for (int l : lev) ptr[l + 1]++;
  for (int l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
  rows.assign(lev.size(), 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (size_t i = 0; i < lev.size(); ++i) rows[fill[lev[i]]++] = (int)i;
}

std::vector<int> padded_levels(const std::vector<int> &ptr, const std::vector<int> &rows) {
  std::vector<int> out;
  out.reserve(rows.size() + 32 * ptr.size());
  for (size_t l = 0; l + 1 < ptr.size(); ++l) {
    out.insert(out.end(), rows.begin() + ptr[l], rows.begin() + ptr[l + 1]);
    while (out.size() % 32) out.push_back(-1);
  }
  return out;
}

}  // namespace

namespace fcg {

int to_zero_based(fcg_context *c, int *a, long long n) {
  if (n <= 0) return FCG_OK;
  k_minus1<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, a);
  FCG_CHECK_LAUNCH(c, "to_zero_based");
  return FCG_OK;
}

int bind_topology_device(fcg_context *c, const int *own0, const int *nei0,
                         const std::vector<int> &own_host, const int cnt[B_NTYPES],
                         const int fst[B_NTYPES], const int bst[B_NTYPES], std::string &err) {
  const int n = c->n, nf = c->nf, nin = c->nin;
  const long long nnz = (long long)n + 2LL * nin;
  MeshView &v = c->mv;
  SellView &sv = c->sv;
  int rc;
  // --- CSR, 0-based, owned by the mesh -----------------------------------------------
  int *io = bound_alloc<int>(c, (size_t)n + 1), *ja = bound_alloc<int>(c, (size_t)nnz),
      *dg = bound_alloc<int>(c, n), *spn = bound_alloc<int>(c, std::max(nin, 1)),
      *snp = bound_alloc<int>(c, std::max(nin, 1));
  if (!io || !ja || !dg || !spn || !snp)
    return set_error(c, FCG_ERR_NOMEM, "device allocation for the mesh topology failed");
  Tmp work, scan;
  FCG_CUDA_TRY(c, work.b.ensure(sizeof(int) * (4 + 2 * (size_t)n)));
  int *flag = work.b.as<int>(), *cntr = flag + 4, *cursor = cntr + n;
  FCG_CUDA_TRY(c, cudaMemsetAsync(flag, 0, sizeof(int), c->stream));
  const int G = grid_for(n, c->num_sms);
  k_fill_int<<<G, kTPB, 0, c->stream>>>(cntr, n, 1);
  if (nin > 0)
    k_csr_count<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, own0, nei0, 0, cntr);
  if ((rc = scan_exclusive(c, cntr, io, n, scan))) return rc;
  k_csr_fill_diag<<<G, kTPB, 0, c->stream>>>(n, io, ja, cursor);
  if (nin > 0)
    k_csr_fill_faces<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, own0, nei0, 0, io,
                                                                         cursor, ja);
  k_csr_sort<<<G, kTPB, 0, c->stream>>>(n, io, ja, dg, flag);
  if (nin > 0)
    k_csr_slots<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, own0, nei0, 0, io, ja,
                                                                    spn, snp);
  k_minus1<<<grid_for(nnz, c->num_sms), kTPB, 0, c->stream>>>(nnz, ja);
  k_minus1<<<G, kTPB, 0, c->stream>>>(n, dg);
  if (nin > 0) {
    k_minus1<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, spn);
    k_minus1<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, snp);
  }
  FCG_CHECK_LAUNCH(c, "device CSR");
  int hflag = 0;
  if ((rc = read_flag(c, flag, &hflag))) return rc;
  if (hflag) {
    err = flag_text(hflag);
    return FCG_ERR_INDEX;
  }
  c->nnz = nnz;
  v.ioffset = io;
  v.ja = ja;
  v.diag = dg;
  v.slot_pn = spn;
  v.slot_np = snp;

  // --- transpose positions and incidence lists ---------------------------------------
  const long long ncf = nnz - n;
  int *tpos = bound_alloc<int>(c, (size_t)nnz), *cfp = bound_alloc<int>(c, (size_t)n + 1),
      *cfe = bound_alloc<int>(c, std::max<long long>(ncf, 1)),
      *cfs = bound_alloc<int>(c, std::max<long long>(ncf, 1));
  if (!tpos || !cfp || !cfe || !cfs)
    return set_error(c, FCG_ERR_NOMEM, "device allocation for the mesh topology failed");
  {
    Tmp fa;
    FCG_CUDA_TRY(c, fa.b.ensure(sizeof(int) * (size_t)nnz));
    k_tpos0<<<G, kTPB, 0, c->stream>>>(n, io, ja, tpos);
    k_cf_ptr0<<<grid_for(n + 1, c->num_sms), kTPB, 0, c->stream>>>(n, io, cfp);
    if (nin > 0)
      k_face_at0<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, spn, snp,
                                                                    fa.b.as<int>());
    k_cf_lists0<<<G, kTPB, 0, c->stream>>>(n, io, dg, own0, fa.b.as<int>(), cfe, cfs);
    FCG_CHECK_LAUNCH(c, "incidence lists");
    FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  c->tpos = tpos;
  v.cf_ptr = cfp;
  v.cf_ent = cfe;
  v.cf_slot = cfs;

  // --- boundary lists (host) ------------------------------------------------------------
  {
    std::vector<int> cb_ptr(n + 1, 0);
    for (int ty = 0; ty < B_NTYPES; ++ty)
      for (int i = 0; i < cnt[ty]; ++i) cb_ptr[own_host[fst[ty] + i]]++;
    for (int i = 0; i < n; ++i) cb_ptr[i + 1] += cb_ptr[i];
    std::vector<int> cb_face(cb_ptr[n]), cb_slot(cb_ptr[n]), cb_type(cb_ptr[n]);
    std::vector<int> fill(cb_ptr.begin(), cb_ptr.end() - 1);
    for (int ty = 0; ty < B_NTYPES; ++ty)
      for (int i = 0; i < cnt[ty]; ++i) {
        const int face = fst[ty] + i, e = fill[own_host[face] - 1]++;
        cb_face[e] = face;
        cb_slot[e] = bst[ty] + i;
        cb_type[e] = ty;
      }
    std::vector<int> cbf_ptr(n + 1, 0);
    for (int f = nin; f < nf; ++f) cbf_ptr[own_host[f]]++;
    for (int i = 0; i < n; ++i) cbf_ptr[i + 1] += cbf_ptr[i];
    std::vector<int> cbf_face(cbf_ptr[n]);
    std::vector<int> fill2(cbf_ptr.begin(), cbf_ptr.end() - 1);
    for (int f = nin; f < nf; ++f) cbf_face[fill2[own_host[f] - 1]++] = f;
    if ((rc = bound_upload(c, cb_ptr, &v.cb_ptr)) || (rc = bound_upload(c, cb_face, &v.cb_face)) ||
        (rc = bound_upload(c, cb_slot, &v.cb_slot)) || (rc = bound_upload(c, cb_type, &v.cb_type)) ||
        (rc = bound_upload(c, cbf_ptr, &v.cbf_ptr)) || (rc = bound_upload(c, cbf_face, &v.cbf_face)))
      return rc;
    c->topo.clear();
    auto rec = [&](const void *p, size_t bytes) { c->topo.emplace_back(p, bytes); };
    rec(io, sizeof(int) * (n + 1));
    rec(ja, sizeof(int) * nnz);
    rec(dg, sizeof(int) * n);
    rec(spn, sizeof(int) * nin);
    rec(snp, sizeof(int) * nin);
    rec(tpos, sizeof(int) * nnz);
    rec(cfp, sizeof(int) * (n + 1));
    rec(cfe, sizeof(int) * ncf);
    rec(cfs, sizeof(int) * ncf);
    rec(v.cb_ptr, sizeof(int) * cb_ptr.size());
    rec(v.cb_face, sizeof(int) * cb_face.size());
    rec(v.cb_slot, sizeof(int) * cb_slot.size());
    rec(v.cb_type, sizeof(int) * cb_type.size());
    rec(v.cbf_ptr, sizeof(int) * cbf_ptr.size());
    rec(v.cbf_face, sizeof(int) * cbf_face.size());
  }

  // --- sliced ELL ---------------------------------------------------------------------
  const int ns = (n + 31) / 32;
  int maxrow = 0;
  {
    Tmp mr;
    FCG_CUDA_TRY(c, mr.b.ensure(sizeof(int)));
    FCG_CUDA_TRY(c, cudaMemsetAsync(mr.b.p, 0, sizeof(int), c->stream));
    k_maxrow<<<G, kTPB, 0, c->stream>>>(n, io, mr.b.as<int>());
    FCG_CUDA_TRY(c, cudaMemcpyAsync(&maxrow, mr.b.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  const int ucap = std::max(1, (3 * maxrow + 1) / 2);
  Tmp shape;
  FCG_CUDA_TRY(c, shape.b.ensure(sizeof(int) * (2 * (size_t)ns + (size_t)ns * ucap)));
  int *dw = shape.b.as<int>(), *dk = dw + ns, *du = dk + ns;
  k_sell_shape0<<<grid_for(32LL * ns, c->num_sms), kTPB, 0, c->stream>>>(n, ns, io, ja, ucap, dw, dk,
                                                                         du);
  FCG_CHECK_LAUNCH(c, "k_sell_shape0");
  std::vector<int> width(ns), kind(ns);
  FCG_CUDA_TRY(c, cudaMemcpyAsync(width.data(), dw, sizeof(int) * ns, cudaMemcpyDeviceToHost, c->stream));
  FCG_CUDA_TRY(c, cudaMemcpyAsync(kind.data(), dk, sizeof(int) * ns, cudaMemcpyDeviceToHost, c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  std::vector<long long> ptr(ns + 1, 0), colp(ns + 1, 0);
  std::vector<int> offp(ns + 1, 0);
  int maxw = 0;
  long long nuni = 0;
  for (int sl = 0; sl < ns; ++sl) {
    const int w = width[sl];
    maxw = std::max(maxw, w);
    ptr[sl + 1] = ptr[sl] + 32LL * w;
    offp[sl + 1] = offp[sl] + (kind[sl] == 0 ? w : 0);
    colp[sl + 1] = colp[sl] + (kind[sl] == 1 ? 32LL * w : 0);
    nuni += kind[sl] == 0;
  }
  const long long noff = (long long)offp[ns] + colp[ns];
  if (noff > INT_MAX) {
    err = "the sliced ELL column blocks do not fit 32-bit offsets";
    return FCG_ERR_ARG;
  }
  for (int sl = 0; sl < ns; ++sl)
    if (kind[sl] == 1) offp[sl] = (int)(offp[ns] + colp[sl]);
  const long long len = ptr[ns];
  if ((rc = bound_upload(c, ptr, &sv.ptr)) || (rc = bound_upload(c, width, &sv.width)) ||
      (rc = bound_upload(c, kind, &sv.kind)) || (rc = bound_upload(c, offp, &sv.offp)))
    return rc;
  int *off = bound_alloc<int>(c, std::max<long long>(noff, 1)),
      *src = bound_alloc<int>(c, std::max<long long>(len, 1));
  if (!off || !src) return set_error(c, FCG_ERR_NOMEM, "device allocation for the sliced ELL failed");
  k_sell_fill0<<<grid_for(32LL * ns, c->num_sms), kTPB, 0, c->stream>>>(
      n, ns, io, ja, ucap, du, sv.width, sv.kind, sv.ptr, sv.offp, off, src);
  FCG_CHECK_LAUNCH(c, "k_sell_fill0");
  sv.nslices = ns;
  sv.off = off;
  sv.src = src;
  c->sell_maxw = maxw;
  c->sell_len = len;
  c->sell_nuniform = nuni;
  auto rec = [&](const void *p, size_t bytes) { c->topo.emplace_back(p, bytes); };
  rec(sv.ptr, sizeof(long long) * (ns + 1));
  rec(sv.width, sizeof(int) * ns);
  rec(sv.kind, sizeof(int) * ns);
  rec(sv.offp, sizeof(int) * (ns + 1));
  rec(off, sizeof(int) * noff);
  rec(src, sizeof(int) * len);

  // --- level schedules ------------------------------------------------------------------
  {
    Tmp lw;
    FCG_CUDA_TRY(c, lw.b.ensure(sizeof(int) * ((size_t)n + 4)));
    int *lev = lw.b.as<int>(), *ctl = lev + n;
    std::vector<int> hlev(n);
    Level *lvs[2] = {&c->lf, &c->lb};
    std::vector<int> rows[2], pads[2];
    for (int upper = 0; upper < 2; ++upper) {
      k_fill_int<<<G, kTPB, 0, c->stream>>>(lev, n, -1);
      FCG_CUDA_TRY(c, cudaMemsetAsync(ctl, 0, 4 * sizeof(int), c->stream));
      k_levels0<<<std::min(G, c->num_sms * 8), kTPB, 0, c->stream>>>(n, io, ja, dg, upper, lev, ctl,
                                                                      ctl + 1, 1 << 22);
      FCG_CHECK_LAUNCH(c, "k_levels0");
      int herr = 0;
      FCG_CUDA_TRY(c, cudaMemcpyAsync(hlev.data(), lev, sizeof(int) * n, cudaMemcpyDeviceToHost,
                                      c->stream));
      FCG_CUDA_TRY(c, cudaMemcpyAsync(&herr, ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      if (herr) {
        err = "a level wait gave up";
        return FCG_ERR_TIMEOUT;
      }
      Level &L = *lvs[upper];
      group_levels(hlev, L.ptr, rows[upper]);
      L.count = (int)L.ptr.size() - 1;
      pads[upper] = padded_levels(L.ptr, rows[upper]);
      const int *d;
      if ((rc = bound_upload(c, rows[upper], &d))) return rc;
      L.rows = const_cast<int *>(d);
      if ((rc = bound_upload(c, pads[upper], &d))) return rc;
      L.pad = const_cast<int *>(d);
      L.pad_len = (int)pads[upper].size();
    }
    rec(c->lf.rows, sizeof(int) * n);
    rec(c->lb.rows, sizeof(int) * n);
    rec(c->lf.pad, sizeof(int) * c->lf.pad_len);
    rec(c->lb.pad, sizeof(int) * c->lb.pad_len);
    FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  return FCG_OK;
}

}  // namespace fcg
