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
#include <climits>

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

int scan_exclusive(fcg_context *c, const int *in, int *out, int n, Tmp &tmp) {
  const int nb = (n + kScanChunk - 1) / kScanChunk;
  FCG_CUDA_TRY(c, tmp.b.ensure(sizeof(int) * (nb > 0 ? nb : 1)));
  if (n == 0) {
    FCG_CUDA_TRY(c, cudaMemsetAsync(out, 0, sizeof(int), c->stream));
    return FCG_OK;
  }
  k_scan_local<<<nb, kScanThreads, 0, c->stream>>>(in, out, n, tmp.b.as<int>());
  k_scan_sums<<<1, kScanThreads, 0, c->stream>>>(tmp.b.as<int>(), nb);
  k_scan_add<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(out, in, n, tmp.b.as<int>());
  FCG_CHECK_LAUNCH(c, "scan_exclusive");
  return FCG_OK;
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
__global__ void k_csr_count(int nin, const int *__restrict__ owner,
                            const int *__restrict__ neighbour, int *__restrict__ cnt) {
  FCG_GRID_STRIDE(f, nin) {
    atomicAdd(&cnt[owner[f] - 1], 1);
    atomicAdd(&cnt[neighbour[f] - 1], 1);
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
                                 const int *__restrict__ neighbour, const int *__restrict__ off,
                                 int *__restrict__ cursor, int *__restrict__ ja) {
  FCG_GRID_STRIDE(f, nin) {
    const int o = owner[f] - 1, q = neighbour[f] - 1;
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
                            const int *__restrict__ neighbour, const int *__restrict__ off,
                            const int *__restrict__ ja, int *__restrict__ slot_pn,
                            int *__restrict__ slot_np) {
  FCG_GRID_STRIDE(f, nin) {
    const int o = owner[f] - 1, q = neighbour[f] - 1;
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
    k_csr_count<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, ow, nb, cnt);
  FCG_CHECK_LAUNCH(c, "k_csr_count");
  if ((rc = scan_exclusive(c, cnt, off, n, scan))) return rc;
  int *dj = (int *)dja;
  k_csr_fill_diag<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, off, dj, cursor);
  if (nin > 0)
    k_csr_fill_faces<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, ow, nb, off, cursor,
                                                                         dj);
  k_csr_sort<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(n, off, dj, (int *)ddg, flag);
  if (nin > 0)
    k_csr_slots<<<grid_for(nin, c->num_sms), kTPB, 0, c->stream>>>(nin, ow, nb, off, dj,
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
