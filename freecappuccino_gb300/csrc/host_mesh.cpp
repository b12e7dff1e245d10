// Synthetic hexahedral meshes and their geometry (host side of libfcgpu.so).
//
// The geometry routine restates mesh_geometry (src/mesh_geometry_and_topology.f90:
// 859-1079): the same expressions in the same order, but organised as per-cell
// gathers over the cell's faces in ascending face order, so that it runs on all host
// threads and still sums every cell quantity in the order of the Fortran face loop.
// Compiled with -ffp-contract=off: no fused multiply-add, bit-identical to the loop.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/fcgpu.h"
#include "../../include/fcgpu_meshgen.h"
#include "host_util.h"

namespace {

const uint64_t kJitterStream = 0x6A177E4ULL;  // counter = 3*point + axis

inline long long pid(int N, int i, int j, int k) {
  long long M = N + 1;
  return (long long)i + M * j + M * M * k;
}

}  // namespace

extern "C" int fcg_hex_mesh_sizes(int N, int *numNodes, int *numCells, int *numFaces,
                                  int *numInnerFaces) {
  if (N < 1 || N > 1290) return FCG_ERR_ARG;  // keeps every count below 2^31
  long long M = N + 1, n = (long long)N * N * N;
  long long nin = 3LL * N * N * (N - 1), nb = 6LL * N * N;
  if (numNodes) *numNodes = (int)(M * M * M);
  if (numCells) *numCells = (int)n;
  if (numFaces) *numFaces = (int)(nin + nb);
  if (numInnerFaces) *numInnerFaces = (int)nin;
  return FCG_OK;
}

extern "C" int fcg_uniform_fill(unsigned long long seed, unsigned long long stream,
                                long long count, double lo, double hi, double *out) {
  if (count < 0 || (!out && count > 0)) return FCG_ERR_ARG;
  double w = hi - lo;
  fcg::parallel_for(count, [&](long long i) { out[i] = lo + w * fcg::uniform01(seed, stream, i); });
  return FCG_OK;
}

extern "C" int fcg_hex_mesh_build(int N, double jitter, unsigned long long seed, double *x,
                                  double *y, double *z, int *face_ptr, int *face_nodes,
                                  int *owner, int *neighbour, int *patches) {
  int nn, nc, nf, nin;
  if (fcg_hex_mesh_sizes(N, &nn, &nc, &nf, &nin) != FCG_OK) return FCG_ERR_ARG;
  if (!x || !y || !z || !face_ptr || !face_nodes || !owner || (nin && !neighbour) || !patches)
    return FCG_ERR_ARG;
  const double h = 1.0 / N;
  const long long M = N + 1;
  // Points: (i,j,k)/N; interior points jittered.
  fcg::parallel_for((long long)nn, [&](long long p) {
    int i = (int)(p % M), j = (int)((p / M) % M), k = (int)(p / (M * M));
    double px = i * h, py = j * h, pz = k * h;
    if (i > 0 && i < N && j > 0 && j < N && k > 0 && k < N && jitter != 0.0) {
      px += (2.0 * fcg::uniform01(seed, kJitterStream, 3 * (uint64_t)p + 0) - 1.0) * jitter * h;
      py += (2.0 * fcg::uniform01(seed, kJitterStream, 3 * (uint64_t)p + 1) - 1.0) * jitter * h;
      pz += (2.0 * fcg::uniform01(seed, kJitterStream, 3 * (uint64_t)p + 2) - 1.0) * jitter * h;
    }
    if (i == N) px = 1.0;
    if (j == N) py = 1.0;
    if (k == N) pz = 1.0;
    x[p] = px;
    y[p] = py;
    z[p] = pz;
  });
  for (long long f = 0; f <= nf; ++f) face_ptr[f] = (int)(4 * f);
  auto P = [&](int i, int j, int k) { return (int)(pid(N, i, j, k) + 1); };
  auto put = [&](long long f, int a, int b, int c, int d, int own, int nb) {
    face_nodes[4 * f + 0] = a;
    face_nodes[4 * f + 1] = b;
    face_nodes[4 * f + 2] = c;
    face_nodes[4 * f + 3] = d;
    owner[f] = own;
    if (nb > 0) neighbour[f] = nb;
  };
  // Inner faces in owner order; for one owner the neighbours c+1 < c+N < c+N^2.
  // Cell (i,j,k) owns [i<N-1] + [j<N-1] + [k<N-1] inner faces, so its first face is
  // the count owned by the cells before it: k full planes (each 3N^2-2N faces), then
  // j full rows of plane k (each 2N-1 + N[k<N-1]), then i cells of row j
  // (each 1 + [j<N-1] + [k<N-1], since every i' < i has i' < N-1).
  const long long NN = (long long)N * N;
  fcg::parallel_for((long long)nc, [&](long long c) {
    int i = (int)(c % N), j = (int)((c / N) % N), k = (int)(c / NN);
    long long zk = (k < N - 1) ? 1 : 0, yj = (j < N - 1) ? 1 : 0;
    long long f = (long long)k * (3LL * N * N - 2LL * N) + (long long)j * (2LL * N - 1 + N * zk) +
                  (long long)i * (1 + yj + zk);
    int own = (int)c + 1;
    if (i < N - 1)
      put(f++, P(i + 1, j, k), P(i + 1, j + 1, k), P(i + 1, j + 1, k + 1), P(i + 1, j, k + 1), own,
          own + 1);
    if (j < N - 1)
      put(f++, P(i, j + 1, k), P(i, j + 1, k + 1), P(i + 1, j + 1, k + 1), P(i + 1, j + 1, k), own,
          own + N);
    if (k < N - 1)
      put(f++, P(i, j, k + 1), P(i + 1, j, k + 1), P(i + 1, j + 1, k + 1), P(i, j + 1, k + 1), own,
          own + (int)NN);
  });
  // Boundary faces: symmetry x=1, y=0, y=1, z=0, z=1, then wall x=0.
  long long f = nin;
  auto cell = [&](int i, int j, int k) { return (int)(i + (long long)N * j + NN * k) + 1; };
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      put(f++, P(N, j, k), P(N, j + 1, k), P(N, j + 1, k + 1), P(N, j, k + 1), cell(N - 1, j, k), 0);
  for (int k = 0; k < N; ++k)
    for (int i = 0; i < N; ++i)
      put(f++, P(i, 0, k), P(i + 1, 0, k), P(i + 1, 0, k + 1), P(i, 0, k + 1), cell(i, 0, k), 0);
  for (int k = 0; k < N; ++k)
    for (int i = 0; i < N; ++i)
      put(f++, P(i, N, k), P(i, N, k + 1), P(i + 1, N, k + 1), P(i + 1, N, k), cell(i, N - 1, k), 0);
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i)
      put(f++, P(i, j, 0), P(i, j + 1, 0), P(i + 1, j + 1, 0), P(i + 1, j, 0), cell(i, j, 0), 0);
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i)
      put(f++, P(i, j, N), P(i + 1, j, N), P(i + 1, j + 1, N), P(i, j + 1, N), cell(i, j, N - 1), 0);
  long long wall_start = f;
  for (int k = 0; k < N; ++k)
    for (int j = 0; j < N; ++j)
      put(f++, P(0, j, k), P(0, j, k + 1), P(0, j + 1, k + 1), P(0, j + 1, k), cell(0, j, k), 0);
  if (f != nf) return FCG_ERR_INDEX;
  patches[0] = (int)(5 * NN);
  patches[1] = nin;
  patches[2] = (int)NN;
  patches[3] = (int)wall_start;
  return FCG_OK;
}

// ---------------------------------------------------------------------------
// Geometry (mesh_geometry_and_topology.f90:859-1079)
// ---------------------------------------------------------------------------
namespace {

// centroid_component_part_polymesh (:162-183), evaluated left to right.
inline double cc_part(double a, double b, double c, double nx, double vol) {
  double t = 1.0 / (2.0 * vol);
  t = t * 1.0;
  t = t / 24.0;
  t = t * nx;
  return t * ((a + b) * (a + b) + (b + c) * (b + c) + (c + a) * (c + a));
}

// find_intersection_point (:201-274): determinant ratio, term for term.
inline void intersection(double x1, double y1, double z1, double x2, double y2, double z2,
                         double x3, double y3, double z3, double x4, double y4, double z4,
                         double x5, double y5, double z5, double &xj, double &yj, double &zj) {
  const double tiny = (double)1e-30f;
  double num = x2 * (y3 * z4 - y4 * z3) - x1 * (y3 * z4 - y4 * z3) - x3 * (y2 * z4 - y4 * z2) +
               x1 * (y2 * z4 - y4 * z2) + x3 * (y1 * z4 - y4 * z1) - x2 * (y1 * z4 - y4 * z1) +
               x4 * (y2 * z3 - y3 * z2) - x1 * (y2 * z3 - y3 * z2) - x4 * (y1 * z3 - y3 * z1) +
               x2 * (y1 * z3 - y3 * z1) + x4 * (y1 * z2 - y2 * z1) - x3 * (y1 * z2 - y2 * z1);
  double den = x2 * (y3 * (z5 - z4) - (y5 - y4) * z3) - x1 * (y3 * (z5 - z4) - (y5 - y4) * z3) -
               x3 * (y2 * (z5 - z4) - (y5 - y4) * z2) + x1 * (y2 * (z5 - z4) - (y5 - y4) * z2) +
               x3 * (y1 * (z5 - z4) - (y5 - y4) * z1) - x2 * (y1 * (z5 - z4) - (y5 - y4) * z1) +
               (x5 - x4) * (y2 * z3 - y3 * z2) - (x5 - x4) * (y1 * z3 - y3 * z1) +
               (x5 - x4) * (y1 * z2 - y2 * z1) + tiny;
  double t = -num / den;
  xj = x4 + (x5 - x4) * t;
  yj = y4 + (y5 - y4) * t;
  zj = z4 + (z5 - z4) * t;
}

}  // namespace

extern "C" int fcg_mesh_geometry(int numNodes, const double *x, const double *y, const double *z,
                                 int numCells, int numFaces, int numInnerFaces,
                                 const int *face_ptr, const int *face_nodes, const int *owner,
                                 const int *neighbour, double *arx, double *ary, double *arz,
                                 double *xf, double *yf, double *zf, double *xc, double *yc,
                                 double *zc, double *vol, double *facint) {
  if (numCells <= 0 || numFaces <= 0 || numInnerFaces < 0 || numInnerFaces > numFaces ||
      !x || !y || !z || !face_ptr || !face_nodes || !owner || !arx || !ary || !arz || !xf ||
      !yf || !zf || !xc || !yc || !zc || !vol || (numInnerFaces > 0 && (!neighbour || !facint)))
    return FCG_ERR_ARG;
  // Validate the face list and cell indices before any gather.
  for (int f = 0; f < numFaces; ++f) {
    int nnod = face_ptr[f + 1] - face_ptr[f];
    if (nnod < 3 || owner[f] < 1 || owner[f] > numCells) return FCG_ERR_INDEX;
    if (f < numInnerFaces && (neighbour[f] < 1 || neighbour[f] > numCells)) return FCG_ERR_INDEX;
    for (int q = face_ptr[f]; q < face_ptr[f + 1]; ++q)
      if (face_nodes[q] < 1 || face_nodes[q] > numNodes) return FCG_ERR_INDEX;
  }
  const double half = 0.5, one_third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  // Pass 1a: per-face area vectors and centres (:866-948).
  fcg::parallel_for(numFaces, [&](long long f) {
    const int *nd = face_nodes + face_ptr[f];
    int nnod = face_ptr[f + 1] - face_ptr[f];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int i = 1; i <= nnod - 2; ++i) {
      double px = x[nd[i] - 1] - x[nd[0] - 1], py = y[nd[i] - 1] - y[nd[0] - 1],
             pz = z[nd[i] - 1] - z[nd[0] - 1];
      double qx = x[nd[i + 1] - 1] - x[nd[0] - 1], qy = y[nd[i + 1] - 1] - y[nd[0] - 1],
             qz = z[nd[i + 1] - 1] - z[nd[0] - 1];
      ax = ax + half * (py * qz - pz * qy);
      ay = ay + half * (pz * qx - px * qz);
      az = az + half * (px * qy - py * qx);
    }
    arx[f] = ax;
    ary[f] = ay;
    arz[f] = az;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int q = 0; q < nnod; ++q) {
      sx = sx + x[nd[q] - 1];
      sy = sy + y[nd[q] - 1];
      sz = sz + z[nd[q] - 1];
    }
    xf[f] = sx / (double)nnod;
    yf[f] = sy / (double)nnod;
    zf[f] = sz / (double)nnod;
  });
  // Cell -> faces in ascending face order (owner and neighbour roles).
  std::vector<int> cptr(numCells + 1, 0);
  for (int f = 0; f < numFaces; ++f) {
    cptr[owner[f]]++;
    if (f < numInnerFaces) cptr[neighbour[f]]++;
  }
  for (int c = 0; c < numCells; ++c) cptr[c + 1] += cptr[c];
  std::vector<int> clist(cptr[numCells]);
  {
    std::vector<int> fill(cptr.begin(), cptr.end() - 1);
    for (int f = 0; f < numFaces; ++f) {
      clist[fill[owner[f] - 1]++] = f + 1;  // + owner role
      if (f < numInnerFaces) clist[fill[neighbour[f] - 1]++] = -(f + 1);
    }
  }
  // Pass 1b: volumes (:915-921), per cell in face order, triangles in order.
  fcg::parallel_for(numCells, [&](long long c) {
    double v = 0.0;
    for (int e = cptr[c]; e < cptr[c + 1]; ++e) {
      int f = std::abs(clist[e]) - 1;
      bool own = clist[e] > 0;
      const int *nd = face_nodes + face_ptr[f];
      int nnod = face_ptr[f + 1] - face_ptr[f];
      for (int i = 1; i <= nnod - 2; ++i) {
        double x1 = x[nd[0] - 1], y1 = y[nd[0] - 1], z1 = z[nd[0] - 1];
        double x2 = x[nd[i] - 1], y2 = y[nd[i] - 1], z2 = z[nd[i] - 1];
        double x3 = x[nd[i + 1] - 1], y3 = y[nd[i + 1] - 1], z3 = z[nd[i + 1] - 1];
        double px = x2 - x1, py = y2 - y1, pz = z2 - z1;
        double qx = x3 - x1, qy = y3 - y1, qz = z3 - z1;
        double nx = py * qz - pz * qy, ny = pz * qx - px * qz, nz = px * qy - py * qx;
        double cx = one_third * (x3 + x2 + x1), cy = one_third * (y3 + y2 + y1),
               cz = one_third * (z3 + z2 + z1);
        if (own)
          v = v + sixth * (cx * nx + cy * ny + cz * nz);
        else
          v = v + sixth * (cx * -nx + cy * -ny + cz * -nz);
      }
    }
    vol[c] = v;
  });
  // Pass 2: centroids (:972-1008).
  fcg::parallel_for(numCells, [&](long long c) {
    double sx = 0.0, sy = 0.0, sz = 0.0, vc = vol[c];
    for (int e = cptr[c]; e < cptr[c + 1]; ++e) {
      int f = std::abs(clist[e]) - 1;
      bool own = clist[e] > 0;
      const int *nd = face_nodes + face_ptr[f];
      int nnod = face_ptr[f + 1] - face_ptr[f];
      for (int i = 1; i <= nnod - 2; ++i) {
        double x1 = x[nd[0] - 1], y1 = y[nd[0] - 1], z1 = z[nd[0] - 1];
        double x2 = x[nd[i] - 1], y2 = y[nd[i] - 1], z2 = z[nd[i] - 1];
        double x3 = x[nd[i + 1] - 1], y3 = y[nd[i + 1] - 1], z3 = z[nd[i + 1] - 1];
        double px = x2 - x1, py = y2 - y1, pz = z2 - z1;
        double qx = x3 - x1, qy = y3 - y1, qz = z3 - z1;
        double nx = py * qz - pz * qy, ny = pz * qx - px * qz, nz = px * qy - py * qx;
        if (own) {
          sx = sx + cc_part(x1, x2, x3, nx, vc);
          sy = sy + cc_part(y1, y2, y3, ny, vc);
          sz = sz + cc_part(z1, z2, z3, nz, vc);
        } else {
          sx = sx + cc_part(x1, x3, x2, -nx, vc);
          sy = sy + cc_part(y1, y3, y2, -ny, vc);
          sz = sz + cc_part(z1, z3, z2, -nz, vc);
        }
      }
    }
    xc[c] = sx;
    yc[c] = sy;
    zc[c] = sz;
  });
  // Pass 3: interpolation factors (:1030-1079).
  fcg::parallel_for(numInnerFaces, [&](long long f) {
    const int *nd = face_nodes + face_ptr[f];
    int inp = owner[f] - 1, inn = neighbour[f] - 1;
    double xpn = xc[inn] - xc[inp], ypn = yc[inn] - yc[inp], zpn = zc[inn] - zc[inp];
    double dpn = std::sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    double xj, yj, zj;
    intersection(x[nd[0] - 1], y[nd[0] - 1], z[nd[0] - 1], x[nd[1] - 1], y[nd[1] - 1],
                 z[nd[1] - 1], x[nd[2] - 1], y[nd[2] - 1], z[nd[2] - 1], xc[inp], yc[inp],
                 zc[inp], xc[inn], yc[inn], zc[inn], xj, yj, zj);
    xpn = xj - xc[inp];
    ypn = yj - yc[inp];
    zpn = zj - zc[inp];
    double djn = std::sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    facint[f] = djn / dpn;
  });
  return FCG_OK;
}
