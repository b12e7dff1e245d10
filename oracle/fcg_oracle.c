/*
 * fcg_oracle.c -- CPU restatement of freeCappuccino's pressure-correction path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for libfcgpu.so, never part of the
 * product.  See fcg_oracle.h for the conventions.  Build with
 *   gcc -O2 -ffp-contract=off -fPIC -shared
 * (no fused multiply-add, no reassociation) so that every expression below is
 * evaluated in the order the Fortran source writes it.
 *
 * All citations are paths inside the freeCappuccino source tree.
 */
#include "fcg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Default-REAL (single precision) literals promoted to real(dp). */
double orc_const_small_src(void) { return (double)1e-20f; }  /* modules_allocatable.f90:27 */
double orc_const_small_test(void) { return (double)1e-30f; } /* tests/test_sparse_solvers.f90:36 */
double orc_const_tol(void) { return (double)1e-13f; }        /* dpcg.f90:37, iccg.f90:191 */
static double s0_init(void) { return (double)1.e20f; }        /* dpcg.f90:76 */
static double geo_tiny(void) { return (double)1e-30f; }       /* mesh_geometry_and_topology.f90:57 */

/* Fortran 1-based accessors. */
#define F(arr, i) ((arr)[(i)-1])
#define G3(arr, c, i) ((arr)[3 * ((i)-1) + ((c)-1)]) /* dPhidxi(c,i), component fastest */

/* ------------------------------------------------------------------------- */
/* Geometry: mesh_geometry_and_topology.f90:859-1079                          */
/* ------------------------------------------------------------------------- */

/* find_intersection_point, mesh_geometry_and_topology.f90:201-274: the same
 * determinant-ratio expression, term for term, evaluated left to right. */
static void intersection_point(double x1, double y1, double z1, double x2, double y2, double z2,
                               double x3, double y3, double z3, double x4, double y4, double z4,
                               double x5, double y5, double z5, double *xj, double *yj,
                               double *zj) {
  double num = x2 * (y3 * z4 - y4 * z3) - x1 * (y3 * z4 - y4 * z3) - x3 * (y2 * z4 - y4 * z2) +
               x1 * (y2 * z4 - y4 * z2) + x3 * (y1 * z4 - y4 * z1) - x2 * (y1 * z4 - y4 * z1) +
               x4 * (y2 * z3 - y3 * z2) - x1 * (y2 * z3 - y3 * z2) - x4 * (y1 * z3 - y3 * z1) +
               x2 * (y1 * z3 - y3 * z1) + x4 * (y1 * z2 - y2 * z1) - x3 * (y1 * z2 - y2 * z1);
  double den = x2 * (y3 * (z5 - z4) - (y5 - y4) * z3) - x1 * (y3 * (z5 - z4) - (y5 - y4) * z3) -
               x3 * (y2 * (z5 - z4) - (y5 - y4) * z2) + x1 * (y2 * (z5 - z4) - (y5 - y4) * z2) +
               x3 * (y1 * (z5 - z4) - (y5 - y4) * z1) - x2 * (y1 * (z5 - z4) - (y5 - y4) * z1) +
               (x5 - x4) * (y2 * z3 - y3 * z2) - (x5 - x4) * (y1 * z3 - y3 * z1) +
               (x5 - x4) * (y1 * z2 - y2 * z1) + geo_tiny();
  double t = -num / den;
  *xj = x4 + (x5 - x4) * t;
  *yj = y4 + (y5 - y4) * t;
  *zj = z4 + (z5 - z4) * t;
}

/* centroid_component_part_polymesh, :162-183:
 *   1./(2*vol) * 1./24._dp*nx * ((a+b)**2 + (b+c)**2 + (c+a)**2), left to right. */
static double cc_part(double a, double b, double c, double nx, double vol) {
  double t = 1.0 / (2.0 * vol);
  t = t * 1.0;
  t = t / 24.0;
  t = t * nx;
  return t * ((a + b) * (a + b) + (b + c) * (b + c) + (c + a) * (c + a));
}

int orc_geometry(int numNodes, const double *x, const double *y, const double *z, int numCells,
                 int numFaces, int numInnerFaces, const int *face_ptr, const int *face_nodes,
                 const int *owner, const int *neighbour, double *arx, double *ary, double *arz,
                 double *xf, double *yf, double *zf, double *xc, double *yc, double *zc,
                 double *vol, double *facint) {
  const double half = 0.5;
  const double one_third = 1.0 / 3.0; /* 1./3._dp */
  const double sixth = 1.0 / 6.0;     /* 1./6._dp, cell_volume_part_polymesh :155 */
  (void)numNodes;
  memset(arx, 0, sizeof(double) * numFaces);
  memset(ary, 0, sizeof(double) * numFaces);
  memset(arz, 0, sizeof(double) * numFaces);
  memset(vol, 0, sizeof(double) * numCells);
  memset(xc, 0, sizeof(double) * numCells);
  memset(yc, 0, sizeof(double) * numCells);
  memset(zc, 0, sizeof(double) * numCells);

  /* Pass 1 (:866-950): face area vectors, cell volumes, face centres. */
  for (int iface = 1; iface <= numFaces; ++iface) {
    const int *node = face_nodes + face_ptr[iface - 1]; /* node[0] is node(1) */
    int nnodes = face_ptr[iface] - face_ptr[iface - 1];
    int inp = F(owner, iface);
#define NX(k) F(x, node[(k)-1])
#define NY(k) F(y, node[(k)-1])
#define NZ(k) F(z, node[(k)-1])
    for (int i = 1; i <= nnodes - 2; ++i) {
      double px = NX(i + 1) - NX(1), py = NY(i + 1) - NY(1), pz = NZ(i + 1) - NZ(1);
      double qx = NX(i + 2) - NX(1), qy = NY(i + 2) - NY(1), qz = NZ(i + 2) - NZ(1);
      double nx = py * qz - pz * qy; /* triangular_face_area_components_polymesh :128-130 */
      double ny = pz * qx - px * qz;
      double nz = px * qy - py * qx;
      F(arx, iface) = F(arx, iface) + half * nx;
      F(ary, iface) = F(ary, iface) + half * ny;
      F(arz, iface) = F(arz, iface) + half * nz;
      double cx = one_third * (NX(i + 2) + NX(i + 1) + NX(1));
      double cy = one_third * (NY(i + 2) + NY(i + 1) + NY(1));
      double cz = one_third * (NZ(i + 2) + NZ(i + 1) + NZ(1));
      F(vol, inp) = F(vol, inp) + sixth * (cx * nx + cy * ny + cz * nz);
      if (iface <= numInnerFaces) {
        int inn = F(neighbour, iface);
        F(vol, inn) = F(vol, inn) + sixth * (cx * -nx + cy * -ny + cz * -nz);
      }
    }
    /* Arithmetic-mean face centre (:936-948). */
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int k = 1; k <= nnodes; ++k) {
      sx = sx + NX(k);
      sy = sy + NY(k);
      sz = sz + NZ(k);
    }
    F(xf, iface) = sx / (double)nnodes;
    F(yf, iface) = sy / (double)nnodes;
    F(zf, iface) = sz / (double)nnodes;
  }

  /* Pass 2 (:972-1008): cell centroids. */
  for (int iface = 1; iface <= numFaces; ++iface) {
    const int *node = face_nodes + face_ptr[iface - 1];
    int nnodes = face_ptr[iface] - face_ptr[iface - 1];
    int inp = F(owner, iface);
    for (int i = 1; i <= nnodes - 2; ++i) {
      double px = NX(i + 1) - NX(1), py = NY(i + 1) - NY(1), pz = NZ(i + 1) - NZ(1);
      double qx = NX(i + 2) - NX(1), qy = NY(i + 2) - NY(1), qz = NZ(i + 2) - NZ(1);
      double nx = py * qz - pz * qy;
      double ny = pz * qx - px * qz;
      double nz = px * qy - py * qx;
      F(xc, inp) = F(xc, inp) + cc_part(NX(1), NX(i + 1), NX(i + 2), nx, F(vol, inp));
      F(yc, inp) = F(yc, inp) + cc_part(NY(1), NY(i + 1), NY(i + 2), ny, F(vol, inp));
      F(zc, inp) = F(zc, inp) + cc_part(NZ(1), NZ(i + 1), NZ(i + 2), nz, F(vol, inp));
      if (iface <= numInnerFaces) {
        int inn = F(neighbour, iface);
        F(xc, inn) = F(xc, inn) + cc_part(NX(1), NX(i + 2), NX(i + 1), -nx, F(vol, inn));
        F(yc, inn) = F(yc, inn) + cc_part(NY(1), NY(i + 2), NY(i + 1), -ny, F(vol, inn));
        F(zc, inn) = F(zc, inn) + cc_part(NZ(1), NZ(i + 2), NZ(i + 1), -nz, F(vol, inn));
      }
    }
  }

  /* Pass 3 (:1030-1079): interpolation factor through the plane of nodes 1..3. */
  for (int iface = 1; iface <= numInnerFaces; ++iface) {
    const int *node = face_nodes + face_ptr[iface - 1];
    int inp = F(owner, iface), inn = F(neighbour, iface);
    double xpn = F(xc, inn) - F(xc, inp);
    double ypn = F(yc, inn) - F(yc, inp);
    double zpn = F(zc, inn) - F(zc, inp);
    double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    double xjp, yjp, zjp;
    intersection_point(NX(1), NY(1), NZ(1), NX(2), NY(2), NZ(2), NX(3), NY(3), NZ(3),
                       F(xc, inp), F(yc, inp), F(zc, inp), F(xc, inn), F(yc, inn), F(zc, inn),
                       &xjp, &yjp, &zjp);
    xpn = xjp - F(xc, inp);
    ypn = yjp - F(yc, inp);
    zpn = zjp - F(zc, inp);
    double djn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    F(facint, iface) = djn / dpn;
  }
#undef NX
#undef NY
#undef NZ
  return 0;
}

/* ------------------------------------------------------------------------- */
/* a1: CSR pattern, sparse_matrix.f90:42-172                                  */
/* ------------------------------------------------------------------------- */

typedef struct {
  int i, j;
} ij_pair;

static int ij_compare(const void *pa, const void *pb) {
  const ij_pair *a = (const ij_pair *)pa, *b = (const ij_pair *)pb;
  if (a->i != b->i) return a->i < b->i ? -1 : 1;
  if (a->j != b->j) return a->j < b->j ? -1 : 1;
  return 0;
}

/* csr_to_k, utils.f90:76-128: linear scan of row icell for column jcell (0 if absent). */
static int csr_to_k(int icell, int jcell, const int *ioffset, const int *ja) {
  for (int l = F(ioffset, icell); l <= F(ioffset, icell + 1) - 1; ++l)
    if (F(ja, l) == jcell) return l;
  return 0;
}

int orc_create_csr(int numCells, int numInnerFaces, const int *owner, const int *neighbour,
                   int *ioffset, int *ja, int *diag, int *slot_pn, int *slot_np) {
  long nnz = (long)numCells + 2L * numInnerFaces;
  ij_pair *coo = (ij_pair *)malloc(sizeof(ij_pair) * (size_t)(nnz > 0 ? nnz : 1));
  if (!coo) return -1;
  /* COO fill (:61-72). */
  for (int icell = 1; icell <= numCells; ++icell) coo[icell - 1] = (ij_pair){icell, icell};
  for (int i = 1; i <= numInnerFaces; ++i)
    coo[numCells + i - 1] = (ij_pair){F(owner, i), F(neighbour, i)};
  for (int i = 1; i <= numInnerFaces; ++i)
    coo[numCells + numInnerFaces + i - 1] = (ij_pair){F(neighbour, i), F(owner, i)};
  /* Lexical sort (:77, i4vec2_sort_a). Pairs are unique, so any correct sort gives
   * the same order as the reference's heap sort. */
  qsort(coo, (size_t)nnz, sizeof(ij_pair), ij_compare);
  for (long k = 0; k < nnz; ++k) ja[k] = coo[k].j;
  /* Diagonal positions (:87, find_main_diag_element_positions utils.f90:130-148). */
  int id = 1;
  for (long indx = 1; indx <= nnz; ++indx)
    if (coo[indx - 1].i == coo[indx - 1].j) F(diag, id++) = (int)indx;
  /* Row starts (:97-104, find_index_position utils.f90:151-170). */
  long istart = 1, iend = 1;
  for (int icell = 1; icell <= numCells; ++icell) {
    for (long i = istart; i <= iend; ++i)
      if (coo[i - 1].i == icell) {
        F(ioffset, icell) = (int)i;
        break;
      }
    istart = F(ioffset, icell) + 1;
    iend = nnz;
  }
  F(ioffset, numCells + 1) = (int)(nnz + 1);
  free(coo);
  /* Face -> slot maps (:159-168). */
  for (int i = 1; i <= numInnerFaces; ++i) {
    int ijp = F(owner, i), ijn = F(neighbour, i);
    F(slot_pn, i) = csr_to_k(ijp, ijn, ioffset, ja);
    F(slot_np, i) = csr_to_k(ijn, ijp, ioffset, ja);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Boundary slot offsets, mesh_geometry_and_topology.f90:593-605              */
/* ------------------------------------------------------------------------- */
static int iInletStart(const orc_mesh *m) { return m->numCells; }
static int iOutletStart(const orc_mesh *m) { return m->numCells + m->ninl; }
static int iSymmetryStart(const orc_mesh *m) { return m->numCells + m->ninl + m->nout; }
static int iWallStart(const orc_mesh *m) { return m->numCells + m->ninl + m->nout + m->nsym; }
static int iPressOutletStart(const orc_mesh *m) {
  return m->numCells + m->ninl + m->nout + m->nsym + m->nwal;
}

/* ------------------------------------------------------------------------- */
/* a2: fvm_laplacian.f90                                                      */
/* ------------------------------------------------------------------------- */

/* The pairs' cells and interpolation factors in freshly allocated arrays (free_oc). */
typedef struct { int *ijl, *ijr; double *foc, *srdoc; } oc_pairs;
int orc_oc_geometry(const orc_mesh *m, int *ijl, int *ijr, double *foc, double *srdoc);
static int get_oc(const orc_mesh *m, oc_pairs *o) {
  size_t k = (size_t)(m->noc > 0 ? m->noc : 1);
  o->ijl = malloc(sizeof(int) * k), o->ijr = malloc(sizeof(int) * k);
  o->foc = malloc(sizeof(double) * k), o->srdoc = malloc(sizeof(double) * k);
  if (!o->ijl || !o->ijr || !o->foc || !o->srdoc) return -1;
  if (m->noc > 0) orc_oc_geometry(m, o->ijl, o->ijr, o->foc, o->srdoc);
  return 0;
}
static void free_oc(oc_pairs *o) { free(o->ijl), free(o->ijr), free(o->foc), free(o->srdoc); }

int orc_oc_geometry(const orc_mesh *m, int *ijl, int *ijr, double *foc, double *srdoc) {
  int nreg = m->noc - m->ncyc;
  for (int i = 1; i <= m->noc; ++i) {
    int iface = F(m->ijlFace, i), ifaceFriend = F(m->ijrFace, i); /* :820-824 */
    int inp = F(m->owner, iface), inn = F(m->owner, ifaceFriend);
    F(ijl, i) = inp;
    F(ijr, i) = inn;
    double xpn = F(m->xc, inn) - F(m->xf, ifaceFriend); /* :1094-1100 */
    double ypn = F(m->yc, inn) - F(m->yf, ifaceFriend);
    double zpn = F(m->zc, inn) - F(m->zf, ifaceFriend);
    double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    xpn = F(m->xf, iface) - F(m->xc, inp); /* :1103-1107 */
    ypn = F(m->yf, iface) - F(m->yc, inp);
    zpn = F(m->zf, iface) - F(m->zc, inp);
    double djn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    F(foc, i) = i <= nreg ? djn / (djn + dpn) : 0.5; /* :1109, cyclic :1149 */
    double are = sqrt(F(m->arx, iface) * F(m->arx, iface) + F(m->ary, iface) * F(m->ary, iface) +
                      F(m->arz, iface) * F(m->arz, iface));
    F(srdoc, i) = are / (djn + dpn); /* :1115 */
  }
  return 0;
}

int orc_laplacian(const orc_mesh *m, const int *ioffset, const int *diag, const int *slot_pn,
                  const int *slot_np, const double *mu, const double *phi, double *a,
                  double *su) {
  long nnz = (long)F(ioffset, m->numCells + 1) - 1;
  for (long k = 0; k < nnz; ++k) a[k] = 0.0; /* :33 */
  for (int i = 1; i <= m->numInnerFaces; ++i) { /* :38-65 */
    int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    double arx = F(m->arx, i), ary = F(m->ary, i), arz = F(m->arz, i);
    /* facefluxlaplacian :171-221 */
    double fxn = F(m->facint, i);
    double fxp = 1.0 - fxn;
    double xpn = F(m->xc, ijn) - F(m->xc, ijp);
    double ypn = F(m->yc, ijn) - F(m->yc, ijp);
    double zpn = F(m->zc, ijn) - F(m->zc, ijp);
    double smdpn = (arx * arx + ary * ary + arz * arz) / (arx * xpn + ary * ypn + arz * zpn);
    double cap = (fxp * F(mu, ijp) + fxn * F(mu, ijn)) * smdpn;
    double can = cap;
    F(a, F(slot_pn, i)) = can;
    F(a, F(slot_np, i)) = cap;
    F(a, F(diag, ijp)) = F(a, F(diag, ijp)) - can;
    F(a, F(diag, ijn)) = F(a, F(diag, ijn)) - cap;
  }
  if (m->noc > 0) { /* o- and c-grid cuts (:67-86) */
    int noc = m->noc;
    int *ijl = malloc(sizeof(int) * (size_t)noc), *ijr = malloc(sizeof(int) * (size_t)noc);
    double *foc = malloc(sizeof(double) * (size_t)noc);
    double *srdoc = malloc(sizeof(double) * (size_t)noc);
    if (!ijl || !ijr || !foc || !srdoc) return -1;
    orc_oc_geometry(m, ijl, ijr, foc, srdoc);
    double *ar = a + nnz, *al = a + nnz + noc;
    for (int i = 1; i <= noc; ++i) {
      int iface = m->iOCFacesStart + i;
      int ijp = F(ijl, i), ijn = F(ijr, i);
      double arx = F(m->arx, iface), ary = F(m->ary, iface), arz = F(m->arz, iface);
      /* facefluxlaplacian(ijp, ijn, arx(iface), .., foc(i), mu, al(i), ar(i)) */
      double fxn = F(foc, i);
      double fxp = 1.0 - fxn;
      double xpn = F(m->xc, ijn) - F(m->xc, ijp);
      double ypn = F(m->yc, ijn) - F(m->yc, ijp);
      double zpn = F(m->zc, ijn) - F(m->zc, ijp);
      double smdpn = (arx * arx + ary * ary + arz * arz) / (arx * xpn + ary * ypn + arz * zpn);
      double cap = (fxp * F(mu, ijp) + fxn * F(mu, ijn)) * smdpn;
      F(al, i) = cap;
      F(ar, i) = cap;
      F(a, F(diag, ijp)) = F(a, F(diag, ijp)) - F(ar, i);
      F(a, F(diag, ijn)) = F(a, F(diag, ijn)) - F(al, i);
    }
    free(ijl), free(ijr), free(foc), free(srdoc);
  }
  /* Wall faces (:140-154); inlet/outlet/symmetry add nothing (their loops are commented out). */
  for (int i = 1; i <= m->nwal; ++i) {
    int iface = m->iWallFacesStart + i;
    int ijp = F(m->owner, iface);
    int ijb = iWallStart(m) + i;
    int k = F(diag, ijp);
    double are = sqrt(F(m->arx, iface) * F(m->arx, iface) + F(m->ary, iface) * F(m->ary, iface) +
                      F(m->arz, iface) * F(m->arz, iface));
    double dx = F(m->xc, ijp) - F(m->xf, iface);
    double dy = F(m->yc, ijp) - F(m->yf, iface);
    double dz = F(m->zc, ijp) - F(m->zf, iface);
    double dpw = sqrt(dx * dx + dy * dy + dz * dz);
    F(a, k) = F(a, k) - F(mu, ijp) * are / dpw;
    F(su, ijp) = F(su, ijp) + F(a, k) * F(phi, ijb);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* a3: facefluxmass.f90:34-199 inside calcp-multiple_correction_SIMPLE.f90:34-77 */
/* ------------------------------------------------------------------------- */

/* face_value_central, interpolation.f90:145-199 */
static double face_value_central(const orc_mesh *m, int inp, int inn, double xf, double yf,
                                 double zf, const double *fi, const double *gradfi) {
  double gradfidr = G3(gradfi, 1, inp) * (xf - F(m->xc, inp)) +
                    G3(gradfi, 2, inp) * (yf - F(m->yc, inp)) +
                    G3(gradfi, 3, inp) * (zf - F(m->zc, inp)) +
                    G3(gradfi, 1, inn) * (xf - F(m->xc, inn)) +
                    G3(gradfi, 2, inn) * (yf - F(m->yc, inn)) +
                    G3(gradfi, 3, inn) * (zf - F(m->zc, inn));
  return 0.5 * (F(fi, inp) + F(fi, inn) + gradfidr);
}

/* facefluxmass.f90:34-199 on the face between ijp and ijn with centre (xf, yf, zf), area
 * (arx, ary, arz) and interpolation factor lambda: cap, can and the face mass flux. */
static void ffm_face(const orc_mesh *m, int ijp, int ijn, double xf, double yf, double zf,
                     double arx, double ary, double arz, double lambda, const double *u,
                     const double *v, const double *w, const double *p, const double *dUdxi,
                     const double *dVdxi, const double *dWdxi, const double *dPdxi,
                     const double *apu, const double *apv, const double *apw,
                     const double *den, double *cap_out, double *can_out, double *fm_out) {
  double fxn = lambda;
  double fxp = 1.0 - fxn;
  double xpn = F(m->xc, ijn) - F(m->xc, ijp);
  double ypn = F(m->yc, ijn) - F(m->yc, ijp);
  double zpn = F(m->zc, ijn) - F(m->zc, ijp);
  double are = sqrt(arx * arx + ary * ary + arz * arz);
  double nxx = arx / are, nyy = ary / are, nzz = arz / are;
  double Dpu = fxn * F(m->vol, ijn) * F(apu, ijn) + fxp * F(m->vol, ijp) * F(apu, ijp);
  double Dpv = fxn * F(m->vol, ijn) * F(apv, ijn) + fxp * F(m->vol, ijp) * F(apv, ijp);
  double Dpw = fxn * F(m->vol, ijn) * F(apw, ijn) + fxp * F(m->vol, ijp) * F(apw, ijp);
  double dene = F(den, ijp) * fxp + F(den, ijn) * fxn;
  double sfdpnr = 1.0 / (arx * xpn * nxx + ary * ypn * nyy + arz * zpn * nzz);
  double smdpn = (arx * arx + ary * ary + arz * arz) * sfdpnr;
  double cap = -(dene * Dpu * smdpn);
  double can = cap;
  double ui = face_value_central(m, ijp, ijn, xf, yf, zf, u, dUdxi);
  double vi = face_value_central(m, ijp, ijn, xf, yf, zf, v, dVdxi);
  double wi = face_value_central(m, ijp, ijn, xf, yf, zf, w, dWdxi);
  double dpxi = Dpu * (fxn * G3(dPdxi, 1, ijn) + fxp * G3(dPdxi, 1, ijp)) * xpn * nxx;
  double dpyi = Dpv * (fxn * G3(dPdxi, 2, ijn) + fxp * G3(dPdxi, 2, ijp)) * ypn * nyy;
  double dpzi = Dpw * (fxn * G3(dPdxi, 3, ijn) + fxp * G3(dPdxi, 3, ijp)) * zpn * nzz;
  double xpp = xf - (xf - F(m->xc, ijp)) * nxx;
  double ypp = yf - (yf - F(m->yc, ijp)) * nyy;
  double zpp = zf - (zf - F(m->zc, ijp)) * nzz;
  double xep = xf - (xf - F(m->xc, ijn)) * nxx;
  double yep = yf - (yf - F(m->yc, ijn)) * nyy;
  double zep = zf - (zf - F(m->zc, ijn)) * nzz;
  xpp = xpp - F(m->xc, ijp);
  ypp = ypp - F(m->yc, ijp);
  zpp = zpp - F(m->zc, ijp);
  xep = xep - F(m->xc, ijn);
  yep = yep - F(m->yc, ijn);
  zep = zep - F(m->zc, ijn);
  double dpe = F(p, ijn) - F(p, ijp);
  /* :174-175, including the reference's sign pattern (only the first P term is subtracted). */
  double dpecorr = G3(dPdxi, 1, ijn) * xep + G3(dPdxi, 2, ijn) * yep + G3(dPdxi, 3, ijn) * zep -
                   G3(dPdxi, 1, ijp) * xpp + G3(dPdxi, 2, ijp) * ypp + G3(dPdxi, 3, ijp) * zpp;
  dpe = dpe + dpecorr;
  double dpex = Dpu * dpe * sfdpnr * arx;
  double dpey = Dpv * dpe * sfdpnr * ary;
  double dpez = Dpw * dpe * sfdpnr * arz;
  double ue = ui - dpex + dpxi;
  double ve = vi - dpey + dpyi;
  double we = wi - dpez + dpzi;
  *cap_out = cap;
  *can_out = can;
  *fm_out = dene * (ue * arx + ve * ary + we * arz);
}

/* calcp :34-100.  With O-C pairs a holds ar, al after the nnz CSR values and flmass the
 * pairs' fluxes fmoc after the numInnerFaces inner-face fluxes. */
int orc_facefluxmass(const orc_mesh *m, const int *diag, const int *slot_pn, const int *slot_np,
                     const double *u, const double *v, const double *w, const double *p,
                     const double *dUdxi, const double *dVdxi, const double *dWdxi,
                     const double *dPdxi, const double *apu, const double *apv,
                     const double *apw, const double *den, int nnz, double *a, double *su,
                     double *flmass) {
  for (int k = 0; k < nnz; ++k) a[k] = 0.0;              /* calcp :34 */
  for (int i = 0; i < m->numCells; ++i) su[i] = 0.0;     /* calcp :35 */
  for (int i = 1; i <= m->numInnerFaces; ++i) {
    int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    double cap, can, fm;
    ffm_face(m, ijp, ijn, F(m->xf, i), F(m->yf, i), F(m->zf, i), F(m->arx, i), F(m->ary, i),
             F(m->arz, i), F(m->facint, i), u, v, w, p, dUdxi, dVdxi, dWdxi, dPdxi, apu, apv,
             apw, den, &cap, &can, &fm);
    F(flmass, i) = fm;
    F(a, F(slot_pn, i)) = can;
    F(a, F(slot_np, i)) = cap;
    F(a, F(diag, ijp)) = F(a, F(diag, ijp)) - can;
    F(a, F(diag, ijn)) = F(a, F(diag, ijn)) - cap;
    F(su, ijp) = F(su, ijp) - fm;
    F(su, ijn) = F(su, ijn) + fm;
  }
  if (m->noc > 0) { /* o- and c-grid cuts (:81-100) */
    oc_pairs oc;
    if (get_oc(m, &oc)) return -1;
    double *ar = a + nnz, *al = a + nnz + m->noc, *fmoc = flmass + m->numInnerFaces;
    for (int i = 1; i <= m->noc; ++i) {
      int iface = F(m->ijlFace, i), ijp = F(oc.ijl, i), ijn = F(oc.ijr, i);
      ffm_face(m, ijp, ijn, F(m->xf, iface), F(m->yf, iface), F(m->zf, iface),
               F(m->arx, iface), F(m->ary, iface), F(m->arz, iface), F(oc.foc, i), u, v, w, p,
               dUdxi, dVdxi, dWdxi, dPdxi, apu, apv, apw, den, &F(al, i), &F(ar, i),
               &F(fmoc, i));
      F(a, F(diag, ijp)) = F(a, F(diag, ijp)) - F(ar, i);
      F(a, F(diag, ijn)) = F(a, F(diag, ijn)) - F(al, i);
      F(su, ijp) = F(su, ijp) - F(fmoc, i);
      F(su, ijn) = F(su, ijn) + F(fmoc, i);
    }
    free_oc(&oc);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* a4: fluxmc, facefluxmass.f90:520-607, driven by calcp :193-206             */
/* ------------------------------------------------------------------------- */

/* fluxmc, facefluxmass.f90:520-607, on the face between ijp and ijn (centre, area, factor). */
static double fmc_face(const orc_mesh *m, int ijp, int ijn, double xf, double yf, double zf,
                       double arx, double ary, double arz, double lambda, const double *dPdxi,
                       const double *apu, const double *den) {
  double fxn = lambda;
  double fxp = 1.0 - fxn;
  double xpn = F(m->xc, ijn) - F(m->xc, ijp);
  double ypn = F(m->yc, ijn) - F(m->yc, ijp);
  double zpn = F(m->zc, ijn) - F(m->zc, ijp);
  double are = sqrt(arx * arx + ary * ary + arz * arz);
  double nxx = arx / are, nyy = ary / are, nzz = arz / are;
  double dppnnr = 1.0 / ((xpn * nxx) + (ypn * nyy) + (zpn * nzz));
  double xpp = xf - (xf - F(m->xc, ijp)) * nxx;
  double ypp = yf - (yf - F(m->yc, ijp)) * nyy;
  double zpp = zf - (zf - F(m->zc, ijp)) * nzz;
  double xep = xf - (xf - F(m->xc, ijn)) * nxx;
  double yep = yf - (yf - F(m->yc, ijn)) * nyy;
  double zep = zf - (zf - F(m->zc, ijn)) * nzz;
  xpp = xpp - F(m->xc, ijp);
  ypp = ypp - F(m->yc, ijp);
  zpp = zpp - F(m->zc, ijp);
  xep = xep - F(m->xc, ijn);
  yep = yep - F(m->yc, ijn);
  zep = zep - F(m->zc, ijn);
  double rapr = F(apu, ijp) * F(den, ijp) * F(m->vol, ijp) * fxp +
                F(apu, ijn) * F(den, ijn) * F(m->vol, ijn) * fxn;
  return rapr * are *
         ((G3(dPdxi, 1, ijn) * xep - G3(dPdxi, 1, ijp) * xpp) +
          (G3(dPdxi, 2, ijn) * yep - G3(dPdxi, 2, ijp) * ypp) +
          (G3(dPdxi, 3, ijn) * zep - G3(dPdxi, 3, ijp) * zpp)) *
         dppnnr;
}

/* calcp :193-215; with O-C pairs flmass holds fmoc after the inner-face fluxes. */
int orc_fluxmc(const orc_mesh *m, const double *dPdxi, const double *apu, const double *den,
               double *su, double *flmass) {
  for (int i = 0; i < m->numCells; ++i) su[i] = 0.0; /* calcp :193 */
  for (int i = 1; i <= m->numInnerFaces; ++i) {
    int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    double fmcor = fmc_face(m, ijp, ijn, F(m->xf, i), F(m->yf, i), F(m->zf, i), F(m->arx, i),
                            F(m->ary, i), F(m->arz, i), F(m->facint, i), dPdxi, apu, den);
    F(flmass, i) = F(flmass, i) + fmcor;
    F(su, ijp) = F(su, ijp) - fmcor;
    F(su, ijn) = F(su, ijn) + fmcor;
  }
  if (m->noc > 0) { /* faces along O-C grid cuts (:206-215) */
    oc_pairs oc;
    if (get_oc(m, &oc)) return -1;
    double *fmoc = flmass + m->numInnerFaces;
    for (int i = 1; i <= m->noc; ++i) {
      int iface = F(m->ijlFace, i), ijp = F(oc.ijl, i), ijn = F(oc.ijr, i);
      double fmcor = fmc_face(m, ijp, ijn, F(m->xf, iface), F(m->yf, iface), F(m->zf, iface),
                              F(m->arx, iface), F(m->ary, iface), F(m->arz, iface),
                              F(oc.foc, i), dPdxi, apu, den);
      F(fmoc, i) = F(fmoc, i) + fmcor;
      F(su, ijp) = F(su, ijp) - fmcor;
      F(su, ijn) = F(su, ijn) + fmcor;
    }
    free_oc(&oc);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* a5/a6: grad_gauss.f90, grad_gauss_corrected.f90                           */
/* ------------------------------------------------------------------------- */

/* One pass of grad_gauss.f90:46-113 with old gradient (dfxo,dfyo,dfzo). */
static void gauss_pass(const orc_mesh *m, const double *fi, const double *dfxo,
                       const double *dfyo, const double *dfzo, double *dfx, double *dfy,
                       double *dfz) {
  int n = m->numCells;
  for (int i = 0; i < n; ++i) dfx[i] = dfy[i] = dfz[i] = 0.0;
  for (int i = 1; i <= m->numInnerFaces; ++i) { /* gradco :128-190 */
    int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    double fxn = F(m->facint, i);
    double fxp = 1.0 - fxn;
    double xi = F(m->xc, ijp) * fxp + F(m->xc, ijn) * fxn;
    double yi = F(m->yc, ijp) * fxp + F(m->yc, ijn) * fxn;
    double zi = F(m->zc, ijp) * fxp + F(m->zc, ijn) * fxn;
    double dfxi = F(dfxo, ijp) * fxp + F(dfxo, ijn) * fxn;
    double dfyi = F(dfyo, ijp) * fxp + F(dfyo, ijn) * fxn;
    double dfzi = F(dfzo, ijp) * fxp + F(dfzo, ijn) * fxn;
    double fie = F(fi, ijp) * fxp + F(fi, ijn) * fxn + dfxi * (F(m->xf, i) - xi) +
                 dfyi * (F(m->yf, i) - yi) + dfzi * (F(m->zf, i) - zi);
    double dfxe = fie * F(m->arx, i), dfye = fie * F(m->ary, i), dfze = fie * F(m->arz, i);
    F(dfx, ijp) = F(dfx, ijp) + dfxe;
    F(dfy, ijp) = F(dfy, ijp) + dfye;
    F(dfz, ijp) = F(dfz, ijp) + dfze;
    F(dfx, ijn) = F(dfx, ijn) - dfxe;
    F(dfy, ijn) = F(dfy, ijn) - dfye;
    F(dfz, ijn) = F(dfz, ijn) - dfze;
  }
  if (m->noc > 0) { /* O- and C-grid cuts (:60-67): gradco on face ijlFace(i) with foc(i) */
    oc_pairs oc;
    if (get_oc(m, &oc)) return;
    for (int i = 1; i <= m->noc; ++i) {
      int iface = F(m->ijlFace, i), ijp = F(oc.ijl, i), ijn = F(oc.ijr, i);
      double fxn = F(oc.foc, i);
      double fxp = 1.0 - fxn;
      double xi = F(m->xc, ijp) * fxp + F(m->xc, ijn) * fxn;
      double yi = F(m->yc, ijp) * fxp + F(m->yc, ijn) * fxn;
      double zi = F(m->zc, ijp) * fxp + F(m->zc, ijn) * fxn;
      double dfxi = F(dfxo, ijp) * fxp + F(dfxo, ijn) * fxn;
      double dfyi = F(dfyo, ijp) * fxp + F(dfyo, ijn) * fxn;
      double dfzi = F(dfzo, ijp) * fxp + F(dfzo, ijn) * fxn;
      double fie = F(fi, ijp) * fxp + F(fi, ijn) * fxn + dfxi * (F(m->xf, iface) - xi) +
                   dfyi * (F(m->yf, iface) - yi) + dfzi * (F(m->zf, iface) - zi);
      double dfxe = fie * F(m->arx, iface), dfye = fie * F(m->ary, iface),
             dfze = fie * F(m->arz, iface);
      F(dfx, ijp) = F(dfx, ijp) + dfxe;
      F(dfy, ijp) = F(dfy, ijp) + dfye;
      F(dfz, ijp) = F(dfz, ijp) + dfze;
      F(dfx, ijn) = F(dfx, ijn) - dfxe;
      F(dfy, ijn) = F(dfy, ijn) - dfye;
      F(dfz, ijn) = F(dfz, ijn) - dfze;
    }
    free_oc(&oc);
  }
  /* Boundary loops :70-103 in patch-type order; gradbc :194-211. */
  const int cnt[5] = {m->ninl, m->nout, m->nsym, m->nwal, m->npru};
  const int fst[5] = {m->iInletFacesStart, m->iOutletFacesStart, m->iSymmetryFacesStart,
                      m->iWallFacesStart, m->iPressOutletFacesStart};
  const int bst[5] = {iInletStart(m), iOutletStart(m), iSymmetryStart(m), iWallStart(m),
                      iPressOutletStart(m)};
  for (int t = 0; t < 5; ++t)
    for (int i = 1; i <= cnt[t]; ++i) {
      int iface = fst[t] + i;
      int ijp = F(m->owner, iface);
      int ijb = bst[t] + i;
      F(dfx, ijp) = F(dfx, ijp) + F(fi, ijb) * F(m->arx, iface);
      F(dfy, ijp) = F(dfy, ijp) + F(fi, ijb) * F(m->ary, iface);
      F(dfz, ijp) = F(dfz, ijp) + F(fi, ijb) * F(m->arz, iface);
    }
  for (int ijp = 1; ijp <= n; ++ijp) { /* :108-113 */
    double volr = 1.0 / F(m->vol, ijp);
    F(dfx, ijp) = F(dfx, ijp) * volr;
    F(dfy, ijp) = F(dfy, ijp) * volr;
    F(dfz, ijp) = F(dfz, ijp) * volr;
  }
}

int orc_grad_gauss(const orc_mesh *m, const double *phi, int nigrad, int corrected,
                   double *dPhidxi) {
  int n = m->numCells;
  double *o = (double *)calloc((size_t)3 * n + 3, sizeof(double));
  double *g = (double *)calloc((size_t)3 * n + 3, sizeof(double));
  if (!o || !g) return -1;
  double *dfxo = o, *dfyo = o + n, *dfzo = o + 2 * n;
  double *dfx = g, *dfy = g + n, *dfz = g + 2 * n;
  int passes = nigrad;
  if (corrected) { /* grad_gauss_corrected.f90:38-40: old gradient = incoming */
    for (int i = 0; i < n; ++i) {
      dfxo[i] = dPhidxi[3 * i];
      dfyo[i] = dPhidxi[3 * i + 1];
      dfzo[i] = dPhidxi[3 * i + 2];
    }
    passes = 1;
  }
  for (int lc = 1; lc <= passes; ++lc) {
    gauss_pass(m, phi, dfxo, dfyo, dfzo, dfx, dfy, dfz);
    if (lc != passes) { /* :116-120 */
      memcpy(dfxo, dfx, sizeof(double) * n);
      memcpy(dfyo, dfy, sizeof(double) * n);
      memcpy(dfzo, dfz, sizeof(double) * n);
    }
  }
  for (int i = 0; i < n; ++i) {
    dPhidxi[3 * i] = dfx[i];
    dPhidxi[3 * i + 1] = dfy[i];
    dPhidxi[3 * i + 2] = dfz[i];
  }
  free(o);
  free(g);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* a7: grad_lsq.f90                                                           */
/* ------------------------------------------------------------------------- */

#define DM(c, i) dmat[9 * ((i)-1) + ((c)-1)]

int orc_grad_lsq_matrix(const orc_mesh *m, double *dmat) {
  int n = m->numCells;
  for (long k = 0; k < 9L * n; ++k) dmat[k] = 0.0; /* :54 */
  for (int i = 1; i <= m->numInnerFaces; ++i) {    /* :57-82 */
    int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    double Dx = F(m->xc, ijn) - F(m->xc, ijp);
    double Dy = F(m->yc, ijn) - F(m->yc, ijp);
    double Dz = F(m->zc, ijn) - F(m->zc, ijp);
    DM(1, ijp) += Dx * Dx;
    DM(1, ijn) += Dx * Dx;
    DM(4, ijp) += Dy * Dy;
    DM(4, ijn) += Dy * Dy;
    DM(6, ijp) += Dz * Dz;
    DM(6, ijn) += Dz * Dz;
    DM(2, ijp) += Dx * Dy;
    DM(2, ijn) += Dx * Dy;
    DM(3, ijp) += Dx * Dz;
    DM(3, ijn) += Dx * Dz;
    DM(5, ijp) += Dy * Dz;
    DM(5, ijn) += Dy * Dz;
  }
  if (m->noc > 0) { /* faces along O-C grid cuts (:85-108) */
    oc_pairs oc;
    if (get_oc(m, &oc)) return -1;
    for (int i = 1; i <= m->noc; ++i) {
      int ijp = F(oc.ijl, i), ijn = F(oc.ijr, i);
      double Dx = F(m->xc, ijn) - F(m->xc, ijp);
      double Dy = F(m->yc, ijn) - F(m->yc, ijp);
      double Dz = F(m->zc, ijn) - F(m->zc, ijp);
      DM(1, ijp) += Dx * Dx;
      DM(1, ijn) += Dx * Dx;
      DM(4, ijp) += Dy * Dy;
      DM(4, ijn) += Dy * Dy;
      DM(6, ijp) += Dz * Dz;
      DM(6, ijn) += Dz * Dz;
      DM(2, ijp) += Dx * Dy;
      DM(2, ijn) += Dx * Dy;
      DM(3, ijp) += Dx * Dz;
      DM(3, ijn) += Dx * Dz;
      DM(5, ijp) += Dy * Dz;
      DM(5, ijn) += Dy * Dz;
    }
    free_oc(&oc);
  }
  int nbf = m->numFaces - m->numInnerFaces;
  for (int i = 1; i <= nbf; ++i) { /* :116-130 */
    int iface = m->numInnerFaces + i;
    int ijp = F(m->owner, iface);
    double Dx = F(m->xf, iface) - F(m->xc, ijp);
    double Dy = F(m->yf, iface) - F(m->yc, ijp);
    double Dz = F(m->zf, iface) - F(m->zc, ijp);
    DM(1, ijp) += Dx * Dx;
    DM(4, ijp) += Dy * Dy;
    DM(6, ijp) += Dz * Dz;
    DM(2, ijp) += Dx * Dy;
    DM(3, ijp) += Dx * Dz;
    DM(5, ijp) += Dy * Dz;
  }
  for (int inp = 1; inp <= n; ++inp) { /* :134-165 */
    double d11 = DM(1, inp), d12 = DM(2, inp), d13 = DM(3, inp);
    double d22 = DM(4, inp), d23 = DM(5, inp), d33 = DM(6, inp);
    double d21 = d12, d31 = d13, d32 = d23;
    double tmp = 1.0 / (d11 * d22 * d33 - d11 * d23 * d32 - d12 * d21 * d33 + d12 * d23 * d31 +
                        d13 * d21 * d32 - d13 * d22 * d31);
    DM(1, inp) = (d22 * d33 - d23 * d32) * tmp;
    DM(2, inp) = (d21 * d33 - d23 * d31) * tmp;
    DM(3, inp) = (d21 * d32 - d22 * d31) * tmp;
    DM(4, inp) = (d11 * d33 - d13 * d31) * tmp;
    DM(5, inp) = (d12 * d33 - d13 * d32) * tmp;
    DM(6, inp) = (d11 * d32 - d12 * d31) * tmp;
    DM(7, inp) = (d12 * d23 - d13 * d22) * tmp;
    DM(8, inp) = (d11 * d23 - d13 * d21) * tmp;
    DM(9, inp) = (d11 * d22 - d12 * d21) * tmp;
  }
  return 0;
}

int orc_grad_lsq(const orc_mesh *m, const double *fi, const double *dmat, double *dFidxi) {
  int n = m->numCells;
  double *b = (double *)calloc((size_t)3 * n + 3, sizeof(double));
  if (!b) return -1;
  double *b1 = b, *b2 = b + n, *b3 = b + 2 * n;
  for (int i = 1; i <= m->numInnerFaces; ++i) { /* :179-196 */
    int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    double Dx = (F(m->xc, ijn) - F(m->xc, ijp)) * (F(fi, ijn) - F(fi, ijp));
    double Dy = (F(m->yc, ijn) - F(m->yc, ijp)) * (F(fi, ijn) - F(fi, ijp));
    double Dz = (F(m->zc, ijn) - F(m->zc, ijp)) * (F(fi, ijn) - F(fi, ijp));
    F(b1, ijp) += Dx;
    F(b1, ijn) += Dx;
    F(b2, ijp) += Dy;
    F(b2, ijn) += Dy;
    F(b3, ijp) += Dz;
    F(b3, ijn) += Dz;
  }
  if (m->noc > 0) { /* faces along O-C grid cuts (:198-214) */
    oc_pairs oc;
    if (get_oc(m, &oc)) return -1;
    for (int i = 1; i <= m->noc; ++i) {
      int ijp = F(oc.ijl, i), ijn = F(oc.ijr, i);
      double Dx = (F(m->xc, ijn) - F(m->xc, ijp)) * (F(fi, ijn) - F(fi, ijp));
      double Dy = (F(m->yc, ijn) - F(m->yc, ijp)) * (F(fi, ijn) - F(fi, ijp));
      double Dz = (F(m->zc, ijn) - F(m->zc, ijp)) * (F(fi, ijn) - F(fi, ijp));
      F(b1, ijp) += Dx;
      F(b1, ijn) += Dx;
      F(b2, ijp) += Dy;
      F(b2, ijn) += Dy;
      F(b3, ijp) += Dz;
      F(b3, ijn) += Dz;
    }
    free_oc(&oc);
  }
  const int cnt[5] = {m->ninl, m->nout, m->nsym, m->nwal, m->npru};
  const int fst[5] = {m->iInletFacesStart, m->iOutletFacesStart, m->iSymmetryFacesStart,
                      m->iWallFacesStart, m->iPressOutletFacesStart};
  const int bst[5] = {iInletStart(m), iOutletStart(m), iSymmetryStart(m), iWallStart(m),
                      iPressOutletStart(m)};
  for (int t = 0; t < 5; ++t) /* :220-293 */
    for (int i = 1; i <= cnt[t]; ++i) {
      int iface = fst[t] + i;
      int ijp = F(m->owner, iface);
      int ijn = bst[t] + i;
      double Dx = (F(fi, ijn) - F(fi, ijp)) * (F(m->xf, iface) - F(m->xc, ijp));
      double Dy = (F(fi, ijn) - F(fi, ijp)) * (F(m->yf, iface) - F(m->yc, ijp));
      double Dz = (F(fi, ijn) - F(fi, ijp)) * (F(m->zf, iface) - F(m->zc, ijp));
      F(b1, ijp) += Dx;
      F(b2, ijp) += Dy;
      F(b3, ijp) += Dz;
    }
  for (int inp = 1; inp <= n; ++inp) { /* :300-306 */
    G3(dFidxi, 1, inp) = F(b1, inp) * DM(1, inp) - F(b2, inp) * DM(2, inp) + F(b3, inp) * DM(3, inp);
    G3(dFidxi, 2, inp) = F(b1, inp) * DM(4, inp) - F(b2, inp) * DM(5, inp) - F(b3, inp) * DM(6, inp);
    G3(dFidxi, 3, inp) = F(b1, inp) * DM(7, inp) - F(b2, inp) * DM(8, inp) + F(b3, inp) * DM(9, inp);
  }
  free(b);
  return 0;
}
#undef DM

/* ------------------------------------------------------------------------- */
/* a8: bpres.f90                                                              */
/* ------------------------------------------------------------------------- */

int orc_bpres(const orc_mesh *m, double *p, const double *dPdxi, int istage) {
  const int cnt[5] = {m->ninl, m->nout, m->nsym, m->nwal, m->npru};
  const int fst[5] = {m->iInletFacesStart, m->iOutletFacesStart, m->iSymmetryFacesStart,
                      m->iWallFacesStart, m->iPressOutletFacesStart};
  const int bst[5] = {iInletStart(m), iOutletStart(m), iSymmetryStart(m), iWallStart(m),
                      iPressOutletStart(m)};
  /* the O-C slots follow the pressure-outlet ones (iOCStart, :603) */
  const int ocst = iPressOutletStart(m) + m->npru;
  if (istage == 1) { /* :37-96: every boundary slot takes its owner value */
    for (int t = 0; t < 5; ++t)
      for (int i = 1; i <= cnt[t]; ++i) F(p, bst[t] + i) = F(p, F(m->owner, fst[t] + i));
    for (int i = 1; i <= m->noc; ++i) /* :89-95 */
      F(p, ocst + i) = F(p, F(m->owner, m->iOCFacesStart + i));
  } else { /* :98-148: wall and pressure-outlet slots are extrapolated */
    for (int t = 3; t < 5; ++t)
      for (int i = 1; i <= cnt[t]; ++i) {
        int iface = fst[t] + i;
        int ijp = F(m->owner, iface);
        double xpb = F(m->xf, iface) - F(m->xc, ijp);
        double ypb = F(m->yf, iface) - F(m->yc, ijp);
        double zpb = F(m->zf, iface) - F(m->zc, ijp);
        F(p, bst[t] + i) = F(p, ijp) + G3(dPdxi, 1, ijp) * xpb + G3(dPdxi, 2, ijp) * ypb +
                           G3(dPdxi, 3, ijp) * zpb;
      }
    for (int i = 1; i <= m->noc; ++i) { /* O-C grid cuts :134-148 */
      int ijp = F(m->owner, m->iOCFacesStart + i);
      /* the distance is taken from face i's centre, as :140-142 write it */
      double xpb = F(m->xf, i) - F(m->xc, ijp);
      double ypb = F(m->yf, i) - F(m->yc, ijp);
      double zpb = F(m->zf, i) - F(m->zc, ijp);
      F(p, ocst + i) = F(p, ijp) + G3(dPdxi, 1, ijp) * xpb + G3(dPdxi, 2, ijp) * ypb +
                       G3(dPdxi, 3, ijp) * zpb;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* a9-a11: Krylov solvers                                                     */
/* ------------------------------------------------------------------------- */

int orc_spmv(int n, const int *ioffset, const int *ja, const double *a, const double *x,
             double *y) {
  for (int i = 1; i <= n; ++i) {
    double s = 0.0;
    for (int k = F(ioffset, i); k <= F(ioffset, i + 1) - 1; ++k) s = s + F(a, k) * F(x, F(ja, k));
    F(y, i) = s;
  }
  return 0;
}

/* res = su - A fi and its L1 norm (dpcg.f90:51-64), the O-C couplings after the rows
 * (:58-61). */
static double initial_residual(int n, const int *ioffset, const int *ja, const double *a,
                               const double *su, const double *fi, double *res,
                               const orc_solver_opts *o) {
  for (int i = 1; i <= n; ++i) {
    double r = F(su, i);
    for (int k = F(ioffset, i); k <= F(ioffset, i + 1) - 1; ++k) r = r - F(a, k) * F(fi, F(ja, k));
    F(res, i) = r;
  }
  for (int i = 1; i <= o->noc; ++i) {
    F(res, F(o->ijl, i)) = F(res, F(o->ijl, i)) - F(o->ar, i) * F(fi, F(o->ijr, i));
    F(res, F(o->ijr, i)) = F(res, F(o->ijr, i)) - F(o->al, i) * F(fi, F(o->ijl, i));
  }
  double res0 = 0.0;
  for (int i = 0; i < n; ++i) res0 = res0 + fabs(res[i]);
  return res0;
}

/* M^-1 r with M = (D+L) D^-1 (D+U), d = 1/D (iccg.f90:94-111, bicgstab.f90:117-136). */
static void dic_apply(int n, const int *ioffset, const int *ja, const int *diag, const double *a,
                      const double *d, double small, const double *r, double *zk) {
  for (int i = 1; i <= n; ++i) {
    double z = F(r, i);
    for (int k = F(ioffset, i); k <= F(diag, i) - 1; ++k) z = z - F(a, k) * F(zk, F(ja, k));
    F(zk, i) = z * F(d, i);
  }
  for (int i = 0; i < n; ++i) zk[i] = zk[i] / (d[i] + small);
  for (int i = n; i >= 1; --i) {
    double z = F(zk, i);
    for (int k = F(diag, i) + 1; k <= F(ioffset, i + 1) - 1; ++k) z = z - F(a, k) * F(zk, F(ja, k));
    F(zk, i) = z * F(d, i);
  }
}

static void fill_out(orc_solver_out *out, double res0, double resl, int iters, int written) {
  if (!out) return;
  out->res0 = res0;
  out->resl = resl;
  out->iters = iters;
  out->resor_written = written;
  if (written) out->resor = res0;
}

/* Shared PCG body of dpcg.f90:80-147 / iccg.f90:244-325; dic != NULL selects DIC. */
static int pcg(int n, const int *ioffset, const int *ja, const int *diag, const double *a,
               const double *su, double *fi, double *res, const orc_solver_opts *o,
               orc_solver_out *out, int use_dic) {
  double *pk = (double *)calloc((size_t)n + 1, sizeof(double));
  double *zk = (double *)calloc((size_t)n + 1, sizeof(double));
  double *d = (double *)calloc((size_t)n + 1, sizeof(double));
  if (!pk || !zk || !d) return -1;
  double res0 = initial_residual(n, ioffset, ja, a, su, fi, res, o);
  if (o->early_exit && res0 < orc_const_tol()) { /* dpcg.f90:66-70 */
    fill_out(out, res0, res0, 0, 0);
    free(pk), free(zk), free(d);
    return 0;
  }
  if (use_dic) { /* iccg.f90:231-237 */
    for (int i = 1; i <= n; ++i) {
      double di = F(a, F(diag, i));
      for (int k = F(ioffset, i); k <= F(diag, i) - 1; ++k)
        di = di - F(a, k) * F(a, k) * F(d, F(ja, k));
      F(d, i) = 1.0 / di;
    }
  }
  double s0 = s0_init(), resl = res0, resor = 0.0;
  int itr = 0;
  for (int l = 1; l <= o->nsw; ++l) {
    if (use_dic) {
      dic_apply(n, ioffset, ja, diag, a, d, o->small, res, zk);
    } else {
      for (int i = 1; i <= n; ++i) F(zk, i) = F(res, i) / F(a, F(diag, i));
    }
    double sk = 0.0;
    for (int i = 0; i < n; ++i) sk = sk + res[i] * zk[i];
    double bet = sk / s0;
    for (int i = 0; i < n; ++i) pk[i] = zk[i] + bet * pk[i];
    orc_spmv(n, ioffset, ja, a, pk, zk);
    for (int i = 1; i <= o->noc; ++i) { /* block boundaries, dpcg.f90:113-116 */
      F(zk, F(o->ijl, i)) = F(zk, F(o->ijl, i)) + F(o->ar, i) * F(pk, F(o->ijr, i));
      F(zk, F(o->ijr, i)) = F(zk, F(o->ijr, i)) + F(o->al, i) * F(pk, F(o->ijl, i));
    }
    double pkapk = 0.0;
    for (int i = 0; i < n; ++i) pkapk = pkapk + pk[i] * zk[i];
    double alf = sk / pkapk;
    for (int i = 0; i < n; ++i) fi[i] = fi[i] + alf * pk[i];
    for (int i = 0; i < n; ++i) res[i] = res[i] - alf * zk[i];
    resl = 0.0;
    for (int i = 0; i < n; ++i) resl = resl + fabs(res[i]);
    s0 = sk;
    ++itr;
    if (l == 1) resor = res0;
    double rsm = resl / (resor + o->small);
    if (o->trace) {
      o->trace[2 * (l - 1)] = resl;
      o->trace[2 * (l - 1) + 1] = rsm;
    }
    if (rsm < o->resmax) break;
  }
  fill_out(out, res0, resl, itr, itr > 0);
  free(pk), free(zk), free(d);
  return 0;
}

int orc_dpcg(int n, const int *ioffset, const int *ja, const int *diag, const double *a,
             const double *su, double *fi, double *res, const orc_solver_opts *o,
             orc_solver_out *out) {
  return pcg(n, ioffset, ja, diag, a, su, fi, res, o, out, 0);
}

int orc_iccg(int n, const int *ioffset, const int *ja, const int *diag, const double *a,
             const double *su, double *fi, double *res, const orc_solver_opts *o,
             orc_solver_out *out) {
  return pcg(n, ioffset, ja, diag, a, su, fi, res, o, out, 1);
}

/* bicgstab.f90:1-231 (right-preconditioned, DILU). */
int orc_bicgstab(int n, const int *ioffset, const int *ja, const int *diag, const double *a,
                 const double *su, double *fi, double *res, const orc_solver_opts *o,
                 orc_solver_out *out) {
  size_t sz = (size_t)n + 1;
  double *reso = calloc(sz, sizeof(double)), *pk = calloc(sz, sizeof(double));
  double *uk = calloc(sz, sizeof(double)), *zk = calloc(sz, sizeof(double));
  double *vk = calloc(sz, sizeof(double)), *d = calloc(sz, sizeof(double));
  if (!reso || !pk || !uk || !zk || !vk || !d) return -1;
  double res0 = initial_residual(n, ioffset, ja, a, su, fi, res, o);
  if (o->early_exit && res0 < orc_const_tol()) {
    fill_out(out, res0, res0, 0, 0);
    free(reso), free(pk), free(uk), free(zk), free(vk), free(d);
    return 0;
  }
  /* DILU diagonal (:68-79): the transpose entry a(l) is found by a scan of row ja(k)
   * from its diagonal; when the scan finds nothing l ends one past the row. */
  for (int i = 1; i <= n; ++i) {
    double di = F(a, F(diag, i));
    for (int k = F(ioffset, i); k <= F(diag, i) - 1; ++k) {
      int jr = F(ja, k);
      int l;
      for (l = F(diag, jr); l <= F(ioffset, jr + 1) - 1; ++l)
        if (F(ja, l) == i) break;
      di = di - F(a, k) * F(d, jr) * F(a, l);
    }
    F(d, i) = 1.0 / di;
  }
  memcpy(reso, res, sizeof(double) * n);
  double alf = 1.0, beto = 1.0, gam = 1.0, resl = res0, resor = 0.0;
  int itr = 0;
  for (int l = 1; l <= o->nsw; ++l) {
    double bet = 0.0;
    for (int i = 0; i < n; ++i) bet = bet + res[i] * reso[i];
    double om = bet * gam / (alf * beto + o->small);
    beto = bet;
    for (int i = 0; i < n; ++i) pk[i] = res[i] + om * (pk[i] - alf * uk[i]);
    dic_apply(n, ioffset, ja, diag, a, d, o->small, pk, zk);
    orc_spmv(n, ioffset, ja, a, zk, uk);
    double ukreso = 0.0;
    for (int i = 0; i < n; ++i) ukreso = ukreso + uk[i] * reso[i];
    gam = bet / ukreso;
    for (int i = 0; i < n; ++i) fi[i] = fi[i] + gam * zk[i];
    for (int i = 0; i < n; ++i) res[i] = res[i] - gam * uk[i];
    dic_apply(n, ioffset, ja, diag, a, d, o->small, res, zk);
    orc_spmv(n, ioffset, ja, a, zk, vk);
    double vr = 0.0, vv = 0.0;
    for (int i = 0; i < n; ++i) vr = vr + vk[i] * res[i];
    for (int i = 0; i < n; ++i) vv = vv + vk[i] * vk[i];
    alf = vr / (vv + o->small);
    for (int i = 0; i < n; ++i) fi[i] = fi[i] + alf * zk[i];
    for (int i = 0; i < n; ++i) res[i] = res[i] - alf * vk[i];
    resl = 0.0;
    for (int i = 0; i < n; ++i) resl = resl + fabs(res[i]);
    ++itr;
    if (l == 1) resor = res0;
    double rsm = resl / (resor + o->small);
    if (o->trace) {
      o->trace[2 * (l - 1)] = resl;
      o->trace[2 * (l - 1) + 1] = rsm;
    }
    if (rsm < o->resmax) break;
  }
  fill_out(out, res0, resl, itr, itr > 0);
  free(reso), free(pk), free(uk), free(zk), free(vk), free(d);
  return 0;
}

/* --- calcp corrections after the p' solve --------------------------------------------- */
/* calcp-multiple_correction_SIMPLE.f90:159-171: flmass(i) = flmass(i) + a(k)*(pp(ijn)-pp(ijp)),
 * k = icell_jcell_csr_value_index(i). */
int orc_flux_correct(const orc_mesh *m, const int *slot_pn, const double *a, const double *pp,
                     double *flmass) {
  for (int i = 0; i < m->numInnerFaces; ++i) {
    const int ijp = m->owner[i] - 1, ijn = m->neighbour[i] - 1;
    flmass[i] = flmass[i] + a[slot_pn[i] - 1] * (pp[ijn] - pp[ijp]);
  }
  if (m->noc > 0) { /* faces along O-C grid cuts (calcp :166-171) */
    oc_pairs oc;
    if (get_oc(m, &oc)) return -1;
    const double *ar = a + m->numCells + 2L * m->numInnerFaces;
    double *fmoc = flmass + m->numInnerFaces;
    for (int i = 1; i <= m->noc; ++i)
      F(fmoc, i) = F(fmoc, i) + F(ar, i) * (F(pp, F(oc.ijr, i)) - F(pp, F(oc.ijl, i)));
    free_oc(&oc);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Momentum assembly: calcuvw.f90:48-438                                       */
/* ------------------------------------------------------------------------- */

/* MIN / MAX keeping the first argument on ties. */
static double rmin(double a, double b) { return b < a ? b : a; }
static double rmax(double a, double b) { return b > a ? b : a; }

/* interpolation.f90:65-93 */
static double fv_cds(int ijp, int ijn, double lambda, const double *fi) {
  const double fxn = lambda, fxp = 1.0 - lambda;
  return F(fi, ijp) * fxp + F(fi, ijn) * fxn;
}

/* interpolation.f90:99-139 */
static double fv_cdsc(const orc_mesh *m, int ijp, int ijn, double xf, double yf, double zf,
                      double lambda, const double *fi, const double *g) {
  const double fxn = lambda, fxp = 1.0 - lambda;
  const double xi = F(m->xc, ijp) * fxp + F(m->xc, ijn) * fxn;
  const double yi = F(m->yc, ijp) * fxp + F(m->yc, ijn) * fxn;
  const double zi = F(m->zc, ijp) * fxp + F(m->zc, ijn) * fxn;
  const double dfixi = G3(g, 1, ijp) * fxp + G3(g, 1, ijn) * fxn;
  const double dfiyi = G3(g, 2, ijp) * fxp + G3(g, 2, ijn) * fxn;
  const double dfizi = G3(g, 3, ijp) * fxp + G3(g, 3, ijn) * fxn;
  return F(fi, ijp) * fxp + F(fi, ijn) * fxn +
         (dfixi * (xf - xi) + dfiyi * (yf - yi) + dfizi * (zf - zi));
}

/* interpolation.f90:204-249 */
static double fv_2nd_upwind(const orc_mesh *m, int inp, double xf, double yf, double zf,
                            const double *fi, const double *g) {
  const double gradfidr = G3(g, 1, inp) * (xf - F(m->xc, inp)) + G3(g, 2, inp) * (yf - F(m->yc, inp)) +
                          G3(g, 3, inp) * (zf - F(m->zc, inp));
  return F(fi, inp) + gradfidr;
}

/* interpolation.f90:254-320 */
static double fv_muscl(const orc_mesh *m, int inp, int inn, double xf, double yf, double zf,
                       const double *fi, const double *g) {
  const double theta = 0.125;
  const double phi_p = F(fi, inp), phi_n = F(fi, inn);
  const double xcp = F(m->xc, inp), ycp = F(m->yc, inp), zcp = F(m->zc, inp);
  const double xcn = F(m->xc, inn), ycn = F(m->yc, inn), zcn = F(m->zc, inn);
  const double gpx = G3(g, 1, inp), gpy = G3(g, 2, inp), gpz = G3(g, 3, inp);
  const double gnx = G3(g, 1, inn), gny = G3(g, 2, inn), gnz = G3(g, 3, inn);
  const double gr2 = gpx * (xf - xcp) + gpy * (yf - ycp) + gpz * (zf - zcp);
  const double grc = gpx * (xf - xcp) + gpy * (yf - ycp) + gpz * (zf - zcp) + gnx * (xf - xcn) +
                     gny * (yf - ycn) + gnz * (zf - zcn);
  const double fv2 = (phi_p + gr2);
  const double fvc = 0.5 * (phi_p + phi_n + grc);
  return theta * fvc + (1.0 - theta) * fv2;
}

/* interpolation.f90:325-393 */
static double fv_limiter(const orc_mesh *m, int limiter, int ijp, int ijn, double lambda,
                         const double *u, const double *g) {
  const double fxp = 1.0 - lambda;
  const double xpn = F(m->xc, ijn) - F(m->xc, ijp);
  const double ypn = F(m->yc, ijn) - F(m->yc, ijp);
  const double zpn = F(m->zc, ijn) - F(m->zc, ijp);
  const double r = (2 * G3(g, 1, ijp) * xpn + 2 * G3(g, 2, ijp) * ypn + 2 * G3(g, 3, ijp) * zpn) /
                       (F(u, ijn) - F(u, ijp)) -
                   1.0;
  double psi;
  if (limiter == 0)
    psi = rmax(0., rmin(rmin(2. * r, 0.75 * r + 0.25), 4.));
  else if (limiter == 1)
    psi = rmax(0., rmin(rmin(1.5 * r, 0.75 * r + 0.25), 2.5));
  else if (limiter == 2)
    psi = rmax(0., rmin(rmin(2. * r, 0.5 * r + 0.5), 2.));
  else if (limiter == 3)
    psi = rmax(0., rmin(rmin(rmin(2. * r, 0.75 * r + 0.25), 0.25 * r + 0.75), 2.));
  else if (limiter == 4)
    psi = rmax(0., rmin(rmin(2. * r, 2. / 3. * r + 1. / 3.), 2.));
  else if (limiter == 5)
    psi = (r + fabs(r)) * (3 * r + 1.) / (2 * ((r + 1.) * (r + 1.)));
  else if (limiter == 6)
    psi = 1.5 * r * (r + 1.) / (r * r + r + 1.);
  else
    psi = 1.0;
  return F(u, ijp) + fxp * psi * (F(u, ijn) - F(u, ijp));
}

/* face_value (interpolation.f90:20-60) */
static double face_value(const orc_mesh *m, const orc_uvw_params *prm, int ijp, int ijn,
                         double xf, double yf, double zf, double lambda, const double *u,
                         const double *g) {
  switch (prm->scheme) {
    case 0: return fv_cds(ijp, ijn, lambda, u);
    case 1: return fv_cdsc(m, ijp, ijn, xf, yf, zf, lambda, u, g);
    case 2: return face_value_central(m, ijp, ijn, xf, yf, zf, u, g);
    case 3: return fv_2nd_upwind(m, ijp, xf, yf, zf, u, g);
    case 5: return fv_limiter(m, prm->limiter, ijp, ijn, lambda, u, g);
    default: return fv_muscl(m, ijp, ijn, xf, yf, zf, u, g);
  }
}

/* sngrad_scalar_field with nrelax = 0, approach 'skewness' (gradients.f90:547-721). */
static void sngrad(const orc_mesh *m, int ijp, int ijn, double arx, double ary, double arz,
                   double lambda, const double *fi, const double *g, double *dfixi,
                   double *dfiyi, double *dfizi, double *dfixii, double *dfiyii, double *dfizii) {
  const double fxn = lambda, fxp = 1.0 - lambda;
  const double xpn = F(m->xc, ijn) - F(m->xc, ijp);
  const double ypn = F(m->yc, ijn) - F(m->yc, ijp);
  const double zpn = F(m->zc, ijn) - F(m->zc, ijp);
  const double costn = 1.0;
  const double vole = xpn * arx + ypn * ary + zpn * arz;
  *dfixi = G3(g, 1, ijp) * fxp + G3(g, 1, ijn) * fxn;
  *dfiyi = G3(g, 2, ijp) * fxp + G3(g, 2, ijn) * fxn;
  *dfizi = G3(g, 3, ijp) * fxp + G3(g, 3, ijn) * fxn;
  const double d1x = costn, d1y = costn, d1z = costn;
  const double d2x = xpn * costn, d2y = ypn * costn, d2z = zpn * costn;
  *dfixii = *dfixi * d1x + arx / vole * (F(fi, ijn) - F(fi, ijp) - *dfixi * d2x - *dfiyi * d2y - *dfizi * d2z);
  *dfiyii = *dfiyi * d1y + ary / vole * (F(fi, ijn) - F(fi, ijp) - *dfixi * d2x - *dfiyi * d2y - *dfizi * d2z);
  *dfizii = *dfizi * d1z + arz / vole * (F(fi, ijn) - F(fi, ijp) - *dfixi * d2x - *dfiyi * d2y - *dfizi * d2z);
}

/* facefluxuvw for inner faces (faceflux_velocity.f90:35-184). */
static void facefluxuvw(const orc_mesh *m, const orc_uvw_params *prm, int ijp, int ijn,
                        double xf, double yf, double zf, double arx, double ary, double arz,
                        double flomass, double lambda, double gam, const double *u,
                        const double *v, const double *w, const double *vis,
                        const double *dUdxi, const double *dVdxi, const double *dWdxi,
                        double *cap, double *can, double *sup, double *svp, double *swp) {
  const double fxn = lambda, fxp = 1.0 - lambda;
  const double xpn = F(m->xc, ijn) - F(m->xc, ijp);
  const double ypn = F(m->yc, ijn) - F(m->yc, ijp);
  const double zpn = F(m->zc, ijn) - F(m->zc, ijp);
  const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
  const double are = sqrt(arx * arx + ary * ary + arz * arz);
  const double game = F(vis, ijp) * fxp + F(vis, ijn) * fxn;
  const double de = game * are / dpn;
  *can = -de + rmin(flomass, 0.0);
  *cap = -de - rmax(flomass, 0.0);
  double duxi, duyi, duzi, duxii, duyii, duzii, dvxi, dvyi, dvzi, dvxii, dvyii, dvzii;
  double dwxi, dwyi, dwzi, dwxii, dwyii, dwzii;
  sngrad(m, ijp, ijn, arx, ary, arz, lambda, u, dUdxi, &duxi, &duyi, &duzi, &duxii, &duyii, &duzii);
  sngrad(m, ijp, ijn, arx, ary, arz, lambda, v, dVdxi, &dvxi, &dvyi, &dvzi, &dvxii, &dvyii, &dvzii);
  sngrad(m, ijp, ijn, arx, ary, arz, lambda, w, dWdxi, &dwxi, &dwyi, &dwzi, &dwxii, &dwyii, &dwzii);
  const double fdue = game * ((duxii + duxii) * arx + (duyii + dvxii) * ary + (duzii + dwxii) * arz);
  const double fdve = game * ((duyii + dvxii) * arx + (dvyii + dvyii) * ary + (dvzii + dwyii) * arz);
  const double fdwe = game * ((duzii + dwxii) * arx + (dwyii + dvzii) * ary + (dwzii + dwzii) * arz);
  const double fdui = game * are / dpn * (duxi * xpn + duyi * ypn + duzi * zpn);
  const double fdvi = game * are / dpn * (dvxi * xpn + dvyi * ypn + dvzi * zpn);
  const double fdwi = game * are / dpn * (dwxi * xpn + dwyi * ypn + dwzi * zpn);
  const double fuuds = rmax(flomass, 0.0) * F(u, ijp) + rmin(flomass, 0.0) * F(u, ijn);
  const double fvuds = rmax(flomass, 0.0) * F(v, ijp) + rmin(flomass, 0.0) * F(v, ijn);
  const double fwuds = rmax(flomass, 0.0) * F(w, ijp) + rmin(flomass, 0.0) * F(w, ijn);
  double ue, ve, we;
  if (flomass >= 0.0) {
    ue = face_value(m, prm, ijp, ijn, xf, yf, zf, fxp, u, dUdxi);
    ve = face_value(m, prm, ijp, ijn, xf, yf, zf, fxp, v, dVdxi);
    we = face_value(m, prm, ijp, ijn, xf, yf, zf, fxp, w, dWdxi);
  } else {
    ue = face_value(m, prm, ijn, ijp, xf, yf, zf, fxn, u, dUdxi);
    ve = face_value(m, prm, ijn, ijp, xf, yf, zf, fxn, v, dVdxi);
    we = face_value(m, prm, ijn, ijp, xf, yf, zf, fxn, w, dWdxi);
  }
  const double fuhigh = flomass * ue, fvhigh = flomass * ve, fwhigh = flomass * we;
  *sup = -gam * (fuhigh - fuuds) + fdue - fdui;
  *svp = -gam * (fvhigh - fvuds) + fdve - fdvi;
  *swp = -gam * (fwhigh - fwuds) + fdwe - fdwi;
}

/* facefluxuvw_cyclic (faceflux_velocity.f90:189-354), which the generic facefluxuvw
 * resolves to for the O-C pairs (calcuvw.f90:193-194): facefluxuvw with the distance
 * dpn = |S| / srd and the vector (xpn, ypn, zpn) = dpn S / |S| (sngrad keeps the cell
 * centres). */
static void facefluxuvw_cyclic(const orc_mesh *m, const orc_uvw_params *prm, int ijp, int ijn,
                               double xf, double yf, double zf, double arx, double ary,
                               double arz, double flomass, double lambda, double gam,
                               double srd, const double *u, const double *v, const double *w,
                               const double *vis, const double *dUdxi, const double *dVdxi,
                               const double *dWdxi, double *cap, double *can, double *sup,
                               double *svp, double *swp) {
  const double fxn = lambda, fxp = 1.0 - lambda;
  const double are = sqrt(arx * arx + ary * ary + arz * arz);
  const double dpn = are / srd;
  const double xpn = dpn * arx / are, ypn = dpn * ary / are, zpn = dpn * arz / are;
  const double game = F(vis, ijp) * fxp + F(vis, ijn) * fxn;
  const double de = game * are / dpn;
  *can = -de + rmin(flomass, 0.0);
  *cap = -de - rmax(flomass, 0.0);
  double duxi, duyi, duzi, duxii, duyii, duzii, dvxi, dvyi, dvzi, dvxii, dvyii, dvzii;
  double dwxi, dwyi, dwzi, dwxii, dwyii, dwzii;
  sngrad(m, ijp, ijn, arx, ary, arz, lambda, u, dUdxi, &duxi, &duyi, &duzi, &duxii, &duyii, &duzii);
  sngrad(m, ijp, ijn, arx, ary, arz, lambda, v, dVdxi, &dvxi, &dvyi, &dvzi, &dvxii, &dvyii, &dvzii);
  sngrad(m, ijp, ijn, arx, ary, arz, lambda, w, dWdxi, &dwxi, &dwyi, &dwzi, &dwxii, &dwyii, &dwzii);
  const double fdue = game * ((duxii + duxii) * arx + (duyii + dvxii) * ary + (duzii + dwxii) * arz);
  const double fdve = game * ((duyii + dvxii) * arx + (dvyii + dvyii) * ary + (dvzii + dwyii) * arz);
  const double fdwe = game * ((duzii + dwxii) * arx + (dwyii + dvzii) * ary + (dwzii + dwzii) * arz);
  const double fdui = game * are / dpn * (duxi * xpn + duyi * ypn + duzi * zpn);
  const double fdvi = game * are / dpn * (dvxi * xpn + dvyi * ypn + dvzi * zpn);
  const double fdwi = game * are / dpn * (dwxi * xpn + dwyi * ypn + dwzi * zpn);
  const double fuuds = rmax(flomass, 0.0) * F(u, ijp) + rmin(flomass, 0.0) * F(u, ijn);
  const double fvuds = rmax(flomass, 0.0) * F(v, ijp) + rmin(flomass, 0.0) * F(v, ijn);
  const double fwuds = rmax(flomass, 0.0) * F(w, ijp) + rmin(flomass, 0.0) * F(w, ijn);
  double ue, ve, we;
  if (flomass >= 0.0) {
    ue = face_value(m, prm, ijp, ijn, xf, yf, zf, fxp, u, dUdxi);
    ve = face_value(m, prm, ijp, ijn, xf, yf, zf, fxp, v, dVdxi);
    we = face_value(m, prm, ijp, ijn, xf, yf, zf, fxp, w, dWdxi);
  } else {
    ue = face_value(m, prm, ijn, ijp, xf, yf, zf, fxn, u, dUdxi);
    ve = face_value(m, prm, ijn, ijp, xf, yf, zf, fxn, v, dVdxi);
    we = face_value(m, prm, ijn, ijp, xf, yf, zf, fxn, w, dWdxi);
  }
  const double fuhigh = flomass * ue, fvhigh = flomass * ve, fwhigh = flomass * we;
  *sup = -gam * (fuhigh - fuuds) + fdue - fdui;
  *svp = -gam * (fvhigh - fvuds) + fdve - fdvi;
  *swp = -gam * (fwhigh - fwuds) + fdwe - fdwi;
}

/* The cb coefficient of facefluxuvw_boundary (faceflux_velocity.f90:403-468): the only
 * result calcuvw's inlet and outlet loops use. */
static double boundary_cb(const orc_mesh *m, int ijp, int ijb, int iface, double flomass,
                          const double *vis) {
  const double xpn = F(m->xf, iface) - F(m->xc, ijp);
  const double ypn = F(m->yf, iface) - F(m->yc, ijp);
  const double zpn = F(m->zf, iface) - F(m->zc, ijp);
  const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
  const double arx = F(m->arx, iface), ary = F(m->ary, iface), arz = F(m->arz, iface);
  const double are = sqrt(arx * arx + ary * ary + arz * arz);
  const double game = F(vis, ijb);
  const double de = game * are / dpn;
  return -de + rmin(flomass, 0.0);
}

/* Fortran SUM over a(ioffset(i):ioffset(i+1)-1). */
static double row_sum(const int *ioffset, const double *a, int i) {
  double s = 0.0;
  for (int k = F(ioffset, i); k <= F(ioffset, i + 1) - 1; ++k) s = s + F(a, k);
  return s;
}

int orc_calcuvw(const orc_mesh *m, const int *ioffset, const int *diag, const int *slot_pn,
                const int *slot_np, const orc_uvw_params *prm, const double *u, const double *v,
                const double *w, const double *p, const double *vis, const double *den,
                const double *t, const double *uo, const double *vo, const double *wo,
                const double *uoo, const double *voo, const double *woo, const double *dUdxi,
                const double *dVdxi, const double *dWdxi, const double *dPdxi,
                const double *flmass, const double *fmi, const double *fmo, double *a,
                double *diag_vw, double *rhs, double *ap) {
  const int n = m->numCells, nnz = F(ioffset, n + 1) - 1;
  const double small = orc_const_small_src();
  if (n < 3) return -1;
  double *su = calloc(n, sizeof(double)), *sv = calloc(n, sizeof(double)),
         *sw = calloc(n, sizeof(double)), *spu = calloc(n, sizeof(double)),
         *spv = calloc(n, sizeof(double)), *sp = calloc(n, sizeof(double)),
         *du = calloc(n, sizeof(double));
  if (!su || !sv || !sw || !spu || !spv || !sp || !du) return -9;

  /* calcPressDiv (fieldManipulation.f90:57-160), the pressure gradient given */
  for (int i = 1; i <= m->numInnerFaces; ++i) {
    const int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    const double fxn = F(m->facint, i), fxp = 1.0 - fxn;
    const double xi = F(m->xc, ijp) * fxp + F(m->xc, ijn) * fxn;
    const double yi = F(m->yc, ijp) * fxp + F(m->yc, ijn) * fxn;
    const double zi = F(m->zc, ijp) * fxp + F(m->zc, ijn) * fxn;
    /* df(ijp,k) on the (3,numCells) array dPdxi: flat element ijp + 3(k-1) */
    const double dfxi = dPdxi[ijp - 1] * fxp + dPdxi[ijn - 1] * fxn;
    const double dfyi = dPdxi[ijp - 1 + 3] * fxp + dPdxi[ijn - 1 + 3] * fxn;
    const double dfzi = dPdxi[ijp - 1 + 6] * fxp + dPdxi[ijn - 1 + 6] * fxn;
    const double fie = F(p, ijp) * fxp + F(p, ijn) * fxn + dfxi * (F(m->xf, i) - xi) +
                       dfyi * (F(m->yf, i) - yi) + dfzi * (F(m->zf, i) - zi);
    const double dfxe = fie * F(m->arx, i), dfye = fie * F(m->ary, i), dfze = fie * F(m->arz, i);
    F(su, ijp) = F(su, ijp) - dfxe;
    F(sv, ijp) = F(sv, ijp) - dfye;
    F(sw, ijp) = F(sw, ijp) - dfze;
    F(su, ijn) = F(su, ijn) + dfxe;
    F(sv, ijn) = F(sv, ijn) + dfye;
    F(sw, ijn) = F(sw, ijn) + dfze;
  }
  oc_pairs oc;
  if (get_oc(m, &oc)) return -9;
  for (int i = 1; i <= m->noc; ++i) { /* O- and C-grid cuts (fieldManipulation.f90:110-125) */
    const int iface = F(m->ijlFace, i), ijp = F(oc.ijl, i), ijn = F(oc.ijr, i);
    const double fxn = F(oc.foc, i), fxp = 1.0 - fxn;
    const double xi = F(m->xc, ijp) * fxp + F(m->xc, ijn) * fxn;
    const double yi = F(m->yc, ijp) * fxp + F(m->yc, ijn) * fxn;
    const double zi = F(m->zc, ijp) * fxp + F(m->zc, ijn) * fxn;
    const double dfxi = dPdxi[ijp - 1] * fxp + dPdxi[ijn - 1] * fxn;
    const double dfyi = dPdxi[ijp - 1 + 3] * fxp + dPdxi[ijn - 1 + 3] * fxn;
    const double dfzi = dPdxi[ijp - 1 + 6] * fxp + dPdxi[ijn - 1 + 6] * fxn;
    const double fie = F(p, ijp) * fxp + F(p, ijn) * fxn + dfxi * (F(m->xf, iface) - xi) +
                       dfyi * (F(m->yf, iface) - yi) + dfzi * (F(m->zf, iface) - zi);
    const double dfxe = fie * F(m->arx, iface), dfye = fie * F(m->ary, iface),
                 dfze = fie * F(m->arz, iface);
    F(su, ijp) = F(su, ijp) - dfxe;
    F(sv, ijp) = F(sv, ijp) - dfye;
    F(sw, ijp) = F(sw, ijp) - dfze;
    F(su, ijn) = F(su, ijn) + dfxe;
    F(sv, ijn) = F(sv, ijn) + dfye;
    F(sw, ijn) = F(sw, ijn) + dfze;
  }
  {
    const int cnt[5] = {m->ninl, m->nout, m->nsym, m->nwal, m->npru};
    const int fst[5] = {m->iInletFacesStart, m->iOutletFacesStart, m->iSymmetryFacesStart,
                        m->iWallFacesStart, m->iPressOutletFacesStart};
    const int bst[5] = {iInletStart(m), iOutletStart(m), iSymmetryStart(m), iWallStart(m),
                        iPressOutletStart(m)};
    for (int ty = 0; ty < 5; ++ty)
      for (int i = 1; i <= cnt[ty]; ++i) {
        const int iface = fst[ty] + i, ijp = F(m->owner, iface), ijb = bst[ty] + i;
        F(su, ijp) = F(su, ijp) - F(p, ijb) * F(m->arx, iface);
        F(sv, ijp) = F(sv, ijp) - F(p, ijb) * F(m->ary, iface);
        F(sw, ijp) = F(sw, ijp) - F(p, ijb) * F(m->arz, iface);
      }
  }
  /* volume sources (:76-139) */
  for (int inp = 1; inp <= n; ++inp) {
    if (prm->const_mflux) F(su, inp) = F(su, inp) + prm->gradPcmf * F(m->vol, inp);
    if (prm->buoyancy) {
      double heat;
      if (prm->boussinesq)
        heat = prm->beta * prm->densit * (F(t, inp) - prm->tref) * F(m->vol, inp);
      else
        heat = (prm->densit - F(den, inp)) * F(m->vol, inp);
      F(su, inp) = F(su, inp) - prm->gravx * heat;
      F(sv, inp) = F(sv, inp) - prm->gravy * heat;
      F(sw, inp) = F(sw, inp) - prm->gravz * heat;
    }
    if (prm->bdf) {
      const double apotime = F(den, inp) * F(m->vol, inp) / prm->timestep;
      double sut = apotime * ((1 + prm->btime) * F(uo, inp));
      double svt = apotime * ((1 + prm->btime) * F(vo, inp));
      double swt = apotime * ((1 + prm->btime) * F(wo, inp));
      if (prm->btime > (double)0.99f) {
        sut = sut - apotime * ((double)0.5f * prm->btime * F(uoo, inp));
        svt = svt - apotime * ((double)0.5f * prm->btime * F(voo, inp));
        swt = swt - apotime * ((double)0.5f * prm->btime * F(woo, inp));
      }
      F(su, inp) = F(su, inp) + sut;
      F(sv, inp) = F(sv, inp) + svt;
      F(sw, inp) = F(sw, inp) + swt;
      F(spu, inp) = F(spu, inp) + apotime * (1 + (double)0.5f * prm->btime);
      F(spv, inp) = F(spv, inp) + apotime * (1 + (double)0.5f * prm->btime);
      F(sp, inp) = F(sp, inp) + apotime * (1 + (double)0.5f * prm->btime);
    }
  }
  /* inner faces (:157-185) */
  for (int i = 1; i <= m->numInnerFaces; ++i) {
    const int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    double cap, can, sup, svp, swp;
    facefluxuvw(m, prm, ijp, ijn, F(m->xf, i), F(m->yf, i), F(m->zf, i), F(m->arx, i),
                F(m->ary, i), F(m->arz, i), F(flmass, i), F(m->facint, i), prm->gds, u, v, w,
                vis, dUdxi, dVdxi, dWdxi, &cap, &can, &sup, &svp, &swp);
    F(a, F(slot_pn, i)) = can;
    F(a, F(slot_np, i)) = cap;
    F(su, ijp) = F(su, ijp) + sup;
    F(sv, ijp) = F(sv, ijp) + svp;
    F(sw, ijp) = F(sw, ijp) + swp;
    F(su, ijn) = F(su, ijn) - sup;
    F(sv, ijn) = F(sv, ijn) - svp;
    F(sw, ijn) = F(sw, ijn) - swp;
  }
  if (m->noc > 0) { /* O- and C-grid cuts (:186-215): ar, al after the CSR values */
    double *ar = a + nnz, *al = a + nnz + m->noc;
    const double *fmoc = flmass + m->numInnerFaces;
    for (int i = 1; i <= m->noc; ++i) {
      const int iface = F(m->ijlFace, i), ijp = F(oc.ijl, i), ijn = F(oc.ijr, i);
      double sup, svp, swp;
      facefluxuvw_cyclic(m, prm, ijp, ijn, F(m->xf, iface), F(m->yf, iface), F(m->zf, iface),
                         F(m->arx, iface), F(m->ary, iface), F(m->arz, iface), F(fmoc, i),
                         F(oc.foc, i), prm->gds, F(oc.srdoc, i), u, v, w, vis, dUdxi, dVdxi,
                         dWdxi, &F(al, i), &F(ar, i), &sup, &svp, &swp);
      F(spu, ijp) = F(spu, ijp) - F(ar, i);
      F(spv, ijp) = F(spv, ijp) - F(ar, i);
      F(sp, ijp) = F(sp, ijp) - F(ar, i);
      F(spu, ijn) = F(spu, ijn) - F(al, i);
      F(spv, ijn) = F(spv, ijn) - F(al, i);
      F(sp, ijn) = F(sp, ijn) - F(al, i);
      F(su, ijp) = F(su, ijp) + sup;
      F(sv, ijp) = F(sv, ijp) + svp;
      F(sw, ijp) = F(sw, ijp) + swp;
      F(su, ijn) = F(su, ijn) - sup;
      F(sv, ijn) = F(sv, ijn) - svp;
      F(sw, ijn) = F(sw, ijn) - swp;
    }
  }
  free_oc(&oc);
  /* inlet and outlet (:223-264) */
  for (int pass = 0; pass < 2; ++pass) {
    const int cnt = pass == 0 ? m->ninl : m->nout;
    const int fst = pass == 0 ? m->iInletFacesStart : m->iOutletFacesStart;
    const int bst = pass == 0 ? iInletStart(m) : iOutletStart(m);
    const double *fm = pass == 0 ? fmi : fmo;
    for (int i = 1; i <= cnt; ++i) {
      const int iface = fst + i, ijp = F(m->owner, iface), ijb = bst + i;
      const double cb = boundary_cb(m, ijp, ijb, iface, F(fm, i), vis);
      F(spu, ijp) = F(spu, ijp) - cb;
      F(spv, ijp) = F(spv, ijp) - cb;
      F(sp, ijp) = F(sp, ijp) - cb;
      F(su, ijp) = F(su, ijp) - cb * F(u, ijb);
      F(sv, ijp) = F(sv, ijp) - cb * F(v, ijb);
      F(sw, ijp) = F(sw, ijp) - cb * F(w, ijb);
    }
  }
  /* symmetry (:268-306) and wall (:309-378), srds / srdw as init.f90:1002-1027 */
  for (int pass = 0; pass < 2; ++pass) {
    const int cnt = pass == 0 ? m->nsym : m->nwal;
    const int fst = pass == 0 ? m->iSymmetryFacesStart : m->iWallFacesStart;
    const int bst = pass == 0 ? iSymmetryStart(m) : iWallStart(m);
    for (int i = 1; i <= cnt; ++i) {
      const int iface = fst + i, ijp = F(m->owner, iface), ijb = bst + i;
      const double arx = F(m->arx, iface), ary = F(m->ary, iface), arz = F(m->arz, iface);
      const double are = sqrt(arx * arx + ary * ary + arz * arz);
      const double nxf = arx / are, nyf = ary / are, nzf = arz / are;
      const double dn = (F(m->xf, iface) - F(m->xc, ijp)) * nxf +
                        (F(m->yf, iface) - F(m->yc, ijp)) * nyf +
                        (F(m->zf, iface) - F(m->zc, ijp)) * nzf;
      const double srd = are / dn;
      const double dx = F(m->xc, ijp) - F(m->xf, iface), dy = F(m->yc, ijp) - F(m->yf, iface),
                   dz = F(m->zc, ijp) - F(m->zf, iface);
      const double dpb = sqrt(dx * dx + dy * dy + dz * dz);
      const double upb = F(u, ijp) - F(u, ijb), vpb = F(v, ijp) - F(v, ijb),
                   wpb = F(w, ijp) - F(w, ijb);
      if (pass == 0) {
        const double vsi = F(vis, ijb);
        const double cf = vsi * srd;
        const double vsol = vsi * are / dpb;
        const double fdne = 2 * cf * (upb * nxf + vpb * nyf + wpb * nzf);
        F(spu, ijp) = F(spu, ijp) + vsol;
        F(spv, ijp) = F(spv, ijp) + vsol;
        F(sp, ijp) = F(sp, ijp) + vsol;
        F(su, ijp) = F(su, ijp) + vsol * F(u, ijp) - fdne * nxf;
        F(sv, ijp) = F(sv, ijp) + vsol * F(v, ijp) - fdne * nyf;
        F(sw, ijp) = F(sw, ijp) + vsol * F(w, ijp) - fdne * nzf;
      } else {
        const double viss = prm->viscos;
        const double cf = viss * srd;
        const double vsol = viss * are / dpb;
        const double vnp = upb * nxf + vpb * nyf + wpb * nzf;
        const double utp = upb - vnp * nxf, vtp = vpb - vnp * nyf, wtp = wpb - vnp * nzf;
        F(spu, ijp) = F(spu, ijp) + vsol;
        F(spv, ijp) = F(spv, ijp) + vsol;
        F(sp, ijp) = F(sp, ijp) + vsol;
        F(su, ijp) = F(su, ijp) + vsol * F(u, ijp) - cf * utp;
        F(sv, ijp) = F(sv, ijp) + vsol * F(v, ijp) - cf * vtp;
        F(sw, ijp) = F(sw, ijp) + vsol * F(w, ijp) - cf * wtp;
      }
    }
  }
  if (prm->cn)
    for (int k = 1; k <= nnz; ++k) F(a, k) = 0.5 * F(a, k); /* :382-384 */

  /* the three components (:391-553) */
  double *S[3] = {su, sv, sw}, *SP[3] = {spu, spv, sp};
  const double *old[3] = {uo, vo, wo}, *cur[3] = {u, v, w};
  for (int comp = 0; comp < 3; ++comp) {
    double *s = S[comp];
    if (prm->cn) {
      for (int i = 1; i <= m->numInnerFaces; ++i) {
        const int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
        F(s, ijp) = F(s, ijp) - F(a, F(slot_pn, i)) * F(old[comp], ijn);
        F(s, ijn) = F(s, ijn) - F(a, F(slot_np, i)) * F(old[comp], ijp);
      }
      for (int ijp = 1; ijp <= n; ++ijp) {
        const double apotime = F(den, ijp) * F(m->vol, ijp) / prm->timestep;
        const double sum_off = row_sum(ioffset, a, ijp) - F(a, F(diag, ijp));
        F(s, ijp) = F(s, ijp) + (apotime + sum_off) * F(old[comp], ijp);
        F(SP[comp], ijp) = F(SP[comp], ijp) + apotime;
      }
    }
    if (comp > 0)
      for (int inp = 1; inp <= n; ++inp) {
        F(a, F(diag, inp)) = 0.0;
        F(su, inp) = 0.0; /* :473-476: su is the right-hand side of the v and w solves */
      }
    for (int inp = 1; inp <= n; ++inp) {
      const double sum_off = row_sum(ioffset, a, inp) - F(a, F(diag, inp));
      F(a, F(diag, inp)) = F(SP[comp], inp) - sum_off;
      F(a, F(diag, inp)) = F(a, F(diag, inp)) * prm->urfr[comp];
      if (comp == 0)
        F(su, inp) = F(su, inp) + prm->urfm[0] * F(a, F(diag, inp)) * F(u, inp);
      else
        F(su, inp) = F(S[comp], inp) + prm->urfm[comp] * F(a, F(diag, inp)) * F(cur[comp], inp);
      ap[(size_t)comp * n + inp - 1] = (double)1.0f / (F(a, F(diag, inp)) + small);
    }
    for (int inp = 1; inp <= n; ++inp) {
      rhs[(size_t)comp * n + inp - 1] = F(su, inp);
      if (comp == 0)
        du[inp - 1] = F(a, F(diag, inp));
      else
        diag_vw[(size_t)(comp - 1) * n + inp - 1] = F(a, F(diag, inp));
    }
  }
  for (int inp = 1; inp <= n; ++inp) F(a, F(diag, inp)) = du[inp - 1];
  free(su);
  free(sv);
  free(sw);
  free(spu);
  free(spv);
  free(sp);
  free(du);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* PISO pressure path                                                          */
/* ------------------------------------------------------------------------- */

/* get_rAU_x_UEqnH.f90:32-206, loop by loop: su = sv = sw = 0; the cell loop of volume
 * sources (buoyancy :42-56, BDF :62-83, where `0.99` and `0.5` are default-real
 * literals); per component the Crank-Nicolson face loop and cell loop (:90-110), then the
 * H(U) face loop (:113-123); finally u = apu*su on the cells (:204-206). */
int orc_piso_hbya(const orc_mesh *m, const int *ioffset, const int *diag, const int *slot_pn,
                  const int *slot_np, const orc_hbya_params *prm, const double *h,
                  const double *den, const double *t, const double *uo, const double *vo,
                  const double *wo, const double *uoo, const double *voo, const double *woo,
                  const double *apu, const double *apv, const double *apw, double *u, double *v,
                  double *w, double *su, double *sv, double *sw) {
  const int n = m->numCells;
  for (int i = 1; i <= n; ++i) F(su, i) = F(sv, i) = F(sw, i) = 0.0;
  for (int inp = 1; inp <= n; ++inp) {
    if (prm->buoyancy) {
      double heat = 0.0;
      if (prm->boussinesq)
        heat = prm->beta * prm->densit * (F(t, inp) - prm->tref) * F(m->vol, inp);
      else
        heat = (prm->densit - F(den, inp)) * F(m->vol, inp);
      F(su, inp) = F(su, inp) - prm->gravx * heat;
      F(sv, inp) = F(sv, inp) - prm->gravy * heat;
      F(sw, inp) = F(sw, inp) - prm->gravz * heat;
    }
    if (prm->bdf) {
      const double apotime = F(den, inp) * F(m->vol, inp) / prm->timestep;
      double sut = apotime * ((1 + prm->btime) * F(uo, inp));
      double svt = apotime * ((1 + prm->btime) * F(vo, inp));
      double swt = apotime * ((1 + prm->btime) * F(wo, inp));
      if (prm->btime > (double)0.99f) {
        sut = sut - apotime * ((double)0.5f * prm->btime * F(uoo, inp));
        svt = svt - apotime * ((double)0.5f * prm->btime * F(voo, inp));
        swt = swt - apotime * ((double)0.5f * prm->btime * F(woo, inp));
      }
      F(su, inp) = F(su, inp) + sut;
      F(sv, inp) = F(sv, inp) + svt;
      F(sw, inp) = F(sw, inp) + swt;
    }
  }
  double *s[3] = {su, sv, sw};
  const double *cur[3] = {u, v, w}, *old[3] = {uo, vo, wo};
  for (int comp = 0; comp < 3; ++comp) {
    double *S = s[comp];
    if (prm->cn) {
      for (int i = 1; i <= m->numInnerFaces; ++i) {
        const int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
        F(S, ijp) = F(S, ijp) - F(h, F(slot_pn, i)) * F(old[comp], ijn);
        F(S, ijn) = F(S, ijn) - F(h, F(slot_np, i)) * F(old[comp], ijp);
      }
      for (int ijp = 1; ijp <= n; ++ijp) {
        const double apotime = F(den, ijp) * F(m->vol, ijp) / prm->timestep;
        double sum = 0.0; /* sum(h(ioffset(ijp):ioffset(ijp+1)-1)) */
        for (int k = F(ioffset, ijp); k <= F(ioffset, ijp + 1) - 1; ++k) sum = sum + F(h, k);
        const double off_diagonal_terms = sum - F(h, F(diag, ijp));
        F(S, ijp) = F(S, ijp) + (apotime + off_diagonal_terms) * F(old[comp], ijp);
      }
    }
    for (int i = 1; i <= m->numInnerFaces; ++i) {
      const int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
      F(S, ijp) = F(S, ijp) - F(h, F(slot_pn, i)) * F(cur[comp], ijn);
      F(S, ijn) = F(S, ijn) - F(h, F(slot_np, i)) * F(cur[comp], ijp);
    }
  }
  for (int i = 1; i <= n; ++i) {
    F(u, i) = F(apu, i) * F(su, i);
    F(v, i) = F(apv, i) * F(sv, i);
    F(w, i) = F(apw, i) * F(sw, i);
  }
  return 0;
}

/* PISO_multiple_correction.f90:109-148 with facefluxmass_piso (facefluxmass.f90:294-358). */
/* facefluxmass_piso, facefluxmass.f90:294-358, on the face between ijp and ijn (centre,
 * area, factor): cap, can and the face mass flux. */
static void ffp_face(const orc_mesh *m, int ijp, int ijn, double xf, double yf, double zf,
                     double arx, double ary, double arz, double lambda, const double *u,
                     const double *v, const double *w, const double *dUdxi,
                     const double *dVdxi, const double *dWdxi, const double *apu,
                     const double *den, double *cap_out, double *can_out, double *fm_out) {
  const double fxn = lambda;
  const double fxp = 1.0 - fxn;
  const double xpn = F(m->xc, ijn) - F(m->xc, ijp);
  const double ypn = F(m->yc, ijn) - F(m->yc, ijp);
  const double zpn = F(m->zc, ijn) - F(m->zc, ijp);
  const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
  const double are = sqrt(arx * arx + ary * ary + arz * arz);
  const double dene = F(den, ijp) * fxp + F(den, ijn) * fxn;
  const double cap = -(dene *
                       (fxp * F(m->vol, ijp) * F(apu, ijp) + fxn * F(m->vol, ijn) * F(apu, ijn)) *
                       are / dpn);
  const double ui = face_value_central(m, ijp, ijn, xf, yf, zf, u, dUdxi);
  const double vi = face_value_central(m, ijp, ijn, xf, yf, zf, v, dVdxi);
  const double wi = face_value_central(m, ijp, ijn, xf, yf, zf, w, dWdxi);
  *cap_out = cap;
  *can_out = cap;
  *fm_out = dene * (ui * arx + vi * ary + wi * arz);
}

/* PISO :109-174; with O-C pairs a holds ar, al after the CSR values and flmass the
 * pairs' fmoc after the inner faces' fluxes. */
int orc_facefluxmass_piso(const orc_mesh *m, const int *diag, const int *slot_pn,
                          const int *slot_np, const double *u, const double *v, const double *w,
                          const double *dUdxi, const double *dVdxi, const double *dWdxi,
                          const double *apu, const double *den, int nnz, double *a, double *su,
                          double *flmass) {
  for (int k = 0; k < nnz; ++k) a[k] = 0.0;          /* :109 */
  for (int i = 0; i < m->numCells; ++i) su[i] = 0.0; /* :110 */
  for (int i = 1; i <= m->numInnerFaces; ++i) {
    const int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    double cap, can, fm;
    ffp_face(m, ijp, ijn, F(m->xf, i), F(m->yf, i), F(m->zf, i), F(m->arx, i), F(m->ary, i),
             F(m->arz, i), F(m->facint, i), u, v, w, dUdxi, dVdxi, dWdxi, apu, den, &cap, &can,
             &fm);
    F(flmass, i) = fm;
    F(a, F(slot_pn, i)) = can;
    F(a, F(slot_np, i)) = cap;
    F(a, F(diag, ijp)) = F(a, F(diag, ijp)) - can;
    F(a, F(diag, ijn)) = F(a, F(diag, ijn)) - cap;
    F(su, ijp) = F(su, ijp) - fm;
    F(su, ijn) = F(su, ijn) + fm;
  }
  if (m->noc > 0) { /* O- and C-grid cuts (:151-174) */
    oc_pairs oc;
    if (get_oc(m, &oc)) return -1;
    double *ar = a + nnz, *al = a + nnz + m->noc, *fmoc = flmass + m->numInnerFaces;
    for (int i = 1; i <= m->noc; ++i) {
      int iface = F(m->ijlFace, i), ijp = F(oc.ijl, i), ijn = F(oc.ijr, i);
      ffp_face(m, ijp, ijn, F(m->xf, iface), F(m->yf, iface), F(m->zf, iface),
               F(m->arx, iface), F(m->ary, iface), F(m->arz, iface), F(oc.foc, i), u, v, w,
               dUdxi, dVdxi, dWdxi, apu, den, &F(al, i), &F(ar, i), &F(fmoc, i));
      F(a, F(diag, ijp)) = F(a, F(diag, ijp)) - F(ar, i);
      F(a, F(diag, ijn)) = F(a, F(diag, ijn)) - F(al, i);
      F(su, ijp) = F(su, ijp) - F(fmoc, i);
      F(su, ijn) = F(su, ijn) + F(fmoc, i);
    }
    free_oc(&oc);
  }
  return 0;
}

/* adjustMassFlow.f90:15-69. */
int orc_adjust_mass_flow(const orc_mesh *m, const double *den, double flomas, const double *fmi,
                         double *u, double *v, double *w, double *fmo, double *su) {
  const double small = orc_const_small_src();
  for (int i = 1; i <= m->ninl; ++i) {
    const int ijp = F(m->owner, m->iInletFacesStart + i);
    F(su, ijp) = F(su, ijp) - F(fmi, i);
  }
  double flowo = 0.0;
  for (int i = 1; i <= m->nout; ++i) {
    const int iface = m->iOutletFacesStart + i, ijp = F(m->owner, iface);
    const int ijb = iOutletStart(m) + i;
    F(u, ijb) = F(u, ijp);
    F(v, ijb) = F(v, ijp);
    F(w, ijb) = F(w, ijp);
    F(fmo, i) = F(den, ijp) * (F(u, ijb) * F(m->arx, iface) + F(v, ijb) * F(m->ary, iface) +
                               F(w, ijb) * F(m->arz, iface));
    flowo = flowo + F(fmo, i);
  }
  const double fac = flomas / (flowo + small);
  for (int i = 1; i <= m->nout; ++i) {
    const int iface = m->iOutletFacesStart + i, ijp = F(m->owner, iface);
    const int ijb = iOutletStart(m) + i;
    F(fmo, i) = F(fmo, i) * fac;
    F(u, ijb) = F(u, ijb) * fac;
    F(v, ijb) = F(v, ijb) * fac;
    F(w, ijb) = F(w, ijb) * fac;
    F(su, ijp) = F(su, ijp) - F(fmo, i);
  }
  return 0;
}

/* PISO_multiple_correction.f90:188-192. */
int orc_set_reference_pressure(const int *ioffset, const int *diag, int pRefCell,
                               const double *p, double *a, double *su) {
  for (int k = F(ioffset, pRefCell); k <= F(ioffset, pRefCell + 1) - 1; ++k) F(a, k) = 0.0;
  F(a, F(diag, pRefCell)) = 1.0;
  F(su, pRefCell) = F(p, pRefCell);
  return 0;
}

/* PISO_multiple_correction.f90:300-304. */
int orc_correct_velocity_piso(const orc_mesh *m, const double *dPdxi, const double *apu,
                              const double *apv, const double *apw, double *u, double *v,
                              double *w) {
  for (int inp = 1; inp <= m->numCells; ++inp) {
    F(u, inp) = F(u, inp) - F(apu, inp) * G3(dPdxi, 1, inp) * F(m->vol, inp);
    F(v, inp) = F(v, inp) - F(apv, inp) * G3(dPdxi, 2, inp) * F(m->vol, inp);
    F(w, inp) = F(w, inp) - F(apw, inp) * G3(dPdxi, 3, inp) * F(m->vol, inp);
  }
  return 0;
}

/* calcp-multiple_correction_SIMPLE.f90:184-189: velocity and pressure correction,
 * ppref = pp(pRefCell) (:147). */
int orc_correct_fields(const orc_mesh *m, const double *dPdxi, const double *apu,
                       const double *apv, const double *apw, const double *pp, double urf,
                       int pRefCell, double *u, double *v, double *w, double *p) {
  const double ppref = pp[pRefCell - 1];
  for (int inp = 0; inp < m->numCells; ++inp) {
    u[inp] = u[inp] - dPdxi[3 * inp] * m->vol[inp] * apu[inp];
    v[inp] = v[inp] - dPdxi[3 * inp + 1] * m->vol[inp] * apv[inp];
    w[inp] = w[inp] - dPdxi[3 * inp + 2] * m->vol[inp] * apw[inp];
    p[inp] = p[inp] + urf * (pp[inp] - ppref);
  }
  return 0;
}

/* correctBoundaryConditionsVelocity.f90:1-80: outlet slots take their cell's velocity,
 * fmo(i) = den(ijp) (u,v,w)(ijb).S, flowo = sum fmo, fac = flomas/(flowo+small), then
 * fmo and the outlet velocities are scaled by fac; symmetry slots take the cell velocity
 * minus Unmag S with Unmag = (u,v,w)(ijp).S (the area vector, as the reference does). */
int orc_correct_bc_velocity(const orc_mesh *m, const double *den, double flomas, double *u,
                            double *v, double *w, double *fmo) {
  const double small = orc_const_small_src();
  double flowo = 0.0;
  for (int i = 1; i <= m->nout; ++i) {
    const int iface = m->iOutletFacesStart + i, ijp = F(m->owner, iface);
    const int ijb = iOutletStart(m) + i;
    F(u, ijb) = F(u, ijp);
    F(v, ijb) = F(v, ijp);
    F(w, ijb) = F(w, ijp);
    F(fmo, i) = F(den, ijp) * (F(u, ijb) * F(m->arx, iface) + F(v, ijb) * F(m->ary, iface) +
                               F(w, ijb) * F(m->arz, iface));
    flowo = flowo + F(fmo, i);
  }
  const double fac = flomas / (flowo + small);
  for (int i = 1; i <= m->nout; ++i) {
    const int ijb = iOutletStart(m) + i;
    F(fmo, i) = F(fmo, i) * fac;
    F(u, ijb) = F(u, ijb) * fac;
    F(v, ijb) = F(v, ijb) * fac;
    F(w, ijb) = F(w, ijb) * fac;
  }
  for (int i = 1; i <= m->nsym; ++i) {
    const int iface = m->iSymmetryFacesStart + i, ijp = F(m->owner, iface);
    const int ijb = iSymmetryStart(m) + i;
    const double unmag = F(u, ijp) * F(m->arx, iface) + F(v, ijp) * F(m->ary, iface) +
                         F(w, ijp) * F(m->arz, iface);
    F(u, ijb) = F(u, ijp) - unmag * F(m->arx, iface);
    F(v, ijb) = F(v, ijp) - unmag * F(m->ary, iface);
    F(w, ijb) = F(w, ijp) - unmag * F(m->arz, iface);
  }
  return 0;
}

/* continuityErrors.h:1-52: res = 0; per inner face res(ijp) -= flmass(ijp),
 * res(ijn) += flmass(ijp) -- the reference indexes flmass by the owner CELL here, which
 * is kept; then res(owner) -= fmi(i) over inlet faces and -= fmo(i) over outlet faces;
 * sumLocalContErr = sum|res|, globalContErr = sum res (in cell order). */
int orc_continuity_errors(const orc_mesh *m, const double *flmass, const double *fmi,
                          const double *fmo, double *res, double *sum_local, double *global) {
  if (m->numCells > m->numInnerFaces) return -4;
  for (int i = 1; i <= m->numCells; ++i) F(res, i) = 0.0;
  for (int i = 1; i <= m->numInnerFaces; ++i) {
    const int ijp = F(m->owner, i), ijn = F(m->neighbour, i);
    F(res, ijp) = F(res, ijp) - F(flmass, ijp);
    F(res, ijn) = F(res, ijn) + F(flmass, ijp);
  }
  if (m->noc > 0) { /* faces along O-C grid cuts (continuityErrors.h:22-28) */
    oc_pairs oc;
    if (get_oc(m, &oc)) return -1;
    const double *fmoc = flmass + m->numInnerFaces;
    for (int i = 1; i <= m->noc; ++i) {
      F(res, F(oc.ijl, i)) = F(res, F(oc.ijl, i)) - F(fmoc, i);
      F(res, F(oc.ijr, i)) = F(res, F(oc.ijr, i)) + F(fmoc, i);
    }
    free_oc(&oc);
  }
  for (int i = 1; i <= m->ninl; ++i) {
    const int ijp = F(m->owner, m->iInletFacesStart + i);
    F(res, ijp) = F(res, ijp) - F(fmi, i);
  }
  for (int i = 1; i <= m->nout; ++i) {
    const int ijp = F(m->owner, m->iOutletFacesStart + i);
    F(res, ijp) = F(res, ijp) - F(fmo, i);
  }
  double sl = 0.0, sg = 0.0;
  for (int i = 1; i <= m->numCells; ++i) {
    sl = sl + fabs(F(res, i));
    sg = sg + F(res, i);
  }
  *sum_local = sl;
  *global = sg;
  return 0;
}
