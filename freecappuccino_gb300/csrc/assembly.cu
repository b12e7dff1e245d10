// Face-loop assembly kernels: laplacian (fvm_laplacian.f90), the pressure-correction
// coefficients and Rhie-Chow fluxes of calcp/facefluxmass (facefluxmass.f90:34-199)
// and the non-orthogonal corrector source of fluxmc (facefluxmass.f90:520-607).
//
// Each assembly is two kernels and uses no atomics:
//   1. one thread per inner face computes the face's coefficient and flux and writes
//      the two off-diagonal CSR slots (each slot belongs to exactly one face) and, where
//      a per-cell sum follows, a face array;
//   2. one thread per cell gathers its faces through the cell->face incidence list,
//      which holds the faces in the Fortran loop's order, so the diagonal and the
//      source are summed term by term exactly as the reference sums them.
// This file is compiled with --fmad=false: every a*b+c below is a rounded multiply
// followed by a rounded add, as gfortran evaluates it, so the coefficients are
// bit-identical to the reference's loop on the same inputs.
#include <algorithm>

#include "face_geo.h"
#include "fcg_internal.h"
#include "launch.h"

using namespace fcg;

namespace {

// ---------------------------------------------------------------------------
// The face factors (face_geo.h).
// ---------------------------------------------------------------------------
__global__ void k_face_geo(MeshView m, double *__restrict__ g) {
  const long long nin = m.nin;
  FCG_GRID_STRIDE(f, nin) {
    const int p = m.owner[f], q = m.neighbour[f];
    const double xf = m.xf[f], yf = m.yf[f], zf = m.zf[f];
    const double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
    const double xpn = m.xc[q] - m.xc[p], ypn = m.yc[q] - m.yc[p], zpn = m.zc[q] - m.zc[p];
    const double are = sqrt(arx * arx + ary * ary + arz * arz);
    const double nxx = arx / are, nyy = ary / are, nzz = arz / are;
    const double sfdpnr = 1.0 / (arx * xpn * nxx + ary * ypn * nyy + arz * zpn * nzz);
    double xpp = xf - (xf - m.xc[p]) * nxx, ypp = yf - (yf - m.yc[p]) * nyy,
           zpp = zf - (zf - m.zc[p]) * nzz;
    double xep = xf - (xf - m.xc[q]) * nxx, yep = yf - (yf - m.yc[q]) * nyy,
           zep = zf - (zf - m.zc[q]) * nzz;
    xpp = xpp - m.xc[p];
    ypp = ypp - m.yc[p];
    zpp = zpp - m.zc[p];
    xep = xep - m.xc[q];
    yep = yep - m.yc[q];
    zep = zep - m.zc[q];
    // sngrad's arx / vole with vole = xpn arx + ypn ary + zpn arz (gradients.f90:644, 666)
    const double vole = xpn * arx + ypn * ary + zpn * arz;
    // presFaceDivInner's interpolated centre xi = xc(P) fxp + xc(N) fxn
    // (fieldManipulation.f90:429-431)
    const double fxn = m.facint[f], fxp = 1.0 - fxn;
    const double xi = m.xc[p] * fxp + m.xc[q] * fxn, yi = m.yc[p] * fxp + m.yc[q] * fxn,
                 zi = m.zc[p] * fxp + m.zc[q] * fxn;
    const double v[FG_COUNT] = {
        nxx, nyy, nzz, sfdpnr, (arx * arx + ary * ary + arz * arz) * sfdpnr,
        1.0 / ((xpn * nxx) + (ypn * nyy) + (zpn * nzz)), xpp, ypp, zpp, xep, yep, zep,
        xf - m.xc[p], yf - m.yc[p], zf - m.zc[p], xf - m.xc[q], yf - m.yc[q], zf - m.zc[q],
        xpn, ypn, zpn, are,
        (arx * arx + ary * ary + arz * arz) / (arx * xpn + ary * ypn + arz * zpn),
        sqrt(xpn * xpn + ypn * ypn + zpn * zpn), arx / vole, ary / vole, arz / vole,
        xf - xi, yf - yi, zf - zi};
#pragma unroll
    for (int k = 0; k < FG_COUNT; ++k) g[k * nin + f] = v[k];
  }
}

// Boundary-face factors (face_geo.h), one thread per cell over its boundary entries.
__global__ void k_bnd_geo(MeshView m, long long ncb, double *__restrict__ b) {
  FCG_GRID_STRIDE(c, m.n) {
    for (int e = m.cb_ptr[c]; e < m.cb_ptr[c + 1]; ++e) {
      const int f = m.cb_face[e];
      const double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
      const double are = sqrt(arx * arx + ary * ary + arz * arz);
      const double nxf = arx / are, nyf = ary / are, nzf = arz / are;
      const double dn = (m.xf[f] - m.xc[c]) * nxf + (m.yf[f] - m.yc[c]) * nyf +
                        (m.zf[f] - m.zc[c]) * nzf;
      const double dx = m.xc[c] - m.xf[f], dy = m.yc[c] - m.yf[f], dz = m.zc[c] - m.zf[f];
      b[BG_ARE * ncb + e] = are;
      b[BG_DPB * ncb + e] = sqrt(dx * dx + dy * dy + dz * dz);
      b[BG_NX * ncb + e] = nxf;
      b[BG_NY * ncb + e] = nyf;
      b[BG_NZ * ncb + e] = nzf;
      b[BG_SRD * ncb + e] = are / dn;
    }
  }
}

// foc and srdoc of the O-C and cyclic pairs (mesh_geometry_and_topology.f90:1083-1152):
// the distances of the left cell's centre to its face (djn) and of the right cell's
// centre to the friend face (dpn); a cyclic pair takes foc = 1/2 (:1149).
__global__ void k_oc_geo(MeshView m, double *__restrict__ foc, double *__restrict__ srdoc) {
  const int nreg = m.noc - m.ncyc;
  FCG_GRID_STRIDE(i, m.noc) {
    const int f = m.oc_fl[i], g = m.oc_fr[i], p = m.oc_l[i], q = m.oc_r[i];
    double xpn = m.xc[q] - m.xf[g], ypn = m.yc[q] - m.yf[g], zpn = m.zc[q] - m.zf[g];
    const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    xpn = m.xf[f] - m.xc[p];
    ypn = m.yf[f] - m.yc[p];
    zpn = m.zf[f] - m.zc[p];
    const double djn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    foc[i] = (int)i < nreg ? djn / (djn + dpn) : 0.5;
    const double are = sqrt(m.arx[f] * m.arx[f] + m.ary[f] * m.ary[f] + m.arz[f] * m.arz[f]);
    srdoc[i] = are / (djn + dpn);
  }
}

}  // namespace

int fcg::oc_geometry(fcg_context *c) {
  MeshView &m = c->mv;
  c->bound_allocs.emplace_back();
  DBuf &b = c->bound_allocs.back();
  FCG_CUDA_TRY(c, b.ensure(2 * sizeof(double) * (size_t)m.noc));
  double *foc = b.as<double>(), *srdoc = foc + m.noc;
  k_oc_geo<<<grid_for(m.noc, c->num_sms), kTPB, 0, c->stream>>>(m, foc, srdoc);
  FCG_CHECK_LAUNCH(c, "k_oc_geo");
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  m.oc_foc = foc;
  m.oc_srdoc = srdoc;
  return FCG_OK;
}

namespace {

// ---------------------------------------------------------------------------
// laplacian(mu,phi)
// ---------------------------------------------------------------------------
__global__ void k_lap_faces(MeshView m, const double *__restrict__ g, const double *__restrict__ mu,
                            double *__restrict__ a) {
  const long long nin = m.nin;
  FCG_GRID_STRIDE(f, nin) {
    int p = m.owner[f], q = m.neighbour[f];
    double fxn = m.facint[f];  // facefluxlaplacian :195-196
    double fxp = 1.0 - fxn;
    double smdpn = g[FG_SMDPN_LAP * nin + f];  // :214
    double cap = (fxp * mu[p] + fxn * mu[q]) * smdpn;  // :218, can = cap
    a[m.slot_pn[f]] = cap;                              // :48-49
    a[m.slot_np[f]] = cap;                              // :52-53
  }
}

// The O-C pairs (:67-86): facefluxlaplacian(ijl, ijr, area of face iOCFacesStart + i,
// foc(i), mu, al(i), ar(i)), ar and al stored after the CSR values of a.
__global__ void k_lap_oc(MeshView m, const double *__restrict__ mu, double *__restrict__ a) {
  FCG_GRID_STRIDE(i, m.noc) {
    const int p = m.oc_l[i], q = m.oc_r[i], f = m.oc_start + (int)i;
    const double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
    const double fxn = m.oc_foc[i];
    const double fxp = 1.0 - fxn;
    const double xpn = m.xc[q] - m.xc[p], ypn = m.yc[q] - m.yc[p], zpn = m.zc[q] - m.zc[p];
    const double smdpn = (arx * arx + ary * ary + arz * arz) / (arx * xpn + ary * ypn + arz * zpn);
    const double cap = (fxp * mu[p] + fxn * mu[q]) * smdpn;
    a[m.nnz + i] = cap;          // ar(i) = can
    a[m.nnz + m.noc + i] = cap;  // al(i) = cap
  }
}

__global__ void k_lap_cells(MeshView m, const double *__restrict__ mu,
                            const double *__restrict__ phi, double *__restrict__ a,
                            double *__restrict__ su) {
  FCG_GRID_STRIDE(c, m.n) {
    double acc = 0.0;  // a = 0 (:33), then a(diag) -= can/cap in face order (:58-63)
    for (int e = m.cf_ptr[c]; e < m.cf_ptr[c + 1]; ++e) acc = acc - a[m.cf_slot[e]];
    if (m.noc)  // then ar / al of the cell's O-C pairs in pair order (:79-84)
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) acc = acc - a[m.nnz + m.oc_vix[e]];
    double s = su[c];
    for (int e = m.cb_ptr[c]; e < m.cb_ptr[c + 1]; ++e) {  // wall faces :140-154
      if (m.cb_type[e] != B_WALL) continue;
      int f = m.cb_face[e];
      double are = sqrt(m.arx[f] * m.arx[f] + m.ary[f] * m.ary[f] + m.arz[f] * m.arz[f]);
      double dx = m.xc[c] - m.xf[f], dy = m.yc[c] - m.yf[f], dz = m.zc[c] - m.zf[f];
      double dpw = sqrt(dx * dx + dy * dy + dz * dz);
      acc = acc - mu[c] * are / dpw;
      s = s + acc * phi[m.cb_slot[e]];
    }
    a[m.diag[c]] = acc;
    su[c] = s;
  }
}

// ---------------------------------------------------------------------------
// facefluxmass inside calcp :45-77
// ---------------------------------------------------------------------------
struct FlowView {
  const double *u, *v, *w, *p, *dU, *dV, *dW, *dP, *apu, *apv, *apw, *den;
};

// face_value_central, interpolation.f90:145-199, with the face centre's offsets from P
// (dxp..) and N (dxq..)
__device__ __forceinline__ double face_value_central(int p, int q, double dxp, double dyp,
                                                     double dzp, double dxq, double dyq,
                                                     double dzq, const double *__restrict__ fi,
                                                     const double *__restrict__ g) {
  double gradfidr = g[3 * p] * dxp + g[3 * p + 1] * dyp + g[3 * p + 2] * dzp + g[3 * q] * dxq +
                    g[3 * q + 1] * dyq + g[3 * q + 2] * dzq;
  return 0.5 * (fi[p] + fi[q] + gradfidr);
}

__global__ void k_ffm_faces(MeshView m, const double *__restrict__ g, FlowView fl,
                            double *__restrict__ a, double *__restrict__ flmass) {
  const long long nin = m.nin;
  FCG_GRID_STRIDE(f, nin) {
    int p = m.owner[f], q = m.neighbour[f];
    double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
    double fxn = m.facint[f];
    double fxp = 1.0 - fxn;
    const double xpn = g[FG_XPN * nin + f], ypn = g[FG_YPN * nin + f], zpn = g[FG_ZPN * nin + f];
    const double nxx = g[FG_NX * nin + f], nyy = g[FG_NY * nin + f], nzz = g[FG_NZ * nin + f];
    double Dpu = fxn * m.vol[q] * fl.apu[q] + fxp * m.vol[p] * fl.apu[p];  // :86-88
    double Dpv = fxn * m.vol[q] * fl.apv[q] + fxp * m.vol[p] * fl.apv[p];
    double Dpw = fxn * m.vol[q] * fl.apw[q] + fxp * m.vol[p] * fl.apw[p];
    double dene = fl.den[p] * fxp + fl.den[q] * fxn;
    const double sfdpnr = g[FG_SFDPNR * nin + f];  // :94
    const double smdpn = g[FG_SMDPN * nin + f];
    double cap = -(dene * Dpu * smdpn);  // :96, can = cap
    const double dxp = g[FG_DXP * nin + f], dyp = g[FG_DYP * nin + f], dzp = g[FG_DZP * nin + f];
    const double dxq = g[FG_DXQ * nin + f], dyq = g[FG_DYQ * nin + f], dzq = g[FG_DZQ * nin + f];
    double ui = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.u, fl.dU);
    double vi = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.v, fl.dV);
    double wi = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.w, fl.dW);
    const double *dP = fl.dP;
    double dpxi = Dpu * (fxn * dP[3 * q] + fxp * dP[3 * p]) * xpn * nxx;  // :145-147
    double dpyi = Dpv * (fxn * dP[3 * q + 1] + fxp * dP[3 * p + 1]) * ypn * nyy;
    double dpzi = Dpw * (fxn * dP[3 * q + 2] + fxp * dP[3 * p + 2]) * zpn * nzz;
    const double xpp = g[FG_XPP * nin + f], ypp = g[FG_YPP * nin + f], zpp = g[FG_ZPP * nin + f];
    const double xep = g[FG_XEP * nin + f], yep = g[FG_YEP * nin + f], zep = g[FG_ZEP * nin + f];
    double dpe = fl.p[q] - fl.p[p];
    // :174-175 as written: only the first owner term carries the minus sign.
    double dpecorr = dP[3 * q] * xep + dP[3 * q + 1] * yep + dP[3 * q + 2] * zep - dP[3 * p] * xpp +
                     dP[3 * p + 1] * ypp + dP[3 * p + 2] * zpp;
    dpe = dpe + dpecorr;
    double dpex = Dpu * dpe * sfdpnr * arx, dpey = Dpv * dpe * sfdpnr * ary,
           dpez = Dpw * dpe * sfdpnr * arz;
    double ue = ui - dpex + dpxi, ve = vi - dpey + dpyi, we = wi - dpez + dpzi;
    flmass[f] = dene * (ue * arx + ve * ary + we * arz);  // :185
    a[m.slot_pn[f]] = cap;
    a[m.slot_np[f]] = cap;
  }
}

// facefluxmass.f90:34-199 on the face between p and q with centre (xf, yf, zf), area
// (arx, ary, arz) and factor lambda, computed in place (the O-C pairs have no cached face
// factors): cap, can and the mass flux, with the operations of k_ffm_faces and the
// factors k_face_geo caches.
__device__ void ffm_face(const MeshView &m, const FlowView &fl, int p, int q, double xf,
                         double yf, double zf, double arx, double ary, double arz,
                         double lambda, double &cap, double &can, double &fm) {
  double fxn = lambda;
  double fxp = 1.0 - fxn;
  double xpn = m.xc[q] - m.xc[p], ypn = m.yc[q] - m.yc[p], zpn = m.zc[q] - m.zc[p];
  double are = sqrt(arx * arx + ary * ary + arz * arz);
  double nxx = arx / are, nyy = ary / are, nzz = arz / are;
  double Dpu = fxn * m.vol[q] * fl.apu[q] + fxp * m.vol[p] * fl.apu[p];
  double Dpv = fxn * m.vol[q] * fl.apv[q] + fxp * m.vol[p] * fl.apv[p];
  double Dpw = fxn * m.vol[q] * fl.apw[q] + fxp * m.vol[p] * fl.apw[p];
  double dene = fl.den[p] * fxp + fl.den[q] * fxn;
  double sfdpnr = 1.0 / (arx * xpn * nxx + ary * ypn * nyy + arz * zpn * nzz);
  double smdpn = (arx * arx + ary * ary + arz * arz) * sfdpnr;
  cap = -(dene * Dpu * smdpn);
  can = cap;
  const double dxp = xf - m.xc[p], dyp = yf - m.yc[p], dzp = zf - m.zc[p];
  const double dxq = xf - m.xc[q], dyq = yf - m.yc[q], dzq = zf - m.zc[q];
  double ui = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.u, fl.dU);
  double vi = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.v, fl.dV);
  double wi = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.w, fl.dW);
  const double *dP = fl.dP;
  double dpxi = Dpu * (fxn * dP[3 * q] + fxp * dP[3 * p]) * xpn * nxx;
  double dpyi = Dpv * (fxn * dP[3 * q + 1] + fxp * dP[3 * p + 1]) * ypn * nyy;
  double dpzi = Dpw * (fxn * dP[3 * q + 2] + fxp * dP[3 * p + 2]) * zpn * nzz;
  double xpp = xf - (xf - m.xc[p]) * nxx, ypp = yf - (yf - m.yc[p]) * nyy;
  double zpp = zf - (zf - m.zc[p]) * nzz;
  double xep = xf - (xf - m.xc[q]) * nxx, yep = yf - (yf - m.yc[q]) * nyy;
  double zep = zf - (zf - m.zc[q]) * nzz;
  xpp = xpp - m.xc[p];
  ypp = ypp - m.yc[p];
  zpp = zpp - m.zc[p];
  xep = xep - m.xc[q];
  yep = yep - m.yc[q];
  zep = zep - m.zc[q];
  double dpe = fl.p[q] - fl.p[p];
  // :174-175 as written: only the first owner term carries the minus sign.
  double dpecorr = dP[3 * q] * xep + dP[3 * q + 1] * yep + dP[3 * q + 2] * zep - dP[3 * p] * xpp +
                   dP[3 * p + 1] * ypp + dP[3 * p + 2] * zpp;
  dpe = dpe + dpecorr;
  double dpex = Dpu * dpe * sfdpnr * arx, dpey = Dpv * dpe * sfdpnr * ary,
         dpez = Dpw * dpe * sfdpnr * arz;
  double ue = ui - dpex + dpxi, ve = vi - dpey + dpyi, we = wi - dpez + dpzi;
  fm = dene * (ue * arx + ve * ary + we * arz);
}

// The O-C pairs (calcp :81-100): facefluxmass on face ijlFace(i) with foc(i); al(i) = cap,
// ar(i) = can after the CSR values of a, fmoc(i) after the inner faces' fluxes.
__global__ void k_ffm_oc(MeshView m, FlowView fl, double *__restrict__ a,
                         double *__restrict__ flmass) {
  FCG_GRID_STRIDE(i, m.noc) {
    const int f = m.oc_fl[i];
    double cap, can, fm;
    ffm_face(m, fl, m.oc_l[i], m.oc_r[i], m.xf[f], m.yf[f], m.zf[f], m.arx[f], m.ary[f],
             m.arz[f], m.oc_foc[i], cap, can, fm);
    a[m.nnz + m.noc + i] = cap;
    a[m.nnz + i] = can;
    flmass[m.nin + i] = fm;
  }
}

// The O-C pairs of the PISO assembly (PISO_multiple_correction.f90:151-174):
// facefluxmass_piso (facefluxmass.f90:294-358) on face ijlFace(i) with foc(i), computed in
// place with the operations of k_ffp_faces.
__global__ void k_ffp_oc(MeshView m, FlowView fl, double *__restrict__ a,
                         double *__restrict__ flmass) {
  FCG_GRID_STRIDE(i, m.noc) {
    const int p = m.oc_l[i], q = m.oc_r[i], f = m.oc_fl[i];
    const double xf = m.xf[f], yf = m.yf[f], zf = m.zf[f];
    const double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
    const double fxn = m.oc_foc[i];
    const double fxp = 1.0 - fxn;
    const double xpn = m.xc[q] - m.xc[p], ypn = m.yc[q] - m.yc[p], zpn = m.zc[q] - m.zc[p];
    const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    const double are = sqrt(arx * arx + ary * ary + arz * arz);
    const double dene = fl.den[p] * fxp + fl.den[q] * fxn;
    const double cap =
        -(dene * (fxp * m.vol[p] * fl.apu[p] + fxn * m.vol[q] * fl.apu[q]) * are / dpn);
    const double dxp = xf - m.xc[p], dyp = yf - m.yc[p], dzp = zf - m.zc[p];
    const double dxq = xf - m.xc[q], dyq = yf - m.yc[q], dzq = zf - m.zc[q];
    const double ui = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.u, fl.dU);
    const double vi = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.v, fl.dV);
    const double wi = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.w, fl.dW);
    a[m.nnz + m.noc + i] = cap;  // al = cap
    a[m.nnz + i] = cap;          // ar = can = cap
    flmass[m.nin + i] = dene * (ui * arx + vi * ary + wi * arz);
  }
}

// Diagonal from the cell's own off-diagonal slots and su from the face fluxes, both in
// face order (calcp :65-75), then the cell's O-C pairs in pair order (:89-99): ar / al
// off the diagonal and fmoc off / onto su.
__global__ void k_ffm_cells(MeshView m, const double *__restrict__ flmass, double *__restrict__ a,
                            double *__restrict__ su) {
  FCG_GRID_STRIDE(c, m.n) {
    double acc = 0.0, s = 0.0;
    for (int e = m.cf_ptr[c]; e < m.cf_ptr[c + 1]; ++e) {
      int ent = m.cf_ent[e];
      acc = acc - a[m.cf_slot[e]];
      double fm = flmass[(ent > 0 ? ent : -ent) - 1];
      s = ent > 0 ? s - fm : s + fm;
    }
    if (m.noc)
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) {
        const int v = m.oc_vix[e];
        acc = acc - a[m.nnz + v];
        const double fm = flmass[m.nin + (v < m.noc ? v : v - m.noc)];
        s = v < m.noc ? s - fm : s + fm;
      }
    a[m.diag[c]] = acc;
    su[c] = s;
  }
}

// ---------------------------------------------------------------------------
// facefluxmass_piso inside the PISO corrector (PISO_multiple_correction.f90:116-148)
// ---------------------------------------------------------------------------
__global__ void k_ffp_faces(MeshView m, const double *__restrict__ g, FlowView fl,
                            double *__restrict__ a, double *__restrict__ flmass) {
  const long long nin = m.nin;
  FCG_GRID_STRIDE(f, nin) {
    int p = m.owner[f], q = m.neighbour[f];
    double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
    double fxn = m.facint[f];  // facefluxmass.f90:325-326
    double fxp = 1.0 - fxn;
    const double dpn = g[FG_DPN * nin + f];  // :334
    const double are = g[FG_ARE * nin + f];  // :337
    double dene = fl.den[p] * fxp + fl.den[q] * fxn;       // :340
    // :343, cap = -dene*(...)*are/dpn; can = cap
    double cap =
        -(dene * (fxp * m.vol[p] * fl.apu[p] + fxn * m.vol[q] * fl.apu[q]) * are / dpn);
    const double dxp = g[FG_DXP * nin + f], dyp = g[FG_DYP * nin + f], dzp = g[FG_DZP * nin + f];
    const double dxq = g[FG_DXQ * nin + f], dyq = g[FG_DYQ * nin + f], dzq = g[FG_DZQ * nin + f];
    double ui = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.u, fl.dU);  // :349-351
    double vi = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.v, fl.dV);
    double wi = face_value_central(p, q, dxp, dyp, dzp, dxq, dyq, dzq, fl.w, fl.dW);
    flmass[f] = dene * (ui * arx + vi * ary + wi * arz);  // :356
    a[m.slot_pn[f]] = cap;                                // PISO :126-131
    a[m.slot_np[f]] = cap;
  }
}

// ---------------------------------------------------------------------------
// fluxmc inside calcp :193-206
// ---------------------------------------------------------------------------
__global__ void k_fmc_faces(MeshView m, const double *__restrict__ g, const double *__restrict__ dP,
                            const double *__restrict__ apu, const double *__restrict__ den,
                            double *__restrict__ flmass, double *__restrict__ fmcor_out) {
  const long long nin = m.nin;
  FCG_GRID_STRIDE(f, nin) {
    int p = m.owner[f], q = m.neighbour[f];
    double fxn = m.facint[f];
    double fxp = 1.0 - fxn;
    const double are = g[FG_ARE * nin + f];
    const double dppnnr = g[FG_DPPNNR * nin + f];  // :578
    const double xpp = g[FG_XPP * nin + f], ypp = g[FG_YPP * nin + f], zpp = g[FG_ZPP * nin + f];
    const double xep = g[FG_XEP * nin + f], yep = g[FG_YEP * nin + f], zep = g[FG_ZEP * nin + f];
    double rapr = apu[p] * den[p] * m.vol[p] * fxp + apu[q] * den[q] * m.vol[q] * fxn;  // :599
    double fmcor = rapr * are *
                   ((dP[3 * q] * xep - dP[3 * p] * xpp) + (dP[3 * q + 1] * yep - dP[3 * p + 1] * ypp) +
                    (dP[3 * q + 2] * zep - dP[3 * p + 2] * zpp)) *
                   dppnnr;  // :603-605
    flmass[f] = flmass[f] + fmcor;  // calcp :201
    fmcor_out[f] = fmcor;
  }
}

// fluxmc (facefluxmass.f90:520-607) on the O-C pairs (calcp :206-215), computed in place
// with the operations of k_fmc_faces and the factors k_face_geo caches: fmoc(i) += fmcor,
// and fmcor kept after the inner faces' for the cells' sums.
__global__ void k_fmc_oc(MeshView m, const double *__restrict__ dP, const double *__restrict__ apu,
                         const double *__restrict__ den, double *__restrict__ flmass,
                         double *__restrict__ fmcor_out) {
  FCG_GRID_STRIDE(i, m.noc) {
    const int p = m.oc_l[i], q = m.oc_r[i], f = m.oc_fl[i];
    const double xf = m.xf[f], yf = m.yf[f], zf = m.zf[f];
    const double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
    double fxn = m.oc_foc[i];
    double fxp = 1.0 - fxn;
    double xpn = m.xc[q] - m.xc[p], ypn = m.yc[q] - m.yc[p], zpn = m.zc[q] - m.zc[p];
    double are = sqrt(arx * arx + ary * ary + arz * arz);
    double nxx = arx / are, nyy = ary / are, nzz = arz / are;
    double dppnnr = 1.0 / ((xpn * nxx) + (ypn * nyy) + (zpn * nzz));
    double xpp = xf - (xf - m.xc[p]) * nxx, ypp = yf - (yf - m.yc[p]) * nyy;
    double zpp = zf - (zf - m.zc[p]) * nzz;
    double xep = xf - (xf - m.xc[q]) * nxx, yep = yf - (yf - m.yc[q]) * nyy;
    double zep = zf - (zf - m.zc[q]) * nzz;
    xpp = xpp - m.xc[p];
    ypp = ypp - m.yc[p];
    zpp = zpp - m.zc[p];
    xep = xep - m.xc[q];
    yep = yep - m.yc[q];
    zep = zep - m.zc[q];
    double rapr = apu[p] * den[p] * m.vol[p] * fxp + apu[q] * den[q] * m.vol[q] * fxn;
    double fmcor = rapr * are *
                   ((dP[3 * q] * xep - dP[3 * p] * xpp) + (dP[3 * q + 1] * yep - dP[3 * p + 1] * ypp) +
                    (dP[3 * q + 2] * zep - dP[3 * p + 2] * zpp)) *
                   dppnnr;
    flmass[m.nin + i] = flmass[m.nin + i] + fmcor;
    fmcor_out[m.nin + i] = fmcor;
  }
}

__global__ void k_fmc_cells(MeshView m, const double *__restrict__ fmcor, double *__restrict__ su) {
  FCG_GRID_STRIDE(c, m.n) {
    double s = 0.0;  // su = 0 (:193), then -= / += fmcor in face order (:203-204)
    for (int e = m.cf_ptr[c]; e < m.cf_ptr[c + 1]; ++e) {
      int ent = m.cf_ent[e];
      double fm = fmcor[(ent > 0 ? ent : -ent) - 1];
      s = ent > 0 ? s - fm : s + fm;
    }
    if (m.noc)  // then the cell's O-C pairs in pair order (:212-213)
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) {
        const int v = m.oc_vix[e];
        const double fm = fmcor[m.nin + (v < m.noc ? v : v - m.noc)];
        s = v < m.noc ? s - fm : s + fm;
      }
    su[c] = s;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// The face factors of the bound mesh (built at the first face loop that needs them).
int fcg::face_geo(fcg_context *c, const double **g) {
  if (!c->fgeo_ready) {
    const size_t nin = c->nin > 0 ? (size_t)c->nin : 1;
    FCG_CUDA_TRY(c, c->fgeo.ensure(sizeof(double) * FG_COUNT * nin));
    if (c->nin > 0) {
      k_face_geo<<<grid_for(c->nin, c->num_sms), kTPB, 0, c->stream>>>(c->mv,
                                                                       c->fgeo.as<double>());
      FCG_CHECK_LAUNCH(c, "k_face_geo");
    }
    c->fgeo_ready = true;
  }
  *g = c->fgeo.as<double>();
  return FCG_OK;
}

int fcg::bnd_geo(fcg_context *c, const double **b) {
  if (!c->bgeo_ready) {
    long long ncb = 0;
    for (int t = 0; t < B_NTYPES; ++t) ncb += c->cnt[t];
    FCG_CUDA_TRY(c, c->bgeo.ensure(sizeof(double) * BG_COUNT * (ncb > 0 ? ncb : 1)));
    if (ncb > 0) {
      k_bnd_geo<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(c->mv, ncb,
                                                                   c->bgeo.as<double>());
      FCG_CHECK_LAUNCH(c, "k_bnd_geo");
    }
    c->bgeo_ready = true;
  }
  *b = c->bgeo.as<double>();
  return FCG_OK;
}

// ---------------------------------------------------------------------------
extern "C" int fcg_laplacian(fcg_context *c, const double *mu, const double *phi, double *a,
                             double *su) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_laplacian before fcg_bind_mesh");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  void *dmu, *dphi, *da, *dsu;
  bool hmu, hphi, ha, hsu;
  int rc;
  if ((rc = stage_in(c, mu, sizeof(double) * c->n, 0, true, &dmu, &hmu))) return rc;
  if ((rc = stage_in(c, phi, sizeof(double) * c->ntot, 1, true, &dphi, &hphi))) return rc;
  const size_t alen = sizeof(double) * (size_t)a_len(c);
  if ((rc = stage_in(c, a, alen, 2, false, &da, &ha))) return rc;
  if ((rc = stage_in(c, su, sizeof(double) * c->n, 3, true, &dsu, &hsu))) return rc;
  const MeshView &m = c->mv;
  const double *g;
  if ((rc = face_geo(c, &g))) return rc;
  if (m.nin > 0) {
    k_lap_faces<<<grid_for(m.nin, c->num_sms), kTPB, 0, c->stream>>>(m, g, (const double *)dmu,
                                                                        (double *)da);
    FCG_CHECK_LAUNCH(c, "k_lap_faces");
  }
  if (m.noc > 0) {
    k_lap_oc<<<grid_for(m.noc, c->num_sms), kTPB, 0, c->stream>>>(m, (const double *)dmu,
                                                                     (double *)da);
    FCG_CHECK_LAUNCH(c, "k_lap_oc");
  }
  k_lap_cells<<<grid_for(m.n, c->num_sms), kTPB, 0, c->stream>>>(
      m, (const double *)dmu, (const double *)dphi, (double *)da, (double *)dsu);
  FCG_CHECK_LAUNCH(c, "k_lap_cells");
  if ((rc = stage_out(c, a, da, alen, ha))) return rc;
  if ((rc = stage_out(c, su, dsu, sizeof(double) * c->n, hsu))) return rc;
  if (ha || hsu) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_facefluxmass(fcg_context *c, const fcg_flow_fields *f, double *a, double *su,
                                double *flmass) {
  if (!c || !f) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_facefluxmass before fcg_bind_mesh");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t nt = sizeof(double) * c->ntot, n1 = sizeof(double) * c->n, n3 = 3 * n1;
  const double *src[12] = {f->u, f->v, f->w, f->p, f->dUdxi, f->dVdxi, f->dWdxi, f->dPdxi,
                           f->apu, f->apv, f->apw, f->den};
  const size_t bytes[12] = {nt, nt, nt, nt, n3, n3, n3, n3, n1, n1, n1, nt};
  void *dev[12];
  bool host[12];
  int rc;
  for (int i = 0; i < 12; ++i)
    if ((rc = stage_in(c, src[i], bytes[i], i, true, &dev[i], &host[i]))) return rc;
  void *da, *dsu, *dfm;
  bool ha, hsu, hfm;
  // with O-C pairs: ar, al after the CSR values and fmoc after the inner faces' fluxes
  const size_t alen = sizeof(double) * (size_t)a_len(c);
  const size_t flen = sizeof(double) * (size_t)(c->nin + c->mv.noc);
  if ((rc = stage_in(c, a, alen, 12, false, &da, &ha))) return rc;
  if ((rc = stage_in(c, su, n1, 13, false, &dsu, &hsu))) return rc;
  if ((rc = stage_in(c, flmass, flen > 0 ? flen : sizeof(double), 14, false, &dfm, &hfm)))
    return rc;
  FlowView fl{(const double *)dev[0], (const double *)dev[1], (const double *)dev[2],
              (const double *)dev[3], (const double *)dev[4], (const double *)dev[5],
              (const double *)dev[6], (const double *)dev[7], (const double *)dev[8],
              (const double *)dev[9], (const double *)dev[10], (const double *)dev[11]};
  const MeshView &m = c->mv;
  const double *g;
  if ((rc = face_geo(c, &g))) return rc;
  if (m.nin > 0) {
    k_ffm_faces<<<grid_for(m.nin, c->num_sms), kTPB, 0, c->stream>>>(m, g, fl, (double *)da,
                                                                        (double *)dfm);
    FCG_CHECK_LAUNCH(c, "k_ffm_faces");
  }
  if (m.noc > 0) {
    k_ffm_oc<<<grid_for(m.noc, c->num_sms), kTPB, 0, c->stream>>>(m, fl, (double *)da,
                                                                     (double *)dfm);
    FCG_CHECK_LAUNCH(c, "k_ffm_oc");
  }
  k_ffm_cells<<<grid_for(m.n, c->num_sms), kTPB, 0, c->stream>>>(m, (const double *)dfm,
                                                                    (double *)da, (double *)dsu);
  FCG_CHECK_LAUNCH(c, "k_ffm_cells");
  if ((rc = stage_out(c, a, da, alen, ha))) return rc;
  if ((rc = stage_out(c, su, dsu, n1, hsu))) return rc;
  if ((rc = stage_out(c, flmass, dfm, flen, hfm))) return rc;
  if (ha || hsu || hfm) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_facefluxmass_piso(fcg_context *c, const fcg_flow_fields *f, double *a,
                                     double *su, double *flmass) {
  if (!c || !f) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_facefluxmass_piso before fcg_bind_mesh");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t nt = sizeof(double) * c->ntot, n1 = sizeof(double) * c->n, n3 = 3 * n1;
  // the fields facefluxmass_piso reads (facefluxmass.f90:300-302)
  const double *src[8] = {f->u, f->v, f->w, f->dUdxi, f->dVdxi, f->dWdxi, f->apu, f->den};
  const size_t bytes[8] = {nt, nt, nt, n3, n3, n3, n1, nt};
  void *dev[8];
  bool host[8];
  int rc;
  for (int i = 0; i < 8; ++i)
    if ((rc = stage_in(c, src[i], bytes[i], i, true, &dev[i], &host[i]))) return rc;
  void *da, *dsu, *dfm;
  bool ha, hsu, hfm;
  // with O-C pairs: ar, al after the CSR values and fmoc after the inner faces' fluxes
  const size_t alen = sizeof(double) * (size_t)a_len(c);
  const size_t flen = sizeof(double) * (size_t)(c->nin + c->mv.noc);
  if ((rc = stage_in(c, a, alen, 12, false, &da, &ha))) return rc;
  if ((rc = stage_in(c, su, n1, 13, false, &dsu, &hsu))) return rc;
  if ((rc = stage_in(c, flmass, flen > 0 ? flen : sizeof(double), 14, false, &dfm, &hfm)))
    return rc;
  FlowView fl{(const double *)dev[0], (const double *)dev[1], (const double *)dev[2], nullptr,
              (const double *)dev[3], (const double *)dev[4], (const double *)dev[5], nullptr,
              (const double *)dev[6], nullptr, nullptr, (const double *)dev[7]};
  const MeshView &m = c->mv;
  const double *g;
  if ((rc = face_geo(c, &g))) return rc;
  if (m.nin > 0) {
    k_ffp_faces<<<grid_for(m.nin, c->num_sms), kTPB, 0, c->stream>>>(m, g, fl, (double *)da,
                                                                        (double *)dfm);
    FCG_CHECK_LAUNCH(c, "k_ffp_faces");
  }
  if (m.noc > 0) {
    k_ffp_oc<<<grid_for(m.noc, c->num_sms), kTPB, 0, c->stream>>>(m, fl, (double *)da,
                                                                     (double *)dfm);
    FCG_CHECK_LAUNCH(c, "k_ffp_oc");
  }
  // a = 0, su = 0 (PISO :109-110), then the diagonal and su in face order (:133-146) and the
  // O-C pairs (:162-173)
  k_ffm_cells<<<grid_for(m.n, c->num_sms), kTPB, 0, c->stream>>>(m, (const double *)dfm,
                                                                    (double *)da, (double *)dsu);
  FCG_CHECK_LAUNCH(c, "k_ffm_cells");
  if ((rc = stage_out(c, a, da, alen, ha))) return rc;
  if ((rc = stage_out(c, su, dsu, n1, hsu))) return rc;
  if ((rc = stage_out(c, flmass, dfm, flen, hfm))) return rc;
  if (ha || hsu || hfm) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_fluxmc(fcg_context *c, const double *dPdxi, const double *apu,
                          const double *den, double *su, double *flmass) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_fluxmc before fcg_bind_mesh");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  void *dP, *dapu, *dden, *dsu, *dfm;
  bool h0, h1, h2, hsu, hfm;
  int rc;
  const size_t n1 = sizeof(double) * c->n;
  if ((rc = stage_in(c, dPdxi, 3 * n1, 0, true, &dP, &h0))) return rc;
  if ((rc = stage_in(c, apu, n1, 1, true, &dapu, &h1))) return rc;
  if ((rc = stage_in(c, den, sizeof(double) * c->ntot, 2, true, &dden, &h2))) return rc;
  if ((rc = stage_in(c, su, n1, 3, false, &dsu, &hsu))) return rc;
  // with O-C pairs flmass holds fmoc after the inner faces' fluxes
  const size_t flen = sizeof(double) * (size_t)(c->nin + c->mv.noc);
  if ((rc = stage_in(c, flmass, flen > 0 ? flen : sizeof(double), 4, true, &dfm, &hfm)))
    return rc;
  FCG_CUDA_TRY(c, c->scratch.ensure(flen > 0 ? flen : sizeof(double)));
  const MeshView &m = c->mv;
  const double *g;
  if ((rc = face_geo(c, &g))) return rc;
  if (m.nin > 0) {
    k_fmc_faces<<<grid_for(m.nin, c->num_sms), kTPB, 0, c->stream>>>(
        m, g, (const double *)dP, (const double *)dapu, (const double *)dden, (double *)dfm,
        c->scratch.as<double>());
    FCG_CHECK_LAUNCH(c, "k_fmc_faces");
  }
  if (m.noc > 0) {
    k_fmc_oc<<<grid_for(m.noc, c->num_sms), kTPB, 0, c->stream>>>(
        m, (const double *)dP, (const double *)dapu, (const double *)dden, (double *)dfm,
        c->scratch.as<double>());
    FCG_CHECK_LAUNCH(c, "k_fmc_oc");
  }
  k_fmc_cells<<<grid_for(m.n, c->num_sms), kTPB, 0, c->stream>>>(m, c->scratch.as<double>(),
                                                                    (double *)dsu);
  FCG_CHECK_LAUNCH(c, "k_fmc_cells");
  if ((rc = stage_out(c, su, dsu, n1, hsu))) return rc;
  if ((rc = stage_out(c, flmass, dfm, flen, hfm))) return rc;
  if (hsu || hfm) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

// ---------------------------------------------------------------------------
// Corrections of calcp after the p' solve
// ---------------------------------------------------------------------------
namespace fcg {
namespace corr {

// flmass(f) += a(slot_pn(f)) * (pp(N) - pp(P)) (calcp-multiple_correction_SIMPLE.f90:159-171)
__global__ void k_flux_correct(MeshView m, const double *__restrict__ a,
                               const double *__restrict__ pp, double *__restrict__ flmass) {
  FCG_GRID_STRIDE(f, m.nin) {
    const int P = m.owner[f], N = m.neighbour[f];
    flmass[f] = flmass[f] + a[m.slot_pn[f]] * (pp[N] - pp[P]);
  }
}

// fmoc(i) += ar(i) * (pp(ijr(i)) - pp(ijl(i))) (calcp :166-171)
__global__ void k_flux_correct_oc(MeshView m, const double *__restrict__ a,
                                  const double *__restrict__ pp, double *__restrict__ flmass) {
  FCG_GRID_STRIDE(i, m.noc) {
    flmass[m.nin + i] = flmass[m.nin + i] + a[m.nnz + i] * (pp[m.oc_r[i]] - pp[m.oc_l[i]]);
  }
}

// u -= dPdxi(1)*vol*apu, v -= dPdxi(2)*vol*apv, w -= dPdxi(3)*vol*apw,
// p += urf*(pp - ppref) (calcp-multiple_correction_SIMPLE.f90:184-189)
__global__ void k_correct_fields(MeshView m, const double *__restrict__ g,
                                 const double *__restrict__ apu, const double *__restrict__ apv,
                                 const double *__restrict__ apw, const double *__restrict__ pp,
                                 double urf, int ref, double *__restrict__ u,
                                 double *__restrict__ v, double *__restrict__ w,
                                 double *__restrict__ p) {
  const double ppref = pp[ref];
  FCG_GRID_STRIDE(i, m.n) {
    const double vol = m.vol[i];
    u[i] = u[i] - g[3 * i] * vol * apu[i];
    v[i] = v[i] - g[3 * i + 1] * vol * apv[i];
    w[i] = w[i] - g[3 * i + 2] * vol * apw[i];
    p[i] = p[i] + urf * (pp[i] - ppref);
  }
}

// correctBoundaryConditionsVelocity.f90:20-57, outlet part one: one thread walks the
// outlet faces in order (flowo is summed in the reference's order), then fac.
__global__ void k_cbv_outlet(MeshView m, int nout, int fst, int bst, const double *__restrict__ den,
                             double flomas, double small, double *__restrict__ u,
                             double *__restrict__ v, double *__restrict__ w,
                             double *__restrict__ fmo, double *__restrict__ fac) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double flowo = 0.0;
  for (int i = 0; i < nout; ++i) {
    const int f = fst + i, P = m.owner[f], b = bst + i;
    u[b] = u[P];
    v[b] = v[P];
    w[b] = w[P];
    fmo[i] = den[P] * (u[b] * m.arx[f] + v[b] * m.ary[f] + w[b] * m.arz[f]);
    flowo = flowo + fmo[i];
  }
  fac[0] = flomas / (flowo + small);
}

// outlet part two (:45-57): fmo and the outlet velocities times fac
__global__ void k_cbv_scale(int nout, int bst, const double *__restrict__ fac,
                            double *__restrict__ u, double *__restrict__ v, double *__restrict__ w,
                            double *__restrict__ fmo) {
  const double f = fac[0];
  FCG_GRID_STRIDE(i, nout) {
    const int b = bst + (int)i;
    fmo[i] = fmo[i] * f;
    u[b] = u[b] * f;
    v[b] = v[b] * f;
    w[b] = w[b] * f;
  }
}

// symmetry faces (:60-76): the cell velocity minus (u.S) S, S the area vector
__global__ void k_cbv_sym(MeshView m, int nsym, int fst, int bst, double *__restrict__ u,
                          double *__restrict__ v, double *__restrict__ w) {
  FCG_GRID_STRIDE(i, nsym) {
    const int f = fst + (int)i, P = m.owner[f], b = bst + (int)i;
    const double un = u[P] * m.arx[f] + v[P] * m.ary[f] + w[P] * m.arz[f];
    u[b] = u[P] - un * m.arx[f];
    v[b] = v[P] - un * m.ary[f];
    w[b] = w[P] - un * m.arz[f];
  }
}

// continuityErrors.h:7-41 per cell, in the reference's order: the inner faces in face
// order (res(ijp) -= flmass(ijp), res(ijn) += flmass(ijp) -- flmass indexed by the
// owner cell, as the reference does), then the inlet and outlet faces.
__global__ void k_contin_cells(MeshView m, const double *__restrict__ flmass,
                               const double *__restrict__ fmi, const double *__restrict__ fmo,
                               int bst_inl, int bst_out, double *__restrict__ res) {
  FCG_GRID_STRIDE(c, m.n) {
    double r = 0.0;
    for (int e = m.cf_ptr[c]; e < m.cf_ptr[c + 1]; ++e) {
      const int ent = m.cf_ent[e];
      if (ent > 0)
        r = r - flmass[c];
      else
        r = r + flmass[m.owner[-ent - 1]];
    }
    if (m.noc)  // faces along O-C grid cuts (:22-28), fmoc after the inner faces' fluxes
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) {
        const int v = m.oc_vix[e];
        const double fm = flmass[m.nin + (v < m.noc ? v : v - m.noc)];
        r = v < m.noc ? r - fm : r + fm;
      }
    for (int e = m.cb_ptr[c]; e < m.cb_ptr[c + 1]; ++e) {
      const int t = m.cb_type[e];
      if (t == B_INLET) r = r - fmi[m.cb_slot[e] - bst_inl];
      else if (t == B_OUTLET) r = r - fmo[m.cb_slot[e] - bst_out];
    }
    res[c] = r;
  }
}

// sum|res| and sum res: per-block partials (fixed thread order), then one block adds
// them in block order
__global__ void k_contin_part(int n, const double *__restrict__ res, double *__restrict__ part) {
  __shared__ double sh[2][kTPB];
  double a = 0.0, b = 0.0;
  FCG_GRID_STRIDE(i, n) {
    a += fabs(res[i]);
    b += res[i];
  }
  sh[0][threadIdx.x] = a;
  sh[1][threadIdx.x] = b;
  __syncthreads();
  for (int s = kTPB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sh[0][0];
    part[2 * blockIdx.x + 1] = sh[1][0];
  }
}

__global__ void k_contin_total(int nblocks, const double *__restrict__ part,
                               double *__restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a = 0.0, b = 0.0;
  for (int k = 0; k < nblocks; ++k) {
    a += part[2 * k];
    b += part[2 * k + 1];
  }
  out[0] = a;
  out[1] = b;
}

// The outlet part shared by correctBoundaryConditionsVelocity (:20-57) and adjustMassFlow
// (adjustMassFlow.f90:30-63): outlet slots take their cell's velocity, fmo, the sequential
// outflow sum, fac, and fmo and the outlet velocities times fac.  fac lands in scratch[0].
int outlet_flow(fcg_context *c, const double *den, double flomas, double *u, double *v,
                double *w, double *fmo) {
  const int nout = c->cnt[B_OUTLET];
  if (nout <= 0) return FCG_OK;
  FCG_CUDA_TRY(c, c->scratch.ensure(sizeof(double) * 8));
  k_cbv_outlet<<<1, 32, 0, c->stream>>>(
      c->mv, nout, c->fst[B_OUTLET], c->bst[B_OUTLET], den, flomas,
      (double)1e-20f /* parameters::small, modules_allocatable.f90:27 */, u, v, w, fmo,
      c->scratch.as<double>());
  k_cbv_scale<<<grid_for(nout, c->num_sms), kTPB, 0, c->stream>>>(
      nout, c->bst[B_OUTLET], c->scratch.as<double>(), u, v, w, fmo);
  FCG_CHECK_LAUNCH(c, "outlet_flow");
  return FCG_OK;
}

}  // namespace corr
}  // namespace fcg

extern "C" int fcg_correct_bc_velocity(fcg_context *c, const double *den, double flomas,
                                       double *u, double *v, double *w, double *fmo) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_correct_bc_velocity before fcg_bind_mesh");
  if (!den || !u || !v || !w || (!fmo && c->cnt[B_OUTLET] > 0))
    return set_error(c, FCG_ERR_ARG, "NULL array");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t nt = sizeof(double) * c->ntot;
  const int nout = c->cnt[B_OUTLET], nsym = c->cnt[B_SYMMETRY];
  void *dden, *du, *dv, *dw, *dfmo = nullptr;
  bool hden, hu, hv, hw, hfmo = false;
  int rc;
  if ((rc = stage_in(c, den, nt, 0, true, &dden, &hden))) return rc;
  if ((rc = stage_in(c, u, nt, 1, true, &du, &hu))) return rc;
  if ((rc = stage_in(c, v, nt, 2, true, &dv, &hv))) return rc;
  if ((rc = stage_in(c, w, nt, 3, true, &dw, &hw))) return rc;
  if (nout > 0 && (rc = stage_in(c, fmo, sizeof(double) * nout, 4, false, &dfmo, &hfmo))) return rc;
  if ((rc = fcg::corr::outlet_flow(c, (const double *)dden, flomas, (double *)du, (double *)dv,
                                   (double *)dw, (double *)dfmo)))
    return rc;
  if (nsym > 0)
    fcg::corr::k_cbv_sym<<<grid_for(nsym, c->num_sms), kTPB, 0, c->stream>>>(
        c->mv, nsym, c->fst[B_SYMMETRY], c->bst[B_SYMMETRY], (double *)du, (double *)dv,
        (double *)dw);
  FCG_CHECK_LAUNCH(c, "correct_bc_velocity");
  bool any = hu || hv || hw || hfmo;
  if ((rc = stage_out(c, u, du, nt, hu)) || (rc = stage_out(c, v, dv, nt, hv)) ||
      (rc = stage_out(c, w, dw, nt, hw)))
    return rc;
  if (nout > 0 && (rc = stage_out(c, fmo, dfmo, sizeof(double) * nout, hfmo))) return rc;
  if (any) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_continuity_errors(fcg_context *c, const double *flmass, const double *fmi,
                                     const double *fmo, double *res, double *sum_local,
                                     double *global) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_continuity_errors before fcg_bind_mesh");
  if (!flmass || (!fmi && c->cnt[B_INLET] > 0) || (!fmo && c->cnt[B_OUTLET] > 0))
    return set_error(c, FCG_ERR_ARG, "NULL array");
  if (c->n > c->nin)
    return set_error(c, FCG_ERR_INDEX,
                     "continuityErrors.h:14 indexes flmass by cell: needs numCells <= numInnerFaces");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const int nin_ = c->cnt[B_INLET], nout = c->cnt[B_OUTLET];
  void *dfm, *dfmi = nullptr, *dfmo = nullptr, *dres;
  bool h0, h1 = false, h2 = false, hres = false;
  int rc;
  if ((rc = stage_in(c, flmass, sizeof(double) * (size_t)(c->nin + c->mv.noc), 0, true, &dfm, &h0)))
    return rc;
  if (nin_ > 0 && (rc = stage_in(c, fmi, sizeof(double) * nin_, 1, true, &dfmi, &h1))) return rc;
  if (nout > 0 && (rc = stage_in(c, fmo, sizeof(double) * nout, 2, true, &dfmo, &h2))) return rc;
  const size_t n1 = sizeof(double) * c->n;
  const int G = std::min(grid_for(c->n, c->num_sms), 1024);
  // scratch: block partials, the two totals and, without a caller array, res itself
  FCG_CUDA_TRY(c, c->scratch.ensure(sizeof(double) * (2 * 1024 + 8 + (res ? 0 : c->n))));
  double *part = c->scratch.as<double>(), *tot = part + 2 * 1024;
  if (res) {
    if ((rc = stage_in(c, res, n1, 3, false, &dres, &hres))) return rc;
  } else {
    dres = tot + 8;
  }
  fcg::corr::k_contin_cells<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(
      c->mv, (const double *)dfm, (const double *)dfmi, (const double *)dfmo, c->bst[B_INLET],
      c->bst[B_OUTLET], (double *)dres);
  fcg::corr::k_contin_part<<<G, kTPB, 0, c->stream>>>(c->n, (const double *)dres, part);
  fcg::corr::k_contin_total<<<1, 32, 0, c->stream>>>(G, part, tot);
  FCG_CHECK_LAUNCH(c, "continuity_errors");
  double h[2];
  FCG_CUDA_TRY(c, cudaMemcpyAsync(h, tot, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  if (res && (rc = stage_out(c, res, dres, n1, hres))) return rc;
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (sum_local) *sum_local = h[0];
  if (global) *global = h[1];
  return FCG_OK;
}

extern "C" int fcg_flux_correct(fcg_context *c, const double *a, const double *pp,
                                double *flmass) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_flux_correct before fcg_bind_mesh");
  if (!a || !pp || !flmass) return set_error(c, FCG_ERR_ARG, "NULL a, pp or flmass");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  void *da, *dpp, *dfm;
  bool ha, hpp, hfm;
  int rc;
  // with O-C pairs: ar, al after the CSR values, fmoc after the inner faces' fluxes
  const size_t flen = sizeof(double) * (size_t)(c->nin + c->mv.noc);
  const size_t nf = flen > 0 ? flen : sizeof(double);
  if ((rc = stage_in(c, a, sizeof(double) * (size_t)a_len(c), 0, true, &da, &ha))) return rc;
  if ((rc = stage_in(c, pp, sizeof(double) * c->ntot, 1, true, &dpp, &hpp))) return rc;
  if ((rc = stage_in(c, flmass, nf, 2, true, &dfm, &hfm))) return rc;
  if (c->nin > 0) {
    fcg::corr::k_flux_correct<<<grid_for(c->nin, c->num_sms), kTPB, 0, c->stream>>>(
        c->mv, (const double *)da, (const double *)dpp, (double *)dfm);
    FCG_CHECK_LAUNCH(c, "k_flux_correct");
  }
  if (c->mv.noc > 0) {
    fcg::corr::k_flux_correct_oc<<<grid_for(c->mv.noc, c->num_sms), kTPB, 0, c->stream>>>(
        c->mv, (const double *)da, (const double *)dpp, (double *)dfm);
    FCG_CHECK_LAUNCH(c, "k_flux_correct_oc");
  }
  if ((rc = stage_out(c, flmass, dfm, flen, hfm))) return rc;
  if (hfm) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_correct_fields(fcg_context *c, const double *dPdxi, const double *apu,
                                  const double *apv, const double *apw, const double *pp,
                                  double urf, int pRefCell, double *u, double *v, double *w,
                                  double *p) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_correct_fields before fcg_bind_mesh");
  if (!dPdxi || !apu || !apv || !apw || !pp || !u || !v || !w || !p)
    return set_error(c, FCG_ERR_ARG, "NULL array");
  if (pRefCell < 1 || pRefCell > c->n) return set_error(c, FCG_ERR_INDEX, "pRefCell out of range");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t n1 = sizeof(double) * c->n, nt = sizeof(double) * c->ntot;
  const void *in[6] = {dPdxi, apu, apv, apw, pp, nullptr};
  const size_t inb[5] = {3 * n1, n1, n1, n1, nt};
  void *din[5];
  bool hin[5];
  int rc;
  for (int k = 0; k < 5; ++k)
    if ((rc = stage_in(c, in[k], inb[k], k, true, &din[k], &hin[k]))) return rc;
  double *out[4] = {u, v, w, p};
  void *dout[4];
  bool hout[4];
  for (int k = 0; k < 4; ++k)
    if ((rc = stage_in(c, out[k], nt, 5 + k, true, &dout[k], &hout[k]))) return rc;
  fcg::corr::k_correct_fields<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(
      c->mv, (const double *)din[0], (const double *)din[1], (const double *)din[2],
      (const double *)din[3], (const double *)din[4], urf, pRefCell - 1, (double *)dout[0],
      (double *)dout[1], (double *)dout[2], (double *)dout[3]);
  FCG_CHECK_LAUNCH(c, "k_correct_fields");
  bool any = false;
  for (int k = 0; k < 4; ++k) {
    if ((rc = stage_out(c, out[k], dout[k], nt, hout[k]))) return rc;
    any = any || hout[k];
  }
  if (any) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}
