// Momentum assembly of calcuvw (calcuvw.f90:48-438): the u, v and w systems that the
// three bicgstab calls (or one multi-RHS solve) take.
//
// Two kernels and no atomics, like the pressure assembly:
//   1. one thread per inner face computes facefluxuvw (faceflux_velocity.f90:35-184) and
//      the pressure-divergence term of presFaceDivInner (fieldManipulation.f90:395-443),
//      writes the face's two off-diagonal slots and keeps its six source terms;
//   2. one thread per cell adds every source in the reference's order -- the pressure
//      divergence, the volume sources, the face fluxes, the boundary loops,
//      Crank-Nicolson -- and assembles the three diagonals from its own CSR row.
// Compiled with --fmad=false: bit-identical to the reference's loops on the same inputs.
//
// MIN and MAX keep the first argument on ties (only the sign of a zero can differ).
#include "face_geo.h"
#include "fcg_internal.h"
#include "launch.h"

using namespace fcg;

namespace {

__device__ __forceinline__ double rmin(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double rmax(double a, double b) { return b > a ? b : a; }

struct UvwView {
  const double *u, *v, *w, *p, *vis, *den, *t, *uo, *vo, *wo, *uoo, *voo, *woo;
  const double *dU, *dV, *dW, *dP, *flmass, *fmi, *fmo;
};

// The face's offsets that face_value reads, with the upwind cell first: the face centre
// minus the upwind cell's centre (du*) and minus the downwind cell's centre (dd*), from
// the cached face factors.
struct Offs {
  double dux, duy, duz, ddx, ddy, ddz;
};

// face_value (interpolation.f90:20-60) with the first cell upwind: f is the first cell,
// s the second, lam the weight of the second (the caller passes fxp or fxn as the
// reference does).  One instantiation per scheme: the scheme is fixed for a call.
template <int S>
__device__ __forceinline__ double face_value(const MeshView &m, int limiter, int f, int s,
                                             double lam, long long fi_face, const Offs &o,
                                             const double *__restrict__ fi,
                                             const double *__restrict__ g) {
  if constexpr (S == FCG_CONV_CDS) {  // :65-93
    const double fxn = lam, fxp = 1.0 - lam;
    return fi[f] * fxp + fi[s] * fxn;
  } else if constexpr (S == FCG_CONV_CDS_CORRECTED) {  // :99-139
    const double xf = m.xf[fi_face], yf = m.yf[fi_face], zf = m.zf[fi_face];
    const double fxn = lam, fxp = 1.0 - lam;
    const double xi = m.xc[f] * fxp + m.xc[s] * fxn, yi = m.yc[f] * fxp + m.yc[s] * fxn,
                 zi = m.zc[f] * fxp + m.zc[s] * fxn;
    const double dx = g[3 * f] * fxp + g[3 * s] * fxn, dy = g[3 * f + 1] * fxp + g[3 * s + 1] * fxn,
                 dz = g[3 * f + 2] * fxp + g[3 * s + 2] * fxn;
    return fi[f] * fxp + fi[s] * fxn + (dx * (xf - xi) + dy * (yf - yi) + dz * (zf - zi));
  } else if constexpr (S == FCG_CONV_CENTRAL) {  // :145-199
    const double r = g[3 * f] * o.dux + g[3 * f + 1] * o.duy + g[3 * f + 2] * o.duz +
                     g[3 * s] * o.ddx + g[3 * s + 1] * o.ddy + g[3 * s + 2] * o.ddz;
    return 0.5 * (fi[f] + fi[s] + r);
  } else if constexpr (S == FCG_CONV_SECOND_UPWIND) {  // :204-249
    const double r = g[3 * f] * o.dux + g[3 * f + 1] * o.duy + g[3 * f + 2] * o.duz;
    return fi[f] + r;
  } else if constexpr (S == FCG_CONV_FLUX_LIMITER) {  // :325-393
    const double fxp = 1.0 - lam;
    const double xpn = m.xc[s] - m.xc[f], ypn = m.yc[s] - m.yc[f], zpn = m.zc[s] - m.zc[f];
    const double r = (2.0 * g[3 * f] * xpn + 2.0 * g[3 * f + 1] * ypn + 2.0 * g[3 * f + 2] * zpn) /
                         (fi[s] - fi[f]) -
                     1.0;
    double psi;
    switch (limiter) {
      case FCG_LIM_SMART:
        psi = rmax(0.0, rmin(rmin(2.0 * r, 0.75 * r + 0.25), 4.0));
        break;
      case FCG_LIM_AVL:
        psi = rmax(0.0, rmin(rmin(1.5 * r, 0.75 * r + 0.25), 2.5));
        break;
      case FCG_LIM_MUSCL:
        psi = rmax(0.0, rmin(rmin(2.0 * r, 0.5 * r + 0.5), 2.0));
        break;
      case FCG_LIM_UMIST:
        psi = rmax(0.0, rmin(rmin(rmin(2.0 * r, 0.75 * r + 0.25), 0.25 * r + 0.75), 2.0));
        break;
      case FCG_LIM_KOREN:
        psi = rmax(0.0, rmin(rmin(2.0 * r, 2.0 / 3.0 * r + 1.0 / 3.0), 2.0));
        break;
      case FCG_LIM_CHARM:
        psi = (r + fabs(r)) * (3.0 * r + 1.0) / (2.0 * ((r + 1.0) * (r + 1.0)));
        break;
      case FCG_LIM_OSPRE:
        psi = 1.5 * r * (r + 1.0) / (r * r + r + 1.0);
        break;
      default:
        psi = 1.0;
    }
    return fi[f] + fxp * psi * (fi[s] - fi[f]);
  } else {  // FCG_CONV_MUSCL, :254-320
    const double theta = 0.125;
    // the reference's central correction repeats the upwind one's three products first,
    // so it continues from the same partial sum
    const double g2 = g[3 * f] * o.dux + g[3 * f + 1] * o.duy + g[3 * f + 2] * o.duz;
    const double gc = g2 + g[3 * s] * o.ddx + g[3 * s + 1] * o.ddy + g[3 * s + 2] * o.ddz;
    const double fv2 = fi[f] + g2;
    const double fvc = 0.5 * (fi[f] + fi[s] + gc);
    return theta * fvc + (1.0 - theta) * fv2;
  }
}

// sngrad with nrelax = 0 and the skewness approach (gradients.f90:597-668): the face
// gradient interpolated (dxi..) and corrected (dxii..).  costn = 1, so d1 = 1 and
// d2 = (xpn, ypn, zpn) exactly; rv = (arx, ary, arz) / vole comes from the cached factors.
struct SnGrad {
  double xi, yi, zi, xii, yii, zii;
};

__device__ __forceinline__ SnGrad sngrad(int p, int q, double rvx, double rvy, double rvz,
                                         double fxp, double fxn, double xpn, double ypn,
                                         double zpn, const double *__restrict__ fi,
                                         const double *__restrict__ g) {
  SnGrad s;
  s.xi = g[3 * p] * fxp + g[3 * q] * fxn;
  s.yi = g[3 * p + 1] * fxp + g[3 * q + 1] * fxn;
  s.zi = g[3 * p + 2] * fxp + g[3 * q + 2] * fxn;
  const double r = fi[q] - fi[p] - s.xi * xpn - s.yi * ypn - s.zi * zpn;
  s.xii = s.xi + rvx * r;
  s.yii = s.yi + rvy * r;
  s.zii = s.zi + rvz * r;
  return s;
}

template <int S>
__global__ void __launch_bounds__(kTPB)
    k_uvw_faces(MeshView m, fcg_uvw_params prm, UvwView F, const double *__restrict__ geo,
                double *__restrict__ a, double *__restrict__ fsrc, double *__restrict__ fdiv) {
  const long long nin = m.nin;
  FCG_GRID_STRIDE(f, nin) {
    const int p = m.owner[f], q = m.neighbour[f];
    const double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
    const double lambda = m.facint[f];
    const double flomass = F.flmass[f];
    // facefluxuvw (faceflux_velocity.f90:78-182)
    const double fxn = lambda, fxp = 1.0 - lambda;
    const double xpn = geo[FG_XPN * nin + f], ypn = geo[FG_YPN * nin + f],
                 zpn = geo[FG_ZPN * nin + f];
    const double dpn = geo[FG_DPN * nin + f];
    const double are = geo[FG_ARE * nin + f];
    const double game = F.vis[p] * fxp + F.vis[q] * fxn;
    const double de = game * are / dpn;
    double can = -de + rmin(flomass, 0.0);
    double cap = -de - rmax(flomass, 0.0);
    const double rvx = geo[FG_RVX * nin + f], rvy = geo[FG_RVY * nin + f],
                 rvz = geo[FG_RVZ * nin + f];
    const SnGrad du = sngrad(p, q, rvx, rvy, rvz, fxp, fxn, xpn, ypn, zpn, F.u, F.dU);
    const SnGrad dv = sngrad(p, q, rvx, rvy, rvz, fxp, fxn, xpn, ypn, zpn, F.v, F.dV);
    const SnGrad dw = sngrad(p, q, rvx, rvy, rvz, fxp, fxn, xpn, ypn, zpn, F.w, F.dW);
    const double fdue = game * ((du.xii + du.xii) * arx + (du.yii + dv.xii) * ary + (du.zii + dw.xii) * arz);
    const double fdve = game * ((du.yii + dv.xii) * arx + (dv.yii + dv.yii) * ary + (dv.zii + dw.yii) * arz);
    const double fdwe = game * ((du.zii + dw.xii) * arx + (dw.yii + dv.zii) * ary + (dw.zii + dw.zii) * arz);
    // game * are / dpn * (...) evaluates its first factor as de does
    const double fdui = de * (du.xi * xpn + du.yi * ypn + du.zi * zpn);
    const double fdvi = de * (dv.xi * xpn + dv.yi * ypn + dv.zi * zpn);
    const double fdwi = de * (dw.xi * xpn + dw.yi * ypn + dw.zi * zpn);
    const double fpos = rmax(flomass, 0.0), fneg = rmin(flomass, 0.0);
    const double fuuds = fpos * F.u[p] + fneg * F.u[q];
    const double fvuds = fpos * F.v[p] + fneg * F.v[q];
    const double fwuds = fpos * F.w[p] + fneg * F.w[q];
    // face_value from the upwind side (:129-150): one path for both signs of the flux
    const bool fwd = flomass >= 0.0;
    const int uc = fwd ? p : q, dc = fwd ? q : p;
    const double lam = fwd ? fxp : fxn;
    Offs o{};
    if constexpr (S == FCG_CONV_CENTRAL || S == FCG_CONV_SECOND_UPWIND || S == FCG_CONV_MUSCL) {
      const double dxp = geo[FG_DXP * nin + f], dyp = geo[FG_DYP * nin + f],
                   dzp = geo[FG_DZP * nin + f];
      const double dxq = geo[FG_DXQ * nin + f], dyq = geo[FG_DYQ * nin + f],
                   dzq = geo[FG_DZQ * nin + f];
      o = fwd ? Offs{dxp, dyp, dzp, dxq, dyq, dzq} : Offs{dxq, dyq, dzq, dxp, dyp, dzp};
    }
    const double ue = face_value<S>(m, prm.limiter, uc, dc, lam, f, o, F.u, F.dU);
    const double ve = face_value<S>(m, prm.limiter, uc, dc, lam, f, o, F.v, F.dV);
    const double we = face_value<S>(m, prm.limiter, uc, dc, lam, f, o, F.w, F.dW);
    const double gam = prm.gds;
    fsrc[3 * f] = -gam * (flomass * ue - fuuds) + fdue - fdui;
    fsrc[3 * f + 1] = -gam * (flomass * ve - fvuds) + fdve - fdvi;
    fsrc[3 * f + 2] = -gam * (flomass * we - fwuds) + fdwe - fdwi;
    if (prm.cn) {  // a = 0.5*a (calcuvw.f90:382-384)
      can = 0.5 * can;
      cap = 0.5 * cap;
    }
    a[m.slot_pn[f]] = can;  // :168-173
    a[m.slot_np[f]] = cap;
    // presFaceDivInner (fieldManipulation.f90:426-442).  The reference indexes its
    // (3,numCells) gradient argument as df(ijp,k): element ijp + 3(k-1) of the flat array.
    const double *dP = F.dP;
    const double dfxi = dP[p] * fxp + dP[q] * fxn;
    const double dfyi = dP[p + 3] * fxp + dP[q + 3] * fxn;
    const double dfzi = dP[p + 6] * fxp + dP[q + 6] * fxn;
    const double fie = F.p[p] * fxp + F.p[q] * fxn + dfxi * geo[FG_DXI * nin + f] +
                       dfyi * geo[FG_DYI * nin + f] + dfzi * geo[FG_DZI * nin + f];
    fdiv[3 * f] = fie * arx;
    fdiv[3 * f + 1] = fie * ary;
    fdiv[3 * f + 2] = fie * arz;
  }
}

// The O-C pairs (calcuvw.f90:186-215, fieldManipulation.f90:110-125): facefluxuvw_cyclic
// (faceflux_velocity.f90:189-354, what the generic facefluxuvw resolves to for the
// pairs) and presFaceDivInner on face ijlFace(i) with foc(i), the pair's mass flux fmoc(i)
// after the inner faces' fluxes, computed in place: the distance is |S| / srdoc(i) and
// the vector dpn S / |S|, sngrad keeps the cell centres.  ar = can and al = cap go after
// the CSR values of a (not halved for Crank-Nicolson: :380 halves a only).
template <int S>
__global__ void __launch_bounds__(kTPB)
    k_uvw_oc(MeshView m, fcg_uvw_params prm, UvwView F, double *__restrict__ a,
             double *__restrict__ osrc, double *__restrict__ odiv) {
  FCG_GRID_STRIDE(i, m.noc) {
    const int p = m.oc_l[i], q = m.oc_r[i], f = m.oc_fl[i];
    const double arx = m.arx[f], ary = m.ary[f], arz = m.arz[f];
    const double xf = m.xf[f], yf = m.yf[f], zf = m.zf[f];
    const double lambda = m.oc_foc[i];
    const double flomass = F.flmass[m.nin + i];
    const double fxn = lambda, fxp = 1.0 - lambda;
    const double are = sqrt(arx * arx + ary * ary + arz * arz);
    const double dpn = are / m.oc_srdoc[i];
    const double xpn = dpn * arx / are, ypn = dpn * ary / are, zpn = dpn * arz / are;
    const double game = F.vis[p] * fxp + F.vis[q] * fxn;
    const double de = game * are / dpn;
    const double can = -de + rmin(flomass, 0.0);
    const double cap = -de - rmax(flomass, 0.0);
    const double cxpn = m.xc[q] - m.xc[p], cypn = m.yc[q] - m.yc[p], czpn = m.zc[q] - m.zc[p];
    const double vole = cxpn * arx + cypn * ary + czpn * arz;
    const double rvx = arx / vole, rvy = ary / vole, rvz = arz / vole;
    const SnGrad du = sngrad(p, q, rvx, rvy, rvz, fxp, fxn, cxpn, cypn, czpn, F.u, F.dU);
    const SnGrad dv = sngrad(p, q, rvx, rvy, rvz, fxp, fxn, cxpn, cypn, czpn, F.v, F.dV);
    const SnGrad dw = sngrad(p, q, rvx, rvy, rvz, fxp, fxn, cxpn, cypn, czpn, F.w, F.dW);
    const double fdue = game * ((du.xii + du.xii) * arx + (du.yii + dv.xii) * ary + (du.zii + dw.xii) * arz);
    const double fdve = game * ((du.yii + dv.xii) * arx + (dv.yii + dv.yii) * ary + (dv.zii + dw.yii) * arz);
    const double fdwe = game * ((du.zii + dw.xii) * arx + (dw.yii + dv.zii) * ary + (dw.zii + dw.zii) * arz);
    const double fdui = de * (du.xi * xpn + du.yi * ypn + du.zi * zpn);
    const double fdvi = de * (dv.xi * xpn + dv.yi * ypn + dv.zi * zpn);
    const double fdwi = de * (dw.xi * xpn + dw.yi * ypn + dw.zi * zpn);
    const double fpos = rmax(flomass, 0.0), fneg = rmin(flomass, 0.0);
    const double fuuds = fpos * F.u[p] + fneg * F.u[q];
    const double fvuds = fpos * F.v[p] + fneg * F.v[q];
    const double fwuds = fpos * F.w[p] + fneg * F.w[q];
    const bool fwd = flomass >= 0.0;
    const int uc = fwd ? p : q, dc = fwd ? q : p;
    const double lam = fwd ? fxp : fxn;
    const double dxp = xf - m.xc[p], dyp = yf - m.yc[p], dzp = zf - m.zc[p];
    const double dxq = xf - m.xc[q], dyq = yf - m.yc[q], dzq = zf - m.zc[q];
    const Offs o = fwd ? Offs{dxp, dyp, dzp, dxq, dyq, dzq} : Offs{dxq, dyq, dzq, dxp, dyp, dzp};
    const double ue = face_value<S>(m, prm.limiter, uc, dc, lam, f, o, F.u, F.dU);
    const double ve = face_value<S>(m, prm.limiter, uc, dc, lam, f, o, F.v, F.dV);
    const double we = face_value<S>(m, prm.limiter, uc, dc, lam, f, o, F.w, F.dW);
    const double gam = prm.gds;
    osrc[3 * i] = -gam * (flomass * ue - fuuds) + fdue - fdui;
    osrc[3 * i + 1] = -gam * (flomass * ve - fvuds) + fdve - fdvi;
    osrc[3 * i + 2] = -gam * (flomass * we - fwuds) + fdwe - fdwi;
    a[m.nnz + i] = can;          // ar(i)
    a[m.nnz + m.noc + i] = cap;  // al(i)
    const double *dP = F.dP;  // presFaceDivInner, df(ijp,k) on the flat (3,n) array
    const double dfxi = dP[p] * fxp + dP[q] * fxn;
    const double dfyi = dP[p + 3] * fxp + dP[q + 3] * fxn;
    const double dfzi = dP[p + 6] * fxp + dP[q + 6] * fxn;
    const double xi = m.xc[p] * fxp + m.xc[q] * fxn, yi = m.yc[p] * fxp + m.yc[q] * fxn,
                 zi = m.zc[p] * fxp + m.zc[q] * fxn;
    const double fie = F.p[p] * fxp + F.p[q] * fxn + dfxi * (xf - xi) + dfyi * (yf - yi) +
                       dfzi * (zf - zi);
    odiv[3 * i] = fie * arx;
    odiv[3 * i + 1] = fie * ary;
    odiv[3 * i + 2] = fie * arz;
  }
}

// Sum of the row's values in row order with `dv` in place of the diagonal (Fortran SUM).
__device__ __forceinline__ double row_sum(const MeshView &m, const double *__restrict__ a,
                                          int c, double dv) {
  const int dg = m.diag[c];
  double s = 0.0;
  for (int k = m.ioffset[c]; k < m.ioffset[c + 1]; ++k) s = s + (k == dg ? dv : a[k]);
  return s;
}

__global__ void k_uvw_cells(MeshView m, fcg_uvw_params prm, UvwView F, int bst_inl,
                            int bst_out, const double *__restrict__ bg, long long ncb,
                            double *__restrict__ a,
                            const double *__restrict__ fsrc, const double *__restrict__ fdiv,
                            const double *__restrict__ osrc, const double *__restrict__ odiv,
                            double *__restrict__ diag_vw, double *__restrict__ rhs,
                            double *__restrict__ ap) {
  const double small = (double)1e-20f;  // parameters::small, modules_allocatable.f90:27
  FCG_GRID_STRIDE(c, m.n) {
    const int e0 = m.cf_ptr[c], e1 = m.cf_ptr[c + 1];
    const int b0 = m.cb_ptr[c], b1 = m.cb_ptr[c + 1];
    const double vol = m.vol[c];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;     // su, sv, sw (:49-51)
    double sp0 = 0.0, sp1 = 0.0, sp2 = 0.0;  // spu, spv, sp (:54-56)
    // calcPressDiv: inner faces (fieldManipulation.f90:92-108), then every boundary face
    // in the loop order inlet, outlet, symmetry, wall, pressure outlet (:129-160)
    for (int e = e0; e < e1; ++e) {
      const int ent = m.cf_ent[e];
      const int f = (ent > 0 ? ent : -ent) - 1;
      if (ent > 0) {
        s0 = s0 - fdiv[3 * f];
        s1 = s1 - fdiv[3 * f + 1];
        s2 = s2 - fdiv[3 * f + 2];
      } else {
        s0 = s0 + fdiv[3 * f];
        s1 = s1 + fdiv[3 * f + 1];
        s2 = s2 + fdiv[3 * f + 2];
      }
    }
    if (m.noc)  // the O-C pairs (fieldManipulation.f90:110-125)
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) {
        const int v = m.oc_vix[e], i = v < m.noc ? v : v - m.noc;
        if (v < m.noc) {
          s0 = s0 - odiv[3 * i];
          s1 = s1 - odiv[3 * i + 1];
          s2 = s2 - odiv[3 * i + 2];
        } else {
          s0 = s0 + odiv[3 * i];
          s1 = s1 + odiv[3 * i + 1];
          s2 = s2 + odiv[3 * i + 2];
        }
      }
    for (int e = b0; e < b1; ++e) {
      const int f = m.cb_face[e];
      const double pb = F.p[m.cb_slot[e]];
      s0 = s0 - pb * m.arx[f];
      s1 = s1 - pb * m.ary[f];
      s2 = s2 - pb * m.arz[f];
    }
    // volume sources (:76-139)
    if (prm.const_mflux) s0 = s0 + prm.gradPcmf * vol;
    if (prm.buoyancy) {
      double heat;
      if (prm.boussinesq)
        heat = prm.beta * prm.densit * (F.t[c] - prm.tref) * vol;
      else
        heat = (prm.densit - F.den[c]) * vol;
      s0 = s0 - prm.gravx * heat;
      s1 = s1 - prm.gravy * heat;
      s2 = s2 - prm.gravz * heat;
    }
    if (prm.bdf) {
      const double apotime = F.den[c] * vol / prm.timestep;
      double sut = apotime * ((1.0 + prm.btime) * F.uo[c]);
      double svt = apotime * ((1.0 + prm.btime) * F.vo[c]);
      double swt = apotime * ((1.0 + prm.btime) * F.wo[c]);
      if (prm.btime > (double)0.99f) {
        sut = sut - apotime * (0.5 * prm.btime * F.uoo[c]);
        svt = svt - apotime * (0.5 * prm.btime * F.voo[c]);
        swt = swt - apotime * (0.5 * prm.btime * F.woo[c]);
      }
      s0 = s0 + sut;
      s1 = s1 + svt;
      s2 = s2 + swt;
      const double add = apotime * (1.0 + 0.5 * prm.btime);
      sp0 = sp0 + add;
      sp1 = sp1 + add;
      sp2 = sp2 + add;
    }
    // inner faces (:157-185)
    for (int e = e0; e < e1; ++e) {
      const int ent = m.cf_ent[e];
      const int f = (ent > 0 ? ent : -ent) - 1;
      if (ent > 0) {
        s0 = s0 + fsrc[3 * f];
        s1 = s1 + fsrc[3 * f + 1];
        s2 = s2 + fsrc[3 * f + 2];
      } else {
        s0 = s0 - fsrc[3 * f];
        s1 = s1 - fsrc[3 * f + 1];
        s2 = s2 - fsrc[3 * f + 2];
      }
    }
    if (m.noc)  // the O-C pairs (:186-215): ar (left cell) or al (right) off sp, the sources
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) {
        const int v = m.oc_vix[e], i = v < m.noc ? v : v - m.noc;
        const double co = a[m.nnz + v];
        sp0 = sp0 - co;
        sp1 = sp1 - co;
        sp2 = sp2 - co;
        if (v < m.noc) {
          s0 = s0 + osrc[3 * i];
          s1 = s1 + osrc[3 * i + 1];
          s2 = s2 + osrc[3 * i + 2];
        } else {
          s0 = s0 - osrc[3 * i];
          s1 = s1 - osrc[3 * i + 1];
          s2 = s2 - osrc[3 * i + 2];
        }
      }
    // boundary loops (:223-378): inlet, outlet, symmetry, wall
    for (int e = b0; e < b1; ++e) {
      const int t = m.cb_type[e];
      if (t == B_PRESSOUT) continue;
      const int b = m.cb_slot[e];
      const double are = bg[BG_ARE * ncb + e];
      if (t == B_INLET || t == B_OUTLET) {
        // facefluxuvw_boundary (faceflux_velocity.f90:403-468): only cb is used
        const double flomass = t == B_INLET ? F.fmi[b - bst_inl] : F.fmo[b - bst_out];
        const double dpn = bg[BG_DPB * ncb + e];
        const double de = F.vis[b] * are / dpn;
        const double cb = -de + rmin(flomass, 0.0);
        sp0 = sp0 - cb;
        sp1 = sp1 - cb;
        sp2 = sp2 - cb;
        s0 = s0 - cb * F.u[b];
        s1 = s1 - cb * F.v[b];
        s2 = s2 - cb * F.w[b];
      } else {
        const double nxf = bg[BG_NX * ncb + e], nyf = bg[BG_NY * ncb + e],
                     nzf = bg[BG_NZ * ncb + e];
        // dns / dnw and srds / srdw (init.f90:1002-1027)
        const double srd = bg[BG_SRD * ncb + e];
        const double dpb = bg[BG_DPB * ncb + e];
        const double upb = F.u[c] - F.u[b], vpb = F.v[c] - F.v[b], wpb = F.w[c] - F.w[b];
        if (t == B_SYMMETRY) {  // :268-306
          const double vsi = F.vis[b];
          const double cf = vsi * srd;
          const double vsol = vsi * are / dpb;
          const double fdne = 2.0 * cf * (upb * nxf + vpb * nyf + wpb * nzf);
          sp0 = sp0 + vsol;
          sp1 = sp1 + vsol;
          sp2 = sp2 + vsol;
          s0 = s0 + vsol * F.u[c] - fdne * nxf;
          s1 = s1 + vsol * F.v[c] - fdne * nyf;
          s2 = s2 + vsol * F.w[c] - fdne * nzf;
        } else {  // wall, :309-378 (laminar: viss = viscos)
          const double viss = prm.viscos;
          const double cf = viss * srd;
          const double vsol = viss * are / dpb;
          const double vnp = upb * nxf + vpb * nyf + wpb * nzf;
          const double utp = upb - vnp * nxf, vtp = vpb - vnp * nyf, wtp = wpb - vnp * nzf;
          sp0 = sp0 + vsol;
          sp1 = sp1 + vsol;
          sp2 = sp2 + vsol;
          s0 = s0 + vsol * F.u[c] - cf * utp;
          s1 = s1 + vsol * F.v[c] - cf * vtp;
          s2 = s2 + vsol * F.w[c] - cf * wtp;
        }
      }
    }
    // the diagonal the reference finds in a: halved with the rest of a under CN (:383)
    double d_in = a[m.diag[c]];
    if (prm.cn) d_in = 0.5 * d_in;
    const double apotime = prm.cn ? F.den[c] * vol / prm.timestep : 0.0;
    // u (:392-438)
    const double offu = row_sum(m, a, c, d_in) - d_in;
    if (prm.cn) {
      for (int e = e0; e < e1; ++e) {
        const int ent = m.cf_ent[e];
        const int f = (ent > 0 ? ent : -ent) - 1;
        const int o = ent > 0 ? m.neighbour[f] : m.owner[f];
        s0 = s0 - a[m.cf_slot[e]] * F.uo[o];
      }
      s0 = s0 + (apotime + offu) * F.uo[c];
      sp0 = sp0 + apotime;
    }
    double du = (sp0 - offu) * prm.urfr[0];
    rhs[c] = s0 + prm.urfm[0] * du * F.u[c];
    ap[c] = 1.0 / (du + small);
    // v (:447-495): its CN term sees the u diagonal; its diagonal assembly a zero one
    if (prm.cn) {
      for (int e = e0; e < e1; ++e) {
        const int ent = m.cf_ent[e];
        const int f = (ent > 0 ? ent : -ent) - 1;
        const int o = ent > 0 ? m.neighbour[f] : m.owner[f];
        s1 = s1 - a[m.cf_slot[e]] * F.vo[o];
      }
      s1 = s1 + (apotime + (row_sum(m, a, c, du) - du)) * F.vo[c];
      sp1 = sp1 + apotime;
    }
    // the v and w diagonals see a zero in place of the diagonal (x - 0.0 is x exactly)
    const double rs0 = row_sum(m, a, c, 0.0);
    const double dv = (sp1 - rs0) * prm.urfr[1];
    rhs[m.n + c] = s1 + prm.urfm[1] * dv * F.v[c];
    ap[m.n + c] = 1.0 / (dv + small);
    // w (:504-553): its CN term sees the v diagonal
    if (prm.cn) {
      for (int e = e0; e < e1; ++e) {
        const int ent = m.cf_ent[e];
        const int f = (ent > 0 ? ent : -ent) - 1;
        const int o = ent > 0 ? m.neighbour[f] : m.owner[f];
        s2 = s2 - a[m.cf_slot[e]] * F.wo[o];
      }
      s2 = s2 + (apotime + (row_sum(m, a, c, dv) - dv)) * F.wo[c];
      sp2 = sp2 + apotime;
    }
    const double dw = (sp2 - rs0) * prm.urfr[2];
    rhs[2 * m.n + c] = s2 + prm.urfm[2] * dw * F.w[c];
    ap[2 * m.n + c] = 1.0 / (dw + small);
    a[m.diag[c]] = du;
    diag_vw[c] = dv;
    diag_vw[m.n + c] = dw;
  }
}

}  // namespace

extern "C" int fcg_calcuvw(fcg_context *c, const fcg_uvw_params *prm, const fcg_uvw_fields *f,
                           double *a, double *diag_vw, double *rhs, double *ap) {
  if (!c || !prm || !f) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_calcuvw before fcg_bind_mesh");
  const bool need_old = prm->bdf || prm->cn;
  const bool need_oo = prm->bdf && prm->btime > (double)0.99f;
  const bool need_t = prm->buoyancy && prm->boussinesq;
  const int ninl = c->cnt[B_INLET], nout = c->cnt[B_OUTLET];
  if (!f->u || !f->v || !f->w || !f->p || !f->vis || !f->den || !f->dUdxi || !f->dVdxi ||
      !f->dWdxi || !f->dPdxi || (c->nin > 0 && !f->flmass) || (need_t && !f->t) ||
      (need_old && (!f->uo || !f->vo || !f->wo)) || (need_oo && (!f->uoo || !f->voo || !f->woo)) ||
      (ninl > 0 && !f->fmi) || (nout > 0 && !f->fmo) || !a || !diag_vw || !rhs || !ap)
    return set_error(c, FCG_ERR_ARG, "fcg_calcuvw: NULL array the parameters need");
  if (prm->scheme < FCG_CONV_CDS || prm->scheme > FCG_CONV_FLUX_LIMITER || prm->limiter < 0 ||
      prm->limiter > FCG_LIM_UDS)
    return set_error(c, FCG_ERR_ARG, "fcg_calcuvw: unknown scheme or limiter");
  if ((prm->bdf || prm->cn) && !(prm->timestep != 0.0))
    return set_error(c, FCG_ERR_ARG, "fcg_calcuvw: timestep must be nonzero");
  if (c->n < 3)
    return set_error(c, FCG_ERR_ARG,
                     "fcg_calcuvw: presFaceDivInner's df(ijp,3) index needs numCells >= 3");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t nt = sizeof(double) * c->ntot, n1 = sizeof(double) * c->n, n3 = 3 * n1;
  const size_t fb = sizeof(double) * (c->nin > 0 ? c->nin : 1);
  // flmass with the O-C pairs' fmoc after the inner faces' fluxes
  const size_t fbo = sizeof(double) * (c->nin + c->mv.noc > 0 ? c->nin + c->mv.noc : 1);
  struct In {
    const double *src;
    size_t bytes;
    bool need;
  } ins[] = {{f->u, nt, true},      {f->v, nt, true},        {f->w, nt, true},
             {f->p, nt, true},      {f->vis, nt, true},      {f->den, n1, true},
             {f->t, n1, need_t},    {f->uo, n1, need_old},   {f->vo, n1, need_old},
             {f->wo, n1, need_old}, {f->uoo, n1, need_oo},   {f->voo, n1, need_oo},
             {f->woo, n1, need_oo}, {f->dUdxi, n3, true},    {f->dVdxi, n3, true},
             {f->dWdxi, n3, true},  {f->dPdxi, n3, true},
             {f->flmass, fbo, c->nin + c->mv.noc > 0},
             {f->fmi, sizeof(double) * (ninl > 0 ? ninl : 1), ninl > 0},
             {f->fmo, sizeof(double) * (nout > 0 ? nout : 1), nout > 0}};
  const int NI = (int)(sizeof(ins) / sizeof(ins[0]));
  const double *dev[20] = {};
  int rc;
  for (int k = 0; k < NI; ++k) {
    if (!ins[k].need) continue;
    void *d;
    bool h;
    if ((rc = stage_in(c, ins[k].src, ins[k].bytes, k, true, &d, &h))) return rc;
    dev[k] = (const double *)d;
  }
  UvwView V{dev[0],  dev[1],  dev[2],  dev[3],  dev[4],  dev[5],  dev[6],
            dev[7],  dev[8],  dev[9],  dev[10], dev[11], dev[12], dev[13],
            dev[14], dev[15], dev[16], dev[17], dev[18], dev[19]};
  void *da, *ddv, *drhs, *dap;
  bool ha, hdv, hrhs, hap;
  const size_t alen = sizeof(double) * (size_t)a_len(c);  // with ar, al of the O-C pairs
  if ((rc = stage_in(c, a, alen, NI, true, &da, &ha)) ||
      (rc = stage_in(c, diag_vw, 2 * n1, NI + 1, false, &ddv, &hdv)) ||
      (rc = stage_in(c, rhs, n3, NI + 2, false, &drhs, &hrhs)) ||
      (rc = stage_in(c, ap, n3, NI + 3, false, &dap, &hap)))
    return rc;
  // face terms: 3 sources + 3 pressure-divergence terms per inner face and per O-C pair
  const size_t noc = (size_t)c->mv.noc;
  FCG_CUDA_TRY(c, c->scratch.ensure(6 * fb + 6 * sizeof(double) * (noc > 0 ? noc : 1)));
  double *fsrc = c->scratch.as<double>(), *fdiv = fsrc + 3 * (c->nin > 0 ? c->nin : 1);
  double *osrc = fdiv + 3 * (c->nin > 0 ? c->nin : 1), *odiv = osrc + 3 * (noc > 0 ? noc : 1);
  const MeshView &m = c->mv;
  if (m.noc > 0) {
    auto pairs = k_uvw_oc<FCG_CONV_MUSCL>;
    switch (prm->scheme) {
      case FCG_CONV_CDS: pairs = k_uvw_oc<FCG_CONV_CDS>; break;
      case FCG_CONV_CDS_CORRECTED: pairs = k_uvw_oc<FCG_CONV_CDS_CORRECTED>; break;
      case FCG_CONV_CENTRAL: pairs = k_uvw_oc<FCG_CONV_CENTRAL>; break;
      case FCG_CONV_SECOND_UPWIND: pairs = k_uvw_oc<FCG_CONV_SECOND_UPWIND>; break;
      case FCG_CONV_FLUX_LIMITER: pairs = k_uvw_oc<FCG_CONV_FLUX_LIMITER>; break;
      default: break;
    }
    pairs<<<grid_for(m.noc, c->num_sms), kTPB, 0, c->stream>>>(m, *prm, V, (double *)da, osrc,
                                                                 odiv);
    FCG_CHECK_LAUNCH(c, "k_uvw_oc");
  }
  if (m.nin > 0) {
    const double *geo;
    if ((rc = face_geo(c, &geo))) return rc;
    auto faces = k_uvw_faces<FCG_CONV_MUSCL>;
    switch (prm->scheme) {
      case FCG_CONV_CDS: faces = k_uvw_faces<FCG_CONV_CDS>; break;
      case FCG_CONV_CDS_CORRECTED: faces = k_uvw_faces<FCG_CONV_CDS_CORRECTED>; break;
      case FCG_CONV_CENTRAL: faces = k_uvw_faces<FCG_CONV_CENTRAL>; break;
      case FCG_CONV_SECOND_UPWIND: faces = k_uvw_faces<FCG_CONV_SECOND_UPWIND>; break;
      case FCG_CONV_FLUX_LIMITER: faces = k_uvw_faces<FCG_CONV_FLUX_LIMITER>; break;
      default: break;
    }
    faces<<<grid_for(m.nin, c->num_sms), kTPB, 0, c->stream>>>(m, *prm, V, geo, (double *)da,
                                                                 fsrc, fdiv);
    FCG_CHECK_LAUNCH(c, "k_uvw_faces");
  }
  const double *bg;
  if ((rc = bnd_geo(c, &bg))) return rc;
  long long ncb = 0;
  for (int t = 0; t < B_NTYPES; ++t) ncb += c->cnt[t];
  k_uvw_cells<<<grid_for(m.n, c->num_sms), kTPB, 0, c->stream>>>(
      m, *prm, V, c->bst[B_INLET], c->bst[B_OUTLET], bg, ncb, (double *)da, fsrc, fdiv, osrc,
      odiv, (double *)ddv, (double *)drhs, (double *)dap);
  FCG_CHECK_LAUNCH(c, "k_uvw_cells");
  if ((rc = stage_out(c, a, da, alen, ha)) ||
      (rc = stage_out(c, diag_vw, ddv, 2 * n1, hdv)) ||
      (rc = stage_out(c, rhs, drhs, n3, hrhs)) || (rc = stage_out(c, ap, dap, n3, hap)))
    return rc;
  if (ha || hdv || hrhs || hap) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}
