// The PISO corrector's own steps around the shared pressure kernels
// (PISO_multiple_correction.f90:83-307): HbyA (get_rAU_x_UEqnH.f90), the inlet/outlet
// mass balance (adjustMassFlow.f90), the reference-pressure row (:188-192) and the
// velocity correction (:300-304).  The pressure assembly itself (facefluxmass_piso) is
// in assembly.cu with the other face loops.
//
// Like assembly.cu this file is compiled with --fmad=false and sums every cell's terms
// in the reference's order, so the results are bit-identical to its loops: the face
// loops of the reference scatter into su(ijp) and su(ijn); here one thread per cell
// walks the cell's faces in ascending face order (MeshView::cf_*), which visits the same
// terms in the same order.
#include "fcg_internal.h"
#include "launch.h"

using namespace fcg;

namespace {

struct HbyaArgs {
  const double *h, *den, *t, *uo, *vo, *wo, *uoo, *voo, *woo, *u, *v, *w;
  double *su, *sv, *sw;
};

// su, sv, sw of get_rAU_x_UEqnH.f90:32-199 for every cell.
__global__ void k_hbya_sources(MeshView m, fcg_hbya_params prm, HbyaArgs A) {
  FCG_GRID_STRIDE(c, m.n) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;  // :32-34
    const double vol = m.vol[c];
    if (prm.buoyancy) {  // :42-56
      double heat;
      if (prm.boussinesq)
        heat = prm.beta * prm.densit * (A.t[c] - prm.tref) * vol;
      else
        heat = (prm.densit - A.den[c]) * vol;
      s0 = s0 - prm.gravx * heat;
      s1 = s1 - prm.gravy * heat;
      s2 = s2 - prm.gravz * heat;
    }
    if (prm.bdf) {  // :62-83
      const double apotime = A.den[c] * vol / prm.timestep;
      double sut = apotime * ((1.0 + prm.btime) * A.uo[c]);
      double svt = apotime * ((1.0 + prm.btime) * A.vo[c]);
      double swt = apotime * ((1.0 + prm.btime) * A.wo[c]);
      if (prm.btime > (double)0.99f) {  // a default-real literal in the reference
        sut = sut - apotime * (0.5 * prm.btime * A.uoo[c]);
        svt = svt - apotime * (0.5 * prm.btime * A.voo[c]);
        swt = swt - apotime * (0.5 * prm.btime * A.woo[c]);
      }
      s0 = s0 + sut;
      s1 = s1 + svt;
      s2 = s2 + swt;
    }
    const int e0 = m.cf_ptr[c], e1 = m.cf_ptr[c + 1];
    if (prm.cn) {  // :90-110 and its v, w twins: old-level neighbours, then the cell term
      for (int e = e0; e < e1; ++e) {
        const int ent = m.cf_ent[e];
        const int f = (ent > 0 ? ent : -ent) - 1;
        const int o = ent > 0 ? m.neighbour[f] : m.owner[f];
        const double hk = A.h[m.cf_slot[e]];
        s0 = s0 - hk * A.uo[o];
        s1 = s1 - hk * A.vo[o];
        s2 = s2 - hk * A.wo[o];
      }
      const double apotime = A.den[c] * vol / prm.timestep;
      double off = 0.0;  // sum(h(ioffset(c):ioffset(c+1)-1)), in row order
      for (int k = m.ioffset[c]; k < m.ioffset[c + 1]; ++k) off = off + A.h[k];
      off = off - A.h[m.diag[c]];
      s0 = s0 + (apotime + off) * A.uo[c];
      s1 = s1 + (apotime + off) * A.vo[c];
      s2 = s2 + (apotime + off) * A.wo[c];
    }
    for (int e = e0; e < e1; ++e) {  // H(U) = -sum_nb h(k) U_nb (:113-123)
      const int ent = m.cf_ent[e];
      const int f = (ent > 0 ? ent : -ent) - 1;
      const int o = ent > 0 ? m.neighbour[f] : m.owner[f];
      const double hk = A.h[m.cf_slot[e]];
      s0 = s0 - hk * A.u[o];
      s1 = s1 - hk * A.v[o];
      s2 = s2 - hk * A.w[o];
    }
    A.su[c] = s0;
    A.sv[c] = s1;
    A.sw[c] = s2;
  }
}

// u = apu*su, v = apv*sv, w = apw*sw on the cells (:204-206); a second launch, because
// the first reads the neighbours' old u, v, w.
__global__ void k_hbya_apply(int n, const double *__restrict__ apu, const double *__restrict__ apv,
                             const double *__restrict__ apw, const double *__restrict__ su,
                             const double *__restrict__ sv, const double *__restrict__ sw,
                             double *__restrict__ u, double *__restrict__ v,
                             double *__restrict__ w) {
  FCG_GRID_STRIDE(c, n) {
    u[c] = apu[c] * su[c];
    v[c] = apv[c] * sv[c];
    w[c] = apw[c] * sw[c];
  }
}

// su(owner) -= fmi over the inlet faces, then -= fmo over the outlet faces
// (adjustMassFlow.f90:15-24, 52-69), per cell in the reference's loop order.
__global__ void k_amf_su(MeshView m, const double *__restrict__ fmi,
                         const double *__restrict__ fmo, int bst_inl, int bst_out,
                         double *__restrict__ su) {
  FCG_GRID_STRIDE(c, m.n) {
    const int b0 = m.cb_ptr[c], b1 = m.cb_ptr[c + 1];
    if (b0 == b1) continue;
    double s = su[c];
    for (int e = b0; e < b1; ++e)
      if (m.cb_type[e] == B_INLET) s = s - fmi[m.cb_slot[e] - bst_inl];
    for (int e = b0; e < b1; ++e)
      if (m.cb_type[e] == B_OUTLET) s = s - fmo[m.cb_slot[e] - bst_out];
    su[c] = s;
  }
}

// a(ioffset(ref):ioffset(ref+1)-1) = 0, a(diag(ref)) = 1, su(ref) = p(ref)
// (PISO_multiple_correction.f90:188-192); one block.
__global__ void k_pref(MeshView m, int ref, const double *__restrict__ pref,
                       double *__restrict__ a, double *__restrict__ su) {
  const int lo = m.ioffset[ref], hi = m.ioffset[ref + 1];
  for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) a[k] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    a[m.diag[ref]] = 1.0;
    su[ref] = pref[0];
  }
}

// u -= apu*dPdxi(1)*vol, ... (PISO_multiple_correction.f90:300-304)
__global__ void k_correct_velocity_piso(MeshView m, const double *__restrict__ g,
                                        const double *__restrict__ apu,
                                        const double *__restrict__ apv,
                                        const double *__restrict__ apw, double *__restrict__ u,
                                        double *__restrict__ v, double *__restrict__ w) {
  FCG_GRID_STRIDE(i, m.n) {
    const double vol = m.vol[i];
    u[i] = u[i] - apu[i] * g[3 * i] * vol;
    v[i] = v[i] - apv[i] * g[3 * i + 1] * vol;
    w[i] = w[i] - apw[i] * g[3 * i + 2] * vol;
  }
}

}  // namespace

extern "C" int fcg_piso_hbya(fcg_context *c, const fcg_hbya_params *prm, const fcg_hbya_fields *f,
                             const double *h, double *u, double *v, double *w, double *su,
                             double *sv, double *sw) {
  if (!c || !prm || !f) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_piso_hbya before fcg_bind_mesh");
  const bool need_old = prm->bdf || prm->cn;
  const bool need_oo = prm->bdf && prm->btime > (double)0.99f;
  const bool need_t = prm->buoyancy && prm->boussinesq;
  const bool need_den = prm->bdf || prm->cn || (prm->buoyancy && !prm->boussinesq);
  if (!h || !u || !v || !w || !f->apu || !f->apv || !f->apw || (need_den && !f->den) ||
      (need_t && !f->t) || (need_old && (!f->uo || !f->vo || !f->wo)) ||
      (need_oo && (!f->uoo || !f->voo || !f->woo)))
    return set_error(c, FCG_ERR_ARG, "fcg_piso_hbya: NULL array the parameters need");
  if ((prm->bdf || prm->cn) && !(prm->timestep != 0.0))
    return set_error(c, FCG_ERR_ARG, "fcg_piso_hbya: timestep must be nonzero");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t n1 = sizeof(double) * c->n;
  HbyaArgs A{};
  int rc;
  void *d;
  bool hst;
  // inputs, cell parts only
  struct In {
    const double *src;
    const double **dst;
    bool need;
  } ins[] = {{f->den, &A.den, need_den}, {f->t, &A.t, need_t},     {f->uo, &A.uo, need_old},
             {f->vo, &A.vo, need_old},   {f->wo, &A.wo, need_old}, {f->uoo, &A.uoo, need_oo},
             {f->voo, &A.voo, need_oo},  {f->woo, &A.woo, need_oo}};
  int slot = 0;
  for (const In &x : ins) {
    if (!x.need) continue;
    if ((rc = stage_in(c, x.src, n1, slot++, true, &d, &hst))) return rc;
    *x.dst = (const double *)d;
  }
  const double *ap[3];
  const double *aps[3] = {f->apu, f->apv, f->apw};
  for (int k = 0; k < 3; ++k) {
    if ((rc = stage_in(c, aps[k], n1, slot++, true, &d, &hst))) return rc;
    ap[k] = (const double *)d;
  }
  if ((rc = stage_in(c, h, sizeof(double) * c->nnz, slot++, true, &d, &hst))) return rc;
  A.h = (const double *)d;
  double *vel[3] = {u, v, w};
  void *dvel[3];
  bool hvel[3];
  for (int k = 0; k < 3; ++k)
    if ((rc = stage_in(c, vel[k], n1, slot++, true, &dvel[k], &hvel[k]))) return rc;
  A.u = (const double *)dvel[0];
  A.v = (const double *)dvel[1];
  A.w = (const double *)dvel[2];
  double *srcs[3] = {su, sv, sw};
  void *dsrc[3];
  bool hsrc[3] = {false, false, false};
  FCG_CUDA_TRY(c, c->scratch.ensure(3 * n1 + 16));
  for (int k = 0; k < 3; ++k) {
    if (srcs[k]) {
      if ((rc = stage_in(c, srcs[k], n1, slot++, false, &dsrc[k], &hsrc[k]))) return rc;
    } else {
      dsrc[k] = c->scratch.as<double>() + (size_t)k * c->n;
    }
  }
  A.su = (double *)dsrc[0];
  A.sv = (double *)dsrc[1];
  A.sw = (double *)dsrc[2];
  const int G = grid_for(c->n, c->num_sms);
  k_hbya_sources<<<G, kTPB, 0, c->stream>>>(c->mv, *prm, A);
  FCG_CHECK_LAUNCH(c, "k_hbya_sources");
  k_hbya_apply<<<G, kTPB, 0, c->stream>>>(c->n, ap[0], ap[1], ap[2], A.su, A.sv, A.sw,
                                          (double *)dvel[0], (double *)dvel[1],
                                          (double *)dvel[2]);
  FCG_CHECK_LAUNCH(c, "k_hbya_apply");
  bool any = false;
  for (int k = 0; k < 3; ++k) {
    if ((rc = stage_out(c, vel[k], dvel[k], n1, hvel[k]))) return rc;
    if (srcs[k] && (rc = stage_out(c, srcs[k], dsrc[k], n1, hsrc[k]))) return rc;
    any = any || hvel[k] || hsrc[k];
  }
  if (any) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_adjust_mass_flow(fcg_context *c, const double *den, double flomas,
                                    const double *fmi, double *u, double *v, double *w,
                                    double *fmo, double *su) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_adjust_mass_flow before fcg_bind_mesh");
  const int ninl = c->cnt[B_INLET], nout = c->cnt[B_OUTLET];
  if (!den || !u || !v || !w || !su || (ninl > 0 && !fmi) || (nout > 0 && !fmo))
    return set_error(c, FCG_ERR_ARG, "NULL array");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t nt = sizeof(double) * c->ntot, n1 = sizeof(double) * c->n;
  void *dden, *du, *dv, *dw, *dsu, *dfmi = nullptr, *dfmo = nullptr;
  bool h0, hu, hv, hw, hsu, h1 = false, hfmo = false;
  int rc;
  if ((rc = stage_in(c, den, nt, 0, true, &dden, &h0))) return rc;
  if ((rc = stage_in(c, u, nt, 1, true, &du, &hu))) return rc;
  if ((rc = stage_in(c, v, nt, 2, true, &dv, &hv))) return rc;
  if ((rc = stage_in(c, w, nt, 3, true, &dw, &hw))) return rc;
  if ((rc = stage_in(c, su, n1, 4, true, &dsu, &hsu))) return rc;
  if (ninl > 0 && (rc = stage_in(c, fmi, sizeof(double) * ninl, 5, true, &dfmi, &h1))) return rc;
  if (nout > 0 && (rc = stage_in(c, fmo, sizeof(double) * nout, 6, false, &dfmo, &hfmo)))
    return rc;
  if ((rc = fcg::corr::outlet_flow(c, (const double *)dden, flomas, (double *)du, (double *)dv,
                                   (double *)dw, (double *)dfmo)))
    return rc;
  if (ninl > 0 || nout > 0) {
    k_amf_su<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(
        c->mv, (const double *)dfmi, (const double *)dfmo, c->bst[B_INLET], c->bst[B_OUTLET],
        (double *)dsu);
    FCG_CHECK_LAUNCH(c, "k_amf_su");
  }
  if ((rc = stage_out(c, u, du, nt, hu)) || (rc = stage_out(c, v, dv, nt, hv)) ||
      (rc = stage_out(c, w, dw, nt, hw)) || (rc = stage_out(c, su, dsu, n1, hsu)))
    return rc;
  if (nout > 0 && (rc = stage_out(c, fmo, dfmo, sizeof(double) * nout, hfmo))) return rc;
  if (hu || hv || hw || hsu || hfmo) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_set_reference_pressure(fcg_context *c, int pRefCell, const double *p,
                                          double *a, double *su) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound)
    return set_error(c, FCG_ERR_STATE, "fcg_set_reference_pressure before fcg_bind_mesh");
  if (!p || !a || !su) return set_error(c, FCG_ERR_ARG, "NULL array");
  if (pRefCell < 1 || pRefCell > c->n) return set_error(c, FCG_ERR_INDEX, "pRefCell out of range");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  void *dp, *da, *dsu;
  bool hp, ha, hsu;
  int rc;
  // only p(pRefCell) is read: stage that one value
  if ((rc = stage_in(c, p + (pRefCell - 1), sizeof(double), 0, true, &dp, &hp))) return rc;
  if ((rc = stage_in(c, a, sizeof(double) * c->nnz, 1, true, &da, &ha))) return rc;
  if ((rc = stage_in(c, su, sizeof(double) * c->n, 2, true, &dsu, &hsu))) return rc;
  k_pref<<<1, kTPB, 0, c->stream>>>(c->mv, pRefCell - 1, (const double *)dp, (double *)da,
                                    (double *)dsu);
  FCG_CHECK_LAUNCH(c, "k_pref");
  if ((rc = stage_out(c, a, da, sizeof(double) * c->nnz, ha)) ||
      (rc = stage_out(c, su, dsu, sizeof(double) * c->n, hsu)))
    return rc;
  if (ha || hsu) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_correct_velocity_piso(fcg_context *c, const double *dPdxi, const double *apu,
                                         const double *apv, const double *apw, double *u,
                                         double *v, double *w) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound)
    return set_error(c, FCG_ERR_STATE, "fcg_correct_velocity_piso before fcg_bind_mesh");
  if (!dPdxi || !apu || !apv || !apw || !u || !v || !w)
    return set_error(c, FCG_ERR_ARG, "NULL array");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t n1 = sizeof(double) * c->n;
  const void *in[4] = {dPdxi, apu, apv, apw};
  const size_t inb[4] = {3 * n1, n1, n1, n1};
  void *din[4];
  bool hin[4];
  int rc;
  for (int k = 0; k < 4; ++k)
    if ((rc = stage_in(c, in[k], inb[k], k, true, &din[k], &hin[k]))) return rc;
  double *out[3] = {u, v, w};
  void *dout[3];
  bool hout[3];
  for (int k = 0; k < 3; ++k)
    if ((rc = stage_in(c, out[k], n1, 4 + k, true, &dout[k], &hout[k]))) return rc;
  k_correct_velocity_piso<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(
      c->mv, (const double *)din[0], (const double *)din[1], (const double *)din[2],
      (const double *)din[3], (double *)dout[0], (double *)dout[1], (double *)dout[2]);
  FCG_CHECK_LAUNCH(c, "k_correct_velocity_piso");
  bool any = false;
  for (int k = 0; k < 3; ++k) {
    if ((rc = stage_out(c, out[k], dout[k], n1, hout[k]))) return rc;
    any = any || hout[k];
  }
  if (any) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}
