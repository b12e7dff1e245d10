// Cell-centred gradients and boundary values: grad_gauss (grad_gauss.f90),
// grad_gauss_corrected (grad_gauss_corrected.f90), grad_lsq (grad_lsq.f90) and
// bpres (bpres.f90).
//
// Gauss: one thread per inner face computes the interpolated face value times the
// area vector (gradco :128-190) into a face array; one thread per cell then adds its
// inner faces in face order (+ as owner, - as neighbour), its boundary faces in the
// reference's boundary-loop order (gradbc :194-211) and scales by 1/vol.  LSQ: one
// thread per cell gathers the same per-face terms the reference scatters.  Compiled
// with --fmad=false, so results are bit-identical to the Fortran loops.
#include "fcg_internal.h"
#include "launch.h"

using namespace fcg;

namespace {

// gradco: face value with the old gradient interpolated to the point on PN.
__global__ void k_gauss_faces(MeshView m, const double *__restrict__ fi,
                              const double *__restrict__ gold, double *__restrict__ dfe) {
  FCG_GRID_STRIDE(f, m.nin) {
    int p = m.owner[f], q = m.neighbour[f];
    double fxn = m.facint[f];
    double fxp = 1.0 - fxn;
    double xi = m.xc[p] * fxp + m.xc[q] * fxn;
    double yi = m.yc[p] * fxp + m.yc[q] * fxn;
    double zi = m.zc[p] * fxp + m.zc[q] * fxn;
    double dfxi = gold[3 * p] * fxp + gold[3 * q] * fxn;
    double dfyi = gold[3 * p + 1] * fxp + gold[3 * q + 1] * fxn;
    double dfzi = gold[3 * p + 2] * fxp + gold[3 * q + 2] * fxn;
    double fie = fi[p] * fxp + fi[q] * fxn + dfxi * (m.xf[f] - xi) + dfyi * (m.yf[f] - yi) +
                 dfzi * (m.zf[f] - zi);
    dfe[f] = fie * m.arx[f];
    dfe[m.nin + f] = fie * m.ary[f];
    dfe[2LL * m.nin + f] = fie * m.arz[f];
  }
}

// The same on the O-C pairs (grad_gauss.f90:60-67): face ijlFace(i), factor foc(i).
__global__ void k_gauss_oc(MeshView m, const double *__restrict__ fi,
                           const double *__restrict__ gold, double *__restrict__ dfo) {
  FCG_GRID_STRIDE(i, m.noc) {
    const int p = m.oc_l[i], q = m.oc_r[i], f = m.oc_fl[i];
    double fxn = m.oc_foc[i];
    double fxp = 1.0 - fxn;
    double xi = m.xc[p] * fxp + m.xc[q] * fxn;
    double yi = m.yc[p] * fxp + m.yc[q] * fxn;
    double zi = m.zc[p] * fxp + m.zc[q] * fxn;
    double dfxi = gold[3 * p] * fxp + gold[3 * q] * fxn;
    double dfyi = gold[3 * p + 1] * fxp + gold[3 * q + 1] * fxn;
    double dfzi = gold[3 * p + 2] * fxp + gold[3 * q + 2] * fxn;
    double fie = fi[p] * fxp + fi[q] * fxn + dfxi * (m.xf[f] - xi) + dfyi * (m.yf[f] - yi) +
                 dfzi * (m.zf[f] - zi);
    dfo[i] = fie * m.arx[f];
    dfo[m.noc + i] = fie * m.ary[f];
    dfo[2LL * m.noc + i] = fie * m.arz[f];
  }
}

__global__ void k_gauss_cells(MeshView m, const double *__restrict__ fi,
                              const double *__restrict__ dfe, const double *__restrict__ dfo,
                              double *__restrict__ g) {
  FCG_GRID_STRIDE(c, m.n) {
    double gx = 0.0, gy = 0.0, gz = 0.0;
    for (int e = m.cf_ptr[c]; e < m.cf_ptr[c + 1]; ++e) {
      int ent = m.cf_ent[e];
      long long f = (ent > 0 ? ent : -ent) - 1;
      double ex = dfe[f], ey = dfe[m.nin + f], ez = dfe[2LL * m.nin + f];
      if (ent > 0) {
        gx = gx + ex;
        gy = gy + ey;
        gz = gz + ez;
      } else {
        gx = gx - ex;
        gy = gy - ey;
        gz = gz - ez;
      }
    }
    if (m.noc)  // the O-C pairs after the inner faces, + on the left cell, - on the right
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) {
        const int v = m.oc_vix[e];
        const long long i = v < m.noc ? v : v - m.noc;
        double ex = dfo[i], ey = dfo[m.noc + i], ez = dfo[2LL * m.noc + i];
        if (v < m.noc) {
          gx = gx + ex;
          gy = gy + ey;
          gz = gz + ez;
        } else {
          gx = gx - ex;
          gy = gy - ey;
          gz = gz - ez;
        }
      }
    for (int e = m.cb_ptr[c]; e < m.cb_ptr[c + 1]; ++e) {
      int f = m.cb_face[e];
      double fb = fi[m.cb_slot[e]];
      gx = gx + fb * m.arx[f];
      gy = gy + fb * m.ary[f];
      gz = gz + fb * m.arz[f];
    }
    double volr = 1.0 / m.vol[c];
    g[3 * c] = gx * volr;
    g[3 * c + 1] = gy * volr;
    g[3 * c + 2] = gz * volr;
  }
}

// grad_lsq stage 1: D = sum d d^T over inner faces (face order) and boundary faces
// (face order), then the scaled cofactors (:134-165).
__global__ void k_lsq_matrix(MeshView m, double *__restrict__ dmat) {
  FCG_GRID_STRIDE(c, m.n) {
    double d11 = 0.0, d12 = 0.0, d13 = 0.0, d22 = 0.0, d23 = 0.0, d33 = 0.0;
    for (int e = m.cf_ptr[c]; e < m.cf_ptr[c + 1]; ++e) {
      int ent = m.cf_ent[e];
      int f = (ent > 0 ? ent : -ent) - 1;
      int p = m.owner[f], q = m.neighbour[f];
      double Dx = m.xc[q] - m.xc[p], Dy = m.yc[q] - m.yc[p], Dz = m.zc[q] - m.zc[p];
      d11 = d11 + Dx * Dx;
      d22 = d22 + Dy * Dy;
      d33 = d33 + Dz * Dz;
      d12 = d12 + Dx * Dy;
      d13 = d13 + Dx * Dz;
      d23 = d23 + Dy * Dz;
    }
    if (m.noc)  // the O-C pairs (:85-108)
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) {
        const int v = m.oc_vix[e], i = v < m.noc ? v : v - m.noc;
        const int p = m.oc_l[i], q = m.oc_r[i];
        double Dx = m.xc[q] - m.xc[p], Dy = m.yc[q] - m.yc[p], Dz = m.zc[q] - m.zc[p];
        d11 = d11 + Dx * Dx;
        d22 = d22 + Dy * Dy;
        d33 = d33 + Dz * Dz;
        d12 = d12 + Dx * Dy;
        d13 = d13 + Dx * Dz;
        d23 = d23 + Dy * Dz;
      }
    for (int e = m.cbf_ptr[c]; e < m.cbf_ptr[c + 1]; ++e) {
      int f = m.cbf_face[e];
      double Dx = m.xf[f] - m.xc[c], Dy = m.yf[f] - m.yc[c], Dz = m.zf[f] - m.zc[c];
      d11 = d11 + Dx * Dx;
      d22 = d22 + Dy * Dy;
      d33 = d33 + Dz * Dz;
      d12 = d12 + Dx * Dy;
      d13 = d13 + Dx * Dz;
      d23 = d23 + Dy * Dz;
    }
    double d21 = d12, d31 = d13, d32 = d23;
    double tmp = 1.0 / (d11 * d22 * d33 - d11 * d23 * d32 - d12 * d21 * d33 + d12 * d23 * d31 +
                        d13 * d21 * d32 - d13 * d22 * d31);
    double *D = dmat + 9 * c;
    D[0] = (d22 * d33 - d23 * d32) * tmp;
    D[1] = (d21 * d33 - d23 * d31) * tmp;
    D[2] = (d21 * d32 - d22 * d31) * tmp;
    D[3] = (d11 * d33 - d13 * d31) * tmp;
    D[4] = (d12 * d33 - d13 * d32) * tmp;
    D[5] = (d11 * d32 - d12 * d31) * tmp;
    D[6] = (d12 * d23 - d13 * d22) * tmp;
    D[7] = (d11 * d23 - d13 * d21) * tmp;
    D[8] = (d11 * d22 - d12 * d21) * tmp;
  }
}

// grad_lsq stage 2 (:168-306).
__global__ void k_lsq_cells(MeshView m, const double *__restrict__ fi,
                            const double *__restrict__ dmat, double *__restrict__ g) {
  FCG_GRID_STRIDE(c, m.n) {
    double b1 = 0.0, b2 = 0.0, b3 = 0.0;
    for (int e = m.cf_ptr[c]; e < m.cf_ptr[c + 1]; ++e) {
      int ent = m.cf_ent[e];
      int f = (ent > 0 ? ent : -ent) - 1;
      int p = m.owner[f], q = m.neighbour[f];
      double df = fi[q] - fi[p];
      b1 = b1 + (m.xc[q] - m.xc[p]) * df;
      b2 = b2 + (m.yc[q] - m.yc[p]) * df;
      b3 = b3 + (m.zc[q] - m.zc[p]) * df;
    }
    if (m.noc)  // the O-C pairs (:198-214)
      for (int e = m.oc_cptr[c]; e < m.oc_cptr[c + 1]; ++e) {
        const int v = m.oc_vix[e], i = v < m.noc ? v : v - m.noc;
        const int p = m.oc_l[i], q = m.oc_r[i];
        double df = fi[q] - fi[p];
        b1 = b1 + (m.xc[q] - m.xc[p]) * df;
        b2 = b2 + (m.yc[q] - m.yc[p]) * df;
        b3 = b3 + (m.zc[q] - m.zc[p]) * df;
      }
    for (int e = m.cb_ptr[c]; e < m.cb_ptr[c + 1]; ++e) {
      int f = m.cb_face[e];
      double df = fi[m.cb_slot[e]] - fi[c];
      b1 = b1 + df * (m.xf[f] - m.xc[c]);
      b2 = b2 + df * (m.yf[f] - m.yc[c]);
      b3 = b3 + df * (m.zf[f] - m.zc[c]);
    }
    const double *D = dmat + 9 * c;
    g[3 * c] = b1 * D[0] - b2 * D[1] + b3 * D[2];
    g[3 * c + 1] = b1 * D[3] - b2 * D[4] - b3 * D[5];
    g[3 * c + 2] = b1 * D[6] - b2 * D[7] + b3 * D[8];
  }
}

// bpres: one thread per boundary face listed by type; each writes its own slot.
__global__ void k_bpres(MeshView m, long long nbent, double *__restrict__ p,
                        const double *__restrict__ dP, int istage) {
  FCG_GRID_STRIDE(e, nbent) {
    int f = m.cb_face[e], c = m.owner[f], slot = m.cb_slot[e], t = m.cb_type[e];
    if (istage == 1) {
      p[slot] = p[c];  // :37-96
    } else if (t == B_WALL || t == B_PRESSOUT) {  // :102-132
      double xpb = m.xf[f] - m.xc[c], ypb = m.yf[f] - m.yc[c], zpb = m.zf[f] - m.zc[c];
      p[slot] = p[c] + dP[3 * c] * xpb + dP[3 * c + 1] * ypb + dP[3 * c + 2] * zpb;
    }
  }
}

// bpres on the O-C slots (:89-95, :134-148): slot s0 + i takes the value of the owner of
// face iOCFacesStart + i; from stage 2 on, extrapolated over the distance from the
// centre of face i, as :140-142 write it.
__global__ void k_bpres_oc(MeshView m, long long s0, double *__restrict__ p,
                           const double *__restrict__ dP, int istage) {
  FCG_GRID_STRIDE(i, m.noc) {
    const int c = m.owner[m.oc_start + i];
    if (istage == 1) {
      p[s0 + i] = p[c];
    } else {
      double xpb = m.xf[i] - m.xc[c], ypb = m.yf[i] - m.yc[c], zpb = m.zf[i] - m.zc[c];
      p[s0 + i] = p[c] + dP[3 * c] * xpb + dP[3 * c + 1] * ypb + dP[3 * c + 2] * zpb;
    }
  }
}

int ensure_lsq_matrix(fcg_context *c) {
  if (c->dmat_ready) return FCG_OK;
  FCG_CUDA_TRY(c, c->dmat.ensure(sizeof(double) * 9 * (size_t)c->n));
  k_lsq_matrix<<<grid_for(c->n, c->num_sms), kTPB, 0, c->stream>>>(c->mv, c->dmat.as<double>());
  FCG_CHECK_LAUNCH(c, "k_lsq_matrix");
  c->dmat_ready = true;
  return FCG_OK;
}

}  // namespace

extern "C" int fcg_grad_lsq_matrix(fcg_context *c, double *dmat) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_grad_lsq_matrix before fcg_bind_mesh");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  c->dmat_ready = false;
  int rc = ensure_lsq_matrix(c);
  if (rc) return rc;
  if (dmat) {
    FCG_CUDA_TRY(c, cudaMemcpyAsync(dmat, c->dmat.p, sizeof(double) * 9 * (size_t)c->n,
                                    cudaMemcpyDefault, c->stream));
    FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  return FCG_OK;
}

extern "C" int fcg_grad(fcg_context *c, const double *phi, double *dPhidxi, int method,
                        int nigrad) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_grad before fcg_bind_mesh");
  if (method != FCG_GRAD_GAUSS && method != FCG_GRAD_GAUSS_CORRECTED && method != FCG_GRAD_LSQ)
    return set_error(c, FCG_ERR_ARG, "unknown gradient method");
  if (method == FCG_GRAD_GAUSS && nigrad < 1)
    return set_error(c, FCG_ERR_ARG, "nigrad must be >= 1");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t n3 = sizeof(double) * 3 * (size_t)c->n;
  void *dphi, *dg;
  bool hphi, hg;
  int rc;
  if ((rc = stage_in(c, phi, sizeof(double) * c->ntot, 0, true, &dphi, &hphi))) return rc;
  if ((rc = stage_in(c, dPhidxi, n3, 1, method == FCG_GRAD_GAUSS_CORRECTED, &dg, &hg))) return rc;
  const MeshView &m = c->mv;
  const int gf = grid_for(m.nin, c->num_sms), gc = grid_for(m.n, c->num_sms);
  if (method == FCG_GRAD_LSQ) {
    if ((rc = ensure_lsq_matrix(c))) return rc;
    k_lsq_cells<<<gc, kTPB, 0, c->stream>>>(m, (const double *)dphi, c->dmat.as<double>(),
                                            (double *)dg);
    FCG_CHECK_LAUNCH(c, "k_lsq_cells");
  } else {
    // scratch: dfe[3*nin] | old gradient [3n] | new gradient [3n] | O-C terms [3*noc]
    size_t nin3 = 3 * (size_t)(m.nin > 0 ? m.nin : 1), noc3 = 3 * (size_t)m.noc;
    FCG_CUDA_TRY(c, c->scratch.ensure(sizeof(double) * (nin3 + noc3) + 2 * n3));
    double *dfe = c->scratch.as<double>();
    double *gA = dfe + nin3, *gB = gA + 3 * (size_t)m.n;
    double *dfo = gB + 3 * (size_t)m.n;
    int passes = method == FCG_GRAD_GAUSS_CORRECTED ? 1 : nigrad;
    const double *gold = gA;
    if (method == FCG_GRAD_GAUSS_CORRECTED) {
      gold = (const double *)dg;  // old gradient = incoming (grad_gauss_corrected.f90:38-40)
    } else {
      FCG_CUDA_TRY(c, cudaMemsetAsync(gA, 0, n3, c->stream));  // grad_gauss.f90:38-40
    }
    for (int lc = 1; lc <= passes; ++lc) {
      double *gnew = (gold == gA) ? gB : gA;  // never the buffer the pass reads
      if (m.nin > 0) {
        k_gauss_faces<<<gf, kTPB, 0, c->stream>>>(m, (const double *)dphi, gold, dfe);
        FCG_CHECK_LAUNCH(c, "k_gauss_faces");
      }
      if (m.noc > 0) {
        k_gauss_oc<<<grid_for(m.noc, c->num_sms), kTPB, 0, c->stream>>>(m, (const double *)dphi,
                                                                         gold, dfo);
        FCG_CHECK_LAUNCH(c, "k_gauss_oc");
      }
      k_gauss_cells<<<gc, kTPB, 0, c->stream>>>(m, (const double *)dphi, dfe, dfo, gnew);
      FCG_CHECK_LAUNCH(c, "k_gauss_cells");
      gold = gnew;  // :116-120
    }
    FCG_CUDA_TRY(c, cudaMemcpyAsync(dg, gold, n3, cudaMemcpyDeviceToDevice, c->stream));
  }
  if ((rc = stage_out(c, dPhidxi, dg, n3, hg))) return rc;
  if (hg) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}

extern "C" int fcg_bpres(fcg_context *c, double *p, const double *dPdxi, int istage) {
  if (!c) return FCG_ERR_ARG;
  if (!c->bound) return set_error(c, FCG_ERR_STATE, "fcg_bpres before fcg_bind_mesh");
  if (istage < 1) return set_error(c, FCG_ERR_ARG, "istage must be >= 1");
  FCG_CUDA_TRY(c, cudaSetDevice(c->device));
  void *dp, *dg = nullptr;
  bool hp, hg = false;
  int rc;
  if ((rc = stage_in(c, p, sizeof(double) * c->ntot, 0, true, &dp, &hp))) return rc;
  if (istage >= 2) {
    if ((rc = stage_in(c, dPdxi, sizeof(double) * 3 * (size_t)c->n, 1, true, &dg, &hg))) return rc;
  }
  long long nbent = 0;
  for (int t = 0; t < B_NTYPES; ++t) nbent += c->cnt[t];
  if (nbent > 0) {
    k_bpres<<<grid_for(nbent, c->num_sms), kTPB, 0, c->stream>>>(c->mv, nbent, (double *)dp,
                                                                   (const double *)dg, istage);
    FCG_CHECK_LAUNCH(c, "k_bpres");
  }
  if (c->mv.noc > 0) {  // the O-C slots follow the typed ones (iOCStart, :603)
    k_bpres_oc<<<grid_for(c->mv.noc, c->num_sms), kTPB, 0, c->stream>>>(
        c->mv, (long long)c->n + nbent, (double *)dp, (const double *)dg, istage);
    FCG_CHECK_LAUNCH(c, "k_bpres_oc");
  }
  if ((rc = stage_out(c, p, dp, sizeof(double) * c->ntot, hp))) return rc;
  if (hp) FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return FCG_OK;
}
