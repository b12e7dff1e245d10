// Mesh-constant factors of the inner faces, computed once per bound mesh (k_face_geo in
// assembly.cu) by the same rounded operations the face loops use, so that the loops that
// read them give the same bits as recomputing them: sqrt and divisions dominate those
// loops on this part's FP64 pipe.  Planar: plane q holds factor q of every inner face,
// g[q * nin + f].  P is the owner cell, N the neighbour, S = (arx, ary, arz) the face
// area vector, lambda = facint.
#pragma once

#include "fcg_internal.h"

namespace fcg {

enum FaceGeo {
  FG_NX, FG_NY, FG_NZ,    // unit normal S/|S|
  FG_SFDPNR,              // 1/(arx xpn nx + ary ypn ny + arz zpn nz)   (facefluxmass.f90:94)
  FG_SMDPN,               // |S|^2 sfdpnr                                (:95)
  FG_DPPNNR,              // 1/(xpn nx + ypn ny + zpn nz)                (facefluxmass.f90:578)
  FG_XPP, FG_YPP, FG_ZPP, // P' - P: (f - (f - P) n) - P                 (:155-172, :586-595)
  FG_XEP, FG_YEP, FG_ZEP, // N' - N
  FG_DXP, FG_DYP, FG_DZP, // face centre - P
  FG_DXQ, FG_DYQ, FG_DZQ, // face centre - N
  FG_XPN, FG_YPN, FG_ZPN, // N - P
  FG_ARE,                 // |S|
  FG_SMDPN_LAP,           // |S|^2 / (S . (N - P))                        (fvm_laplacian.f90:214)
  FG_DPN,                 // |N - P|                                     (facefluxmass.f90:334)
  FG_RVX, FG_RVY, FG_RVZ, // S / ((N - P) . S), componentwise           (gradients.f90:644, 666)
  FG_DXI, FG_DYI, FG_DZI, // face centre - (P (1 - lambda) + N lambda)  (fieldManipulation.f90:429-438)
  FG_COUNT
};

// The factors of the bound mesh, built at the first face loop that needs them.
int face_geo(fcg_context *c, const double **g);

// Mesh-constant factors of the boundary faces, per entry e of the cell->boundary-face
// lists (cb_*, the reference's boundary loop order), planar b[q * ncb + e], from the
// face centre f and the owner cell's centre C (init.f90:1002-1027, calcuvw.f90:223-378).
enum BndGeo {
  BG_ARE,                 // |S|
  BG_DPB,                 // |C - f| (= |f - C|: the squares are equal)
  BG_NX, BG_NY, BG_NZ,    // unit normal S/|S|
  BG_SRD,                 // |S| / ((f - C) . n)
  BG_COUNT
};

int bnd_geo(fcg_context *c, const double **b);

}  // namespace fcg
