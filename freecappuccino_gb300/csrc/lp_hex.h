// Plane-staged message-passing layer for meshes whose cells form a lexicographic
// nx x ny x nz hexahedral block (learned_hex.cu).  Host-side interface used by
// learned.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "fcg_internal.h"

namespace fcg {
namespace lphex {

// Cell r = i + nx*j + nx*ny*k.  nxp = nx rounded up to a multiple of 4 (the row pitch of
// the stencil value planes, so that every TMA stride is a multiple of 16 bytes).
struct HexGrid {
  int nx = 0, ny = 0, nz = 0, nxp = 0;
  bool ok = false;
};

// The grid of the plane-staged layer for c's mesh: g->ok when the mesh is a lexicographic
// hex block (c->hex, found at bind time) and the driver accepts the tensor maps.  Call
// it outside stream capture: it also sets the layer kernel's shared-memory limit on c's
// device.
int detect(fcg_context *c, HexGrid *g);

// Floats of the stencil value planes: 7 directions x nz x ny x nxp.
inline size_t value_count(const HexGrid &g) { return 7ull * g.nz * g.ny * g.nxp; }

// Stencil values of the FP32 scaled matrix (the sliced layout the solvers use):
// val[d][k][j][i] for the directions d = -nx*ny, -nx, -1, 0, +1, +nx, +nx*ny (the CSR
// column order of every row), 0 where the row has no such entry.  The padding columns
// i >= nx must be zero already (they are never written).
cudaError_t values(const fcg_context *c, const HexGrid &g, const float *aval, float *val,
                   cudaStream_t st);

// The network's output fused into its last layer: z = r + rms (w_out . h_L + b_out) per
// cell, with wout = [w_out (C values), b_out] and rms a device scalar.  h_L itself is
// then not stored.
struct OutFuse {
  const float *r, *rms, *wout;
  float *z;
};

// One layer h_out = h_in + relu(W_l [h_in; Ahat h_in] + b_l) for all cells, the same
// bits as the sliced gather form.  With `out` given, the kernel writes the output z of
// OutFuse from the layer's tiles instead of h_out, the same bits as the output kernel
// on h_out, and sets *fused; *fused stays false when the form launched cannot fuse it
// (the caller then runs the output kernel).  Returns cudaErrorInvalidValue without
// launching when the driver refuses the tensor maps (the caller then runs the gather
// form), else the launch error, which stays set for the caller's own check.  An
// mbarrier wait that gives up (after 1 s) stores FCG_ERR_TIMEOUT into *status (when
// status is not NULL).
cudaError_t layer(const HexGrid &g, int num_sms, const __nv_bfloat16 *hin, __nv_bfloat16 *hout,
                  const float *val, const __nv_bfloat16 *wl, const float *bl, const int *done,
                  int *status, cudaStream_t st, const OutFuse *out = nullptr,
                  bool *fused = nullptr);

}  // namespace lphex
}  // namespace fcg
