// Detection of a lexicographic hexahedral block in the bound mesh (no reference
// counterpart: the reference treats every mesh as unstructured).
//
// A mesh qualifies when its cells can be read as an nx x ny x nz block, cell
// r = i + nx j + nx ny k, with every CSR row holding exactly the cell and its face
// neighbours inside the block (the hex meshes of the benchmark, and any structured hex
// mesh numbered the same way).  Row 0 is a corner cell: its columns 0, 1, nx, nx ny give
// the extents; one kernel then checks every row.  Kernels that have a block-structured
// form (the plane-staged network layer, the wavefront-tiled triangular sweeps) use it;
// all others, and every other mesh, keep the general sliced / level-scheduled forms.
#include <cuda_runtime.h>

#include "fcg_internal.h"
#include "launch.h"

namespace fcg {
namespace {

// Counts the rows whose entries are not exactly {lower neighbours in the block, the
// row, upper neighbours in the block} in column order.
__global__ void k_hex_block_check(int n, const int *__restrict__ io, const int *__restrict__ ja,
                                  int nx, int ny, int nz, int *bad) {
  const long long nxy = (long long)nx * ny;
  FCG_GRID_STRIDE(r, n) {
    const int i = (int)(r % nx), j = (int)((r / nx) % ny), k = (int)(r / nxy);
    long long want[7];
    int m = 0;
    if (k > 0) want[m++] = r - nxy;
    if (j > 0) want[m++] = r - nx;
    if (i > 0) want[m++] = r - 1;
    want[m++] = r;
    if (i < nx - 1) want[m++] = r + 1;
    if (j < ny - 1) want[m++] = r + nx;
    if (k < nz - 1) want[m++] = r + nxy;
    bool good = io[r + 1] - io[r] == m;
    for (int e = 0; good && e < m; ++e) good = ja[io[r] + e] == want[e];
    if (!good) atomicAdd(bad, 1);
  }
}

}  // namespace

int detect_hex_block(fcg_context *c) {
  c->hex = HexBlock();
  const int n = c->n;
  if (n < 8) return FCG_OK;
  int io[2] = {0, 0};
  FCG_CUDA_TRY(c, cudaMemcpyAsync(io, c->mv.ioffset, sizeof io, cudaMemcpyDeviceToHost, c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (io[1] - io[0] != 4) return FCG_OK;  // a corner cell: itself and three neighbours
  int col[4];
  FCG_CUDA_TRY(c, cudaMemcpyAsync(col, c->mv.ja + io[0], sizeof col, cudaMemcpyDeviceToHost,
                                  c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const long long nx = col[2], nxy = col[3];
  if (col[0] != 0 || col[1] != 1 || nx < 2 || nxy <= nx || nxy % nx != 0 || n % nxy != 0)
    return FCG_OK;
  const long long ny = nxy / nx, nz = n / nxy;
  if (ny < 2 || nz < 2) return FCG_OK;
  FCG_CUDA_TRY(c, c->scratch.ensure(64));
  int *bad = c->scratch.as<int>();
  FCG_CUDA_TRY(c, cudaMemsetAsync(bad, 0, sizeof(int), c->stream));
  k_hex_block_check<<<grid_for(n, c->num_sms), kTPB, 0, c->stream>>>(
      n, c->mv.ioffset, c->mv.ja, (int)nx, (int)ny, (int)nz, bad);
  FCG_CHECK_LAUNCH(c, "k_hex_block_check");
  int nbad = -1;
  FCG_CUDA_TRY(c, cudaMemcpyAsync(&nbad, bad, sizeof nbad, cudaMemcpyDeviceToHost, c->stream));
  FCG_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (nbad != 0) return FCG_OK;
  c->hex.nx = (int)nx;
  c->hex.ny = (int)ny;
  c->hex.nz = (int)nz;
  c->hex.ok = true;
  return FCG_OK;
}

}  // namespace fcg
