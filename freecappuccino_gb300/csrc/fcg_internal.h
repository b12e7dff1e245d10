// Internal state of an fcg_context and the views the kernels receive.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../../include/fcgpu.h"

namespace fcg {

// Boundary types in the reference's loop order (grad_gauss.f90:70-103, bpres.f90:41-96).
enum BType { B_INLET = 0, B_OUTLET = 1, B_SYMMETRY = 2, B_WALL = 3, B_PRESSOUT = 4, B_NTYPES = 5 };

// A growable device allocation owned by the context.
struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t need) {
    if (need <= bytes && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, need ? need : 16);
    if (e == cudaSuccess) bytes = need ? need : 16;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T *as() const { return (T *)p; }
};

// Device-side mesh and pattern, passed by value to kernels.  All indices 0-based.
struct MeshView {
  int n, nf, nin, ntot;
  long long nnz;
  const int *owner, *neighbour;
  const double *arx, *ary, *arz, *xf, *yf, *zf;
  const double *xc, *yc, *zc, *vol, *facint;
  const int *ioffset, *ja, *diag, *slot_pn, *slot_np;
  // inner-face incidence per cell, ascending face order: ent = f+1 (owner) or -(f+1)
  // (neighbour); slot = CSR position of this cell's row entry for that face.
  const int *cf_ptr, *cf_ent, *cf_slot;
  // boundary faces per cell in the reference's boundary loop order (type, then index)
  const int *cb_ptr, *cb_face, *cb_slot, *cb_type;
  // boundary faces per cell in face order (grad_lsq.f90:116-130)
  const int *cbf_ptr, *cbf_face;
  // O-C grid cuts and cyclic faces (mesh_geometry_and_topology.f90:453-462, 800-845):
  // noc pairs, the last ncyc cyclic; pair i couples cell oc_l[i] (owner of its left
  // face oc_fl[i]) to oc_r[i] (owner of the friend face oc_fr[i]), with the area of
  // face oc_start + i (fvm_laplacian.f90:70).  Per cell, its pair entries in pair order
  // (oc_cptr): the coupled cell oc_col and the position oc_vix of the coefficient after
  // the CSR values of a matrix (ar(i) at i for the left cell, al(i) at noc + i for the
  // right).  noc = 0 and null pointers for a mesh without them.
  int noc, ncyc, oc_start;
  const int *oc_l, *oc_r, *oc_fl, *oc_fr;
  const double *oc_foc, *oc_srdoc;
  const int *oc_cptr, *oc_col, *oc_vix;
};

// The O-C couplings of one matrix for the solver kernels (the per-cell lists of the
// MeshView and the coefficients after the CSR values); ptr == nullptr: none.
struct OcView {
  const int *ptr, *col, *vix;
  const double *val;
};

// Sliced-ELL copy of the CSR pattern used by the solvers: slices of 32 rows stored
// column-major inside the slice, so that a warp reads one slot of 32 consecutive rows
// per load.  A uniform slice (kind 0) keeps one column offset per slot (off[offp+j]):
// slot j of row r reads column r + off[offp+j], clamped into range, with value 0 where
// the row has no such entry.  An explicit slice (kind 1) keeps 32 columns per slot at
// off[offp + 32*j + lane] (pads: the row itself, value 0).
struct SellView {
  int nslices;
  const long long *ptr; // [nslices+1] value offset of each slice
  const int *width;     // [nslices] slots per row
  const int *kind;      // [nslices] 0 uniform, 1 explicit
  const int *offp;      // [nslices] start of the slice's offsets or column block in off
  const int *off;       // offsets (uniform) and explicit column blocks
  const int *src;       // [len] CSR position of each value slot (-1: no entry)
};

// A mesh whose cells form a lexicographic nx x ny x nz hexahedral block: cell
// r = i + nx j + nx ny k, and row r of the CSR pattern holds exactly the cell itself and
// its face neighbours inside the block, so the lower entries of a row are (when present)
// -nx ny, -nx, -1 and the upper ones +1, +nx, +nx ny, in that order.  Found at bind time
// (hexblock.cu); kernels with a plane-staged or wavefront-tiled form use it.
struct HexBlock {
  int nx = 0, ny = 0, nz = 0;
  bool ok = false;
};

struct Level {
  std::vector<int> ptr;  // host: level offsets into rows
  int *rows = nullptr;   // device: rows sorted by level, ascending inside a level
  int count = 0;
  // device: the same list with every level padded with -1 to a multiple of 32 entries,
  // so a warp's 32 consecutive entries never span two levels (sync-free sweeps)
  int *pad = nullptr;
  int pad_len = 0;
};

}  // namespace fcg

namespace fcg {
struct KrylovState;
void destroy_krylov(KrylovState *k);
struct MultiState;
void destroy_multi(MultiState *m);
}  // namespace fcg

struct fcg_context {
  unsigned long long uid = 0;  // unique per process: handles key cached state on it
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaEvent_t switch_ev = nullptr;  // orders a new stream after the old (fcg_set_stream)
  std::string err;
  bool bound = false;
  unsigned bind_gen = 0;  // bumped by every fcg_bind_mesh; captured graphs depend on it

  // sizes
  int n = 0, nf = 0, nin = 0, nb = 0, ntot = 0;
  long long nnz = 0;
  int cnt[fcg::B_NTYPES] = {0}, fst[fcg::B_NTYPES] = {0}, bst[fcg::B_NTYPES] = {0};


  // device allocations made by fcg_bind_mesh (mesh arrays and topology)
  std::vector<fcg::DBuf> bound_allocs;
  fcg::MeshView mv{};
  fcg::SellView sv{};
  int sell_maxw = 0;
  long long sell_len = 0, sell_nuniform = 0;
  fcg::Level lf, lb;  // forward (lower) and backward (upper) level schedules
  fcg::HexBlock hex;  // the block structure of the cell numbering, when it has one
  const int *tpos = nullptr;  // CSR position of the transpose entry of every entry
  // every topology array bound to the device (pointer, bytes), for fcg_topology_digest
  std::vector<std::pair<const void *, size_t>> topo;

  // lazily built lsq matrices dmat(9,n)
  fcg::DBuf dmat;
  bool dmat_ready = false;
  // lazily built mesh-constant factors of the inner faces (assembly.cu: laplacian,
  // facefluxmass, fluxmc), planar [FG_COUNT][nin]
  fcg::DBuf fgeo;
  bool fgeo_ready = false;
  // and of the boundary faces (calcuvw's boundary loops), planar [BG_COUNT][ncb]
  fcg::DBuf bgeo;
  bool bgeo_ready = false;
  // diagnostics of the GPU hierarchy build (fcg_set_aggregation_wait_test)
  int agg_test_polls = 0, agg_test_row = -1;

  // per-call staging of host arrays and kernel scratch
  std::vector<fcg::DBuf> stage;
  fcg::DBuf scratch;
  fcg::KrylovState *ks = nullptr;  // solver workspaces and captured graphs (krylov.cu)
  fcg::MultiState *ms = nullptr;   // multi-RHS BiCGStab workspaces (multi.cu)

  ~fcg_context();
};

namespace fcg {

int set_error(fcg_context *c, int status, const std::string &msg);

// Values of a matrix `a` on the bound mesh: the CSR values, then ar and al of the O-C
// pairs (2 noc more when the mesh has them).
inline long long a_len(const fcg_context *c) { return c->nnz + 2LL * c->mv.noc; }

// foc and srdoc of the bound mesh's O-C pairs (assembly.cu), computed at bind.
int oc_geometry(fcg_context *c);

// FCG_ERR_UNSUPPORTED for the entry points that do not take the O-C pairs into account.
inline int refuse_oc(fcg_context *c, const char *what) {
  return c->mv.noc ? set_error(c, FCG_ERR_UNSUPPORTED,
                               std::string(what) + ": O-C grid cuts and cyclic faces (noc > 0)"
                                                   " are supported by the reference's routines"
                                                   " only (assembly, gradients, bpres, dpcg,"
                                                   " iccg, bicgstab, spmv), not by the mixed,"
                                                   " multi-RHS, batched or learned solvers")
                   : FCG_OK;
}
int cuda_fail(fcg_context *c, cudaError_t e, const char *where);

// Host-side construction of the topology (topology.cpp).  Returns a status code.
struct HostTopology {
  std::vector<int> ioffset, ja, diag, slot_pn, slot_np;  // 1-based (reference form)
  std::vector<int> cf_ptr, cf_ent, cf_slot;              // 0-based
  std::vector<int> cb_ptr, cb_face, cb_slot, cb_type;
  std::vector<int> cbf_ptr, cbf_face;
  std::vector<long long> sell_ptr;
  std::vector<int> sell_width, sell_kind, sell_offp, sell_off, sell_src;
  int sell_maxw = 0;
  long long sell_nuniform = 0;
  std::vector<int> lf_ptr, lf_rows, lb_ptr, lb_rows;
  std::vector<int> tpos;
};

// csr_given: t already holds the 1-based CSR and slot maps (built on the GPU by
// fcg_csr_build_gpu, which also refuses duplicate cell pairs).
int build_topology(const fcg_mesh_desc &m, const int cnt[B_NTYPES], const int fst[B_NTYPES],
                   const int bst[B_NTYPES], HostTopology &t, std::string &err,
                   bool csr_given = false);
int validate_topology(const fcg_mesh_desc &m, const int cnt[B_NTYPES], const int fst[B_NTYPES],
                      std::string &err);
int build_csr(const fcg_mesh_desc &m, HostTopology &t, std::string &err);
int build_rest(const fcg_mesh_desc &m, const int cnt[B_NTYPES], const int fst[B_NTYPES],
               const int bst[B_NTYPES], HostTopology &t);
// Exclusive scan of n ints on the context's stream: out[0..n], out[n] the total (setup.cu);
// tmp holds the block sums.
int scan_ints(fcg_context *c, const int *in, int *out, int n, DBuf &tmp);
// a[i] -= 1 on the device (1-based index arrays to 0-based), on c's stream.
int to_zero_based(fcg_context *c, int *a, long long n);
// Fills c->hex from the bound CSR pattern (hexblock.cu); synchronises c's stream.
int detect_hex_block(fcg_context *c);
// The whole topology built on c's device (setup.cu), 0-based and owned by the bound
// mesh, element for element the host construction: fills c->mv's CSR, slot maps and
// incidence lists, c->tpos, c->sv, c->lf / c->lb, c->nnz and c->topo.  own0 / nei0 are
// the device copies (0-based) of owner / neighbour, own_host the 1-based host owner.
int bind_topology_device(fcg_context *c, const int *own0, const int *nei0,
                         const std::vector<int> &own_host, const int cnt[B_NTYPES],
                         const int fst[B_NTYPES], const int bst[B_NTYPES], std::string &err);

// Pointer staging: returns a device pointer for a user array of `bytes` bytes.  A
// device pointer is returned as is; a host array is copied into staging slot `slot`
// when `copy_in` is set.  `was_host` tells the caller to copy results back.
int stage_in(fcg_context *c, const void *user, size_t bytes, int slot, bool copy_in, void **dev,
             bool *was_host);
int stage_out(fcg_context *c, void *user, const void *dev, size_t bytes, bool was_host);
bool is_device_pointer(const void *p);

// Solver matrices shared with the learned preconditioner (krylov.cu): loads CSR values
// a (device) and builds D^-1/2 (FP64) and D^-1/2 A D^-1/2 (FP32) in the sliced layout.
int prepare_scaled32(fcg_context *c, const double *a_dev);
const float *scaled32(const fcg_context *c);
const double *scale64(const fcg_context *c);
const double *sliced64(const fcg_context *c);

// Device vectors of one system of a batched solve (krylov.cu): loads CSR values a
// (device; NULL reuses the loaded matrix), su and the initial guess into the context's
// solver state and returns its FP64 sliced matrix, 1/a(diag) and vectors.
struct BatchVecs {
  const double *val, *invd, *su;
  double *x, *res, *p, *q;
};
int batch_load(fcg_context *c, const double *a_dev, const double *su_dev, const double *fi_dev,
               BatchVecs *out);

namespace corr {
// Outlet velocities, fmo and the flomas scaling (assembly.cu), device arrays; fac is
// left in c->scratch[0].
int outlet_flow(fcg_context *c, const double *den, double flomas, double *u, double *v,
                double *w, double *fmo);
}  // namespace corr

}  // namespace fcg

#define FCG_CUDA_TRY(ctx, expr)                                   \
  do {                                                            \
    cudaError_t _e = (expr);                                      \
    if (_e != cudaSuccess) return fcg::cuda_fail((ctx), _e, #expr); \
  } while (0)

#define FCG_CHECK_LAUNCH(ctx, name)                                   \
  do {                                                                \
    cudaError_t _e = cudaGetLastError();                              \
    if (_e != cudaSuccess) return fcg::cuda_fail((ctx), _e, name);    \
  } while (0)
