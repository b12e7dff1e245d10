// Coarse-grid correction of the learned FCG: aggregation hierarchy (aggregation.cpp,
// host) and its device state and kernels (coarse.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fcg_internal.h"

namespace fcg {
namespace ml {

// A CSR matrix on the host, 0-based, columns ascending in every row.
struct HostCsr {
  int n = 0;
  std::vector<int> ptr, col;
  std::vector<double> val;
};

// One level below the fine matrix: agg maps the rows of the level above to this
// level's rows; mptr/mem list each row's parent rows in ascending order; A holds the
// Galerkin pattern and the host values the matching used.
struct HostLevel {
  int n = 0;
  std::vector<int> agg, mptr, mem;
  HostCsr A;
  // first level with a smoothed prolongation P = (I - omega D^-1 A) P_tent: the pattern
  // of P (p_ptr, p_col: the row's own aggregate and its neighbours' aggregates,
  // ascending), its transpose (t_ptr, t_row, t_pos: for every aggregate the rows whose P
  // row holds it, ascending, and the position in p_col), and the pattern of A P
  // (ap_ptr, ap_col); A is then P^T A P
  std::vector<int> p_ptr, p_col, t_ptr, t_row, t_pos, ap_ptr, ap_col;
};

// One pass of pairwise matching on (ptr, col, val); returns the number of aggregates.
int pair_match(int n, const int *ptr, const int *col, const double *val, std::vector<int> &agg);
// Parent rows of every aggregate, ascending (a counting sort of agg).
void members(int n, int nc, const std::vector<int> &agg, std::vector<int> &mptr,
             std::vector<int> &mem);
// P^T A P for the piecewise-constant P of agg, summed in the documented order.
void galerkin(const HostCsr &A, const std::vector<int> &agg, int nc, const std::vector<int> &mptr,
              const std::vector<int> &mem, HostCsr &out);
// Levels below `fine`: `passes` matching passes per level, until a level has at most
// dense_max rows, stops coarsening, or max_levels levels (the fine one included) exist.
int build_levels(const HostCsr &fine, int max_levels, int dense_max, int passes,
                 std::vector<HostLevel> &levels, double sa_omega = 0.0);
// The smoothed first level (sa_omega > 0 in build_levels): patterns and FP64 values.
void smoothed_level(const HostCsr &A, double omega, HostLevel &lv);

// A CSR matrix on the device, 0-based, columns ascending in every row.
struct DevCsr {
  int n = 0;
  long long nnz = 0;
  const int *ptr = nullptr, *col = nullptr;
  const double *val = nullptr;
};

// A device CSR that owns its arrays.
struct DevMat {
  int n = 0;
  long long nnz = 0;
  DBuf ptr, col, val;
  DevCsr view() const { return {n, nnz, ptr.as<int>(), col.as<int>(), val.as<double>()}; }
  void release() {
    ptr.release();
    col.release();
    val.release();
  }
};

// A HostLevel built on the device (aggregation_gpu.cu): the same arrays, on c's device;
// np is the row count of the level above.  Owns its buffers until release().
struct DevBuiltLevel {
  int n = 0, np = 0;
  DBuf agg, mptr, mem;
  DevMat A;
  long long p_nnz = 0, ap_nnz = 0;
  DBuf p_ptr, p_col, t_ptr, t_row, t_pos, ap_ptr, ap_col;
  void release();
};

// The scaled fine matrix's CSR values on the device: the sliced FP64 values scattered to
// CSR order through src (len slots, -1 for padding), then (a_ik s_i) s_k, as build() forms
// them on the host.
void fine_values(fcg_context *c, const double *sval, const int *src, long long len,
                 const double *s, double *val);

// build_levels on the device, element for element the host's result.  Returns FCG_OK,
// FCG_ERR_TIMEOUT when a dependency wait of the matching gave up, FCG_ERR_UNSUPPORTED when
// a coarse row outgrows the accumulation tables, or FCG_ERR_CUDA; err says which.
int build_levels_device(fcg_context *c, const DevCsr &fine, int max_levels, int dense_max,
                        int passes, double sa_omega, std::vector<DevBuiltLevel> &levels,
                        std::string &err);

// Options of the correction (fcg_lp_set_multilevel).
struct Options {
  int enabled = 1;
  int smoother = 0;  // 0: the network at the fine level, 1: Jacobi sweeps
  int sweeps = 2;    // Jacobi sweeps before and after each coarse level's correction
  int max_levels = 10;
  int dense_max = 128;
  double alpha = 1.8;  // scaling of every unsmoothed prolongated correction
  double omega = 0.67; // Jacobi damping, and the prolongation smoothing of the first level
  int smoothed = 1;    // first level: smoothed prolongation (correction not scaled)
};

// Device arrays of one coarse level.
struct DevLevel {
  int n = 0;
  long long nnz = 0;
  DBuf ints, vals, vecs;
  int *ptr = nullptr, *col = nullptr, *agg = nullptr, *mptr = nullptr, *mem = nullptr;
  float *a32 = nullptr, *dinv = nullptr;  // Galerkin values (FP32), 1 / diagonal
  float *b = nullptr, *x = nullptr, *y = nullptr;  // right-hand side, iterate, ping-pong
};

struct Hierarchy {
  unsigned long long uid = 0;  // context and bind the hierarchy belongs to
  unsigned gen = 0;
  int n0 = 0;
  int passes = 3, max_levels = 10, dense_max = 128, smoothed = 1;
  double sa_omega = 0.0;
  // smoothed first level: P (p_ptr, p_col, p_val), its transpose lists, A P
  DBuf sa_ints, sa_vals;
  int *p_ptr = nullptr, *p_col = nullptr, *t_ptr = nullptr, *t_row = nullptr, *t_pos = nullptr;
  int *ap_ptr = nullptr, *ap_col = nullptr;
  float *p_val = nullptr, *pt_val = nullptr, *ap_val = nullptr;  // pt_val: P in t-list order
  long long p_nnz = 0, ap_nnz = 0;
  std::vector<DevLevel> lv;     // levels 1..L (lv[0] is level 1)
  DBuf dense;                   // inverse of the coarsest matrix (row-major)
  bool has_dense = false;
  DBuf fine_tmp;                // two FP32 vectors of the fine level
  double setup_seconds = 0.0;
  bool built_on_device = false;  // the levels came from aggregation_gpu.cu
  unsigned long long build_id = 0;  // bumped at every build (keys captured graphs)
  bool built_for(const fcg_context *c, const struct Options &o) const {
    return uid == c->uid && gen == c->bind_gen && max_levels == o.max_levels &&
           dense_max == o.dense_max && smoothed == o.smoothed &&
           (!smoothed || sa_omega == o.omega);
  }
  void release();
};

// Builds H for context c from the matrix loaded into its solver state (prepare_scaled32:
// the sliced FP64 values and D^-1/2), scaled to Ahat.
int build(Hierarchy &H, fcg_context *c, const Options &o, std::string &err);
// Galerkin values of every level from the loaded matrix, and the coarsest inverse.
int values(Hierarchy &H, fcg_context *c, cudaStream_t st);
// z += P V(P^T (r - Ahat z)) (alpha P_tent for an unsmoothed first level): the
// correction after the network (fine level).
void enqueue_correction(Hierarchy &H, fcg_context *c, const Options &o, cudaStream_t st,
                        const float *r, float *z, const int *done);
// z = V(r) with Jacobi sweeps at the fine level too (the cycle without the network).
void enqueue_jacobi_cycle(Hierarchy &H, fcg_context *c, const Options &o, cudaStream_t st,
                          const float *r, float *z, const int *done);

}  // namespace ml
}  // namespace fcg
