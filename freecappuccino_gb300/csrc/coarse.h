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
                 std::vector<HostLevel> &levels);

// Options of the correction (fcg_lp_set_multilevel).
struct Options {
  int enabled = 1;
  int smoother = 0;  // 0: the network at the fine level, 1: Jacobi sweeps
  int sweeps = 2;    // Jacobi sweeps before and after each coarse level's correction
  int max_levels = 10;
  int dense_max = 128;
  double alpha = 1.8;  // scaling of every prolongated correction
  double omega = 0.67; // Jacobi damping
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
  int passes = 3, max_levels = 10, dense_max = 128;
  std::vector<DevLevel> lv;     // levels 1..L (lv[0] is level 1)
  DBuf dense;                   // inverse of the coarsest matrix (row-major)
  bool has_dense = false;
  DBuf fine_tmp;                // two FP32 vectors of the fine level
  double setup_seconds = 0.0;
  unsigned long long build_id = 0;  // bumped at every build (keys captured graphs)
  bool built_for(const fcg_context *c, const struct Options &o) const {
    return uid == c->uid && gen == c->bind_gen && max_levels == o.max_levels &&
           dense_max == o.dense_max;
  }
  void release();
};

// Builds H for context c from the matrix loaded into its solver state (prepare_scaled32:
// the sliced FP64 values and D^-1/2), scaled to Ahat.
int build(Hierarchy &H, fcg_context *c, const Options &o, std::string &err);
// Galerkin values of every level from the loaded matrix, and the coarsest inverse.
int values(Hierarchy &H, fcg_context *c, cudaStream_t st);
// z += alpha P V(P^T (r - Ahat z)): the correction after the network (fine level).
void enqueue_correction(Hierarchy &H, fcg_context *c, const Options &o, cudaStream_t st,
                        const float *r, float *z, const int *done);
// z = V(r) with Jacobi sweeps at the fine level too (the cycle without the network).
void enqueue_jacobi_cycle(Hierarchy &H, fcg_context *c, const Options &o, cudaStream_t st,
                          const float *r, float *z, const int *done);

}  // namespace ml
}  // namespace fcg
