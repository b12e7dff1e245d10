// Aggregation hierarchy of the learned FCG's coarse-grid correction, built on the host
// once per mesh from the first scaled matrix it is asked to solve.
//
// A level is formed by three passes of pairwise matching: each row, in ascending order,
// pairs with its unmatched neighbour of most negative coupling (ties go to the lowest
// column); a row left without one then joins the matched pair it is most negatively
// coupled to, if any.  A coarse row so aggregates about eight rows of the level above.  Between passes the matrix is the Galerkin product P^T A P of the
// piecewise-constant prolongation P, summed in a fixed order: member rows ascending,
// and inside each member row the entries in column order, each added to the slot of its
// coarse column in the order met.  Rows of the result are then sorted by column.  These
// host values only steer the matching; the device recomputes every level's values from
// the current matrix on each solve (coarse.cu).
#include <algorithm>
#include <string>
#include <vector>

#include "coarse.h"
#include "host_util.h"

namespace fcg {
namespace ml {

namespace {
// Builds a CSR row by row on all host threads: row(i, cols, vals) appends row i to the
// thread's vectors (its own contiguous block of rows); the blocks are joined in order,
// so the result does not depend on the thread count.
template <class RowFn>
void chunked_csr(int n, std::vector<int> &ptr, std::vector<int> &col, std::vector<double> *val,
                 RowFn &&row) {
  const unsigned nt = n < (1 << 14) ? 1u : std::max(1u, std::thread::hardware_concurrency());
  const long long chunk = ((long long)n + nt - 1) / nt;
  std::vector<std::vector<int>> cols(nt), lens(nt);
  std::vector<std::vector<double>> vals(nt);
  parallel_for(
      nt,
      [&](long long t) {
        const long long b = t * chunk, e = std::min<long long>(n, b + chunk);
        for (long long i = b; i < e; ++i) {
          const size_t before = cols[t].size();
          row((int)i, cols[t], vals[t]);
          lens[t].push_back((int)(cols[t].size() - before));
        }
      },
      1);
  ptr.assign(n + 1, 0);
  std::vector<long long> off(nt + 1, 0);
  for (unsigned t = 0; t < nt; ++t) off[t + 1] = off[t] + (long long)cols[t].size();
  col.resize(off[nt]);
  if (val) val->resize(off[nt]);
  long long r = 0;
  for (unsigned t = 0; t < nt; ++t)
    for (int L : lens[t]) {
      ptr[r + 1] = ptr[r] + L;
      ++r;
    }
  parallel_for(
      nt,
      [&](long long t) {
        std::copy(cols[t].begin(), cols[t].end(), col.begin() + off[t]);
        if (val) std::copy(vals[t].begin(), vals[t].end(), val->begin() + off[t]);
      },
      1);
}

// Sums (column, value) pairs met in order into one entry per column, each column's values
// added in the order met, and appends the row sorted by column.  One per thread: the
// marker array (position of each column in the row, -1 when absent) is reset after every
// row, so a row costs its pair count plus a sort of its distinct columns.
struct RowSum {
  std::vector<int> mk;
  std::vector<std::pair<int, double>> row;
  void begin(int ncols) {
    if ((int)mk.size() < ncols) mk.assign(ncols, -1);
    row.clear();
  }
  void add(int J, double v) {
    const int p = mk[J];
    if (p < 0) {
      mk[J] = (int)row.size();
      row.emplace_back(J, v);
    } else {
      row[p].second += v;
    }
  }
  void end(std::vector<int> &cols, std::vector<double> &vals) {
    for (const auto &e : row) mk[e.first] = -1;
    std::sort(row.begin(), row.end(),
              [](const std::pair<int, double> &a, const std::pair<int, double> &b) {
                return a.first < b.first;
              });
    for (const auto &e : row) {
      cols.push_back(e.first);
      vals.push_back(e.second);
    }
  }
};
}  // namespace

int pair_match(int n, const int *ptr, const int *col, const double *val, std::vector<int> &agg) {
  agg.assign(n, -1);
  std::vector<char> paired;
  paired.reserve(n);
  int nc = 0;
  for (int i = 0; i < n; ++i) {
    if (agg[i] >= 0) continue;
    int best = -1;
    double bv = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      if (j == i || agg[j] >= 0) continue;
      if (val[k] < bv) {
        bv = val[k];
        best = j;
      }
    }
    agg[i] = nc;
    if (best >= 0) agg[best] = nc;
    paired.push_back(best >= 0);
    ++nc;
  }
  // a row left single joins the pair it is most strongly coupled to (pairs as matched,
  // so joins do not chain); the aggregates are then renumbered in their order
  bool moved = false;
  for (int i = 0; i < n; ++i) {
    if (paired[agg[i]]) continue;
    int best = -1;
    double bv = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      if (j == i || !paired[agg[j]]) continue;
      if (val[k] < bv) {
        bv = val[k];
        best = j;
      }
    }
    if (best >= 0) {
      agg[i] = agg[best];
      moved = true;
    }
  }
  if (!moved) return nc;
  std::vector<int> used(nc, 0);
  for (int i = 0; i < n; ++i) used[agg[i]] = 1;
  std::vector<int> id(nc, -1);
  int m = 0;
  for (int I = 0; I < nc; ++I)
    if (used[I]) id[I] = m++;
  for (int i = 0; i < n; ++i) agg[i] = id[agg[i]];
  return m;
}

void members(int n, int nc, const std::vector<int> &agg, std::vector<int> &mptr,
             std::vector<int> &mem) {
  mptr.assign(nc + 1, 0);
  for (int i = 0; i < n; ++i) ++mptr[agg[i] + 1];
  for (int I = 0; I < nc; ++I) mptr[I + 1] += mptr[I];
  mem.assign(n, 0);
  std::vector<int> fill(mptr.begin(), mptr.end() - 1);
  for (int i = 0; i < n; ++i) mem[fill[agg[i]]++] = i;
}

void galerkin(const HostCsr &A, const std::vector<int> &agg, int nc, const std::vector<int> &mptr,
              const std::vector<int> &mem, HostCsr &out) {
  out.n = nc;
  chunked_csr(nc, out.ptr, out.col, &out.val,
              [&](int I, std::vector<int> &cols, std::vector<double> &vals) {
                thread_local RowSum rs;
                rs.begin(nc);
                for (int m = mptr[I]; m < mptr[I + 1]; ++m) {
                  const int i = mem[m];
                  for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) rs.add(agg[A.col[k]], A.val[k]);
                }
                rs.end(cols, vals);
              });
}

// P = (I - omega D^-1 A) P_tent of the level's aggregation, A P and P^T A P, patterns
// sorted by column and FP64 values in the device's order (P: 1 at the own aggregate,
// then minus (omega / a_ii) a_ik for the row's entries in column order; A P: for the
// row's entries in column order, a_ik P_k in P_k's order; P^T A P: for the rows holding
// the aggregate in ascending order, P_iI (A P)_i in column order).
void smoothed_level(const HostCsr &A, double omega, HostLevel &lv) {
  const int n = A.n, nc = lv.n;
  const std::vector<int> &agg = lv.agg;
  // P: pattern and values
  std::vector<double> pv;
  chunked_csr(n, lv.p_ptr, lv.p_col, &pv, [&](int i, std::vector<int> &cols, std::vector<double> &vals) {
    thread_local std::vector<int> row;
    row.clear();
    row.push_back(agg[i]);
    for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) row.push_back(agg[A.col[k]]);
    std::sort(row.begin(), row.end());
    row.erase(std::unique(row.begin(), row.end()), row.end());
    const size_t b = cols.size();
    double d = 0.0;
    for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
      if (A.col[k] == i) d = A.val[k];
    const double w = d > 0.0 ? omega / d : 0.0;
    for (int J : row) {
      cols.push_back(J);
      vals.push_back(J == agg[i] ? 1.0 : 0.0);
    }
    for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
      const size_t p = b + (std::lower_bound(row.begin(), row.end(), agg[A.col[k]]) - row.begin());
      vals[p] -= w * A.val[k];
    }
  });
  // transpose lists: rows ascending within every aggregate
  lv.t_ptr.assign(nc + 1, 0);
  for (int J : lv.p_col) ++lv.t_ptr[J + 1];
  for (int I = 0; I < nc; ++I) lv.t_ptr[I + 1] += lv.t_ptr[I];
  lv.t_row.assign(lv.p_col.size(), 0);
  lv.t_pos.assign(lv.p_col.size(), 0);
  {
    std::vector<int> fill(lv.t_ptr.begin(), lv.t_ptr.end() - 1);
    for (int i = 0; i < n; ++i)
      for (int p = lv.p_ptr[i]; p < lv.p_ptr[i + 1]; ++p) {
        const int f = fill[lv.p_col[p]]++;
        lv.t_row[f] = i;
        lv.t_pos[f] = p;
      }
  }
  // A P: for the row's entries in column order, a_ik P_k in P_k's order
  std::vector<double> apv;
  chunked_csr(n, lv.ap_ptr, lv.ap_col, &apv, [&](int i, std::vector<int> &cols, std::vector<double> &vals) {
    thread_local RowSum rs;
    rs.begin(nc);
    for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
      const int j = A.col[k];
      for (int p = lv.p_ptr[j]; p < lv.p_ptr[j + 1]; ++p) rs.add(lv.p_col[p], A.val[k] * pv[p]);
    }
    rs.end(cols, vals);
  });
  // P^T A P: for the rows holding the aggregate in ascending order, P_iI (A P)_i
  HostCsr &C = lv.A;
  C.n = nc;
  chunked_csr(nc, C.ptr, C.col, &C.val, [&](int I, std::vector<int> &cols, std::vector<double> &vals) {
    thread_local RowSum rs;
    rs.begin(nc);
    for (int m = lv.t_ptr[I]; m < lv.t_ptr[I + 1]; ++m) {
      const int i = lv.t_row[m];
      const double p = pv[lv.t_pos[m]];
      for (int q = lv.ap_ptr[i]; q < lv.ap_ptr[i + 1]; ++q) rs.add(lv.ap_col[q], p * apv[q]);
    }
    rs.end(cols, vals);
  });
}

int build_levels(const HostCsr &fine, int max_levels, int dense_max, int passes,
                 std::vector<HostLevel> &levels, double sa_omega) {
  levels.clear();
  levels.reserve(max_levels);
  const HostCsr *cur = &fine;
  HostCsr work[2];
  int wi = 0;
  while ((int)levels.size() + 1 < max_levels) {
    const int n0 = cur->n;
    if (n0 < 2) break;
    HostLevel lv;
    std::vector<int> comp(n0);
    for (int i = 0; i < n0; ++i) comp[i] = i;
    const HostCsr *a = cur;
    int nc = n0;
    for (int p = 0; p < passes; ++p) {
      std::vector<int> agg, mptr, mem;
      const int m = pair_match(a->n, a->ptr.data(), a->col.data(), a->val.data(), agg);
      if (m == a->n) break;  // no pair formed: this matrix does not coarsen
      members(a->n, m, agg, mptr, mem);
      HostCsr &dst = work[wi];
      wi ^= 1;
      galerkin(*a, agg, m, mptr, mem, dst);
      for (int i = 0; i < n0; ++i) comp[i] = agg[comp[i]];
      a = &dst;
      nc = m;
      if (nc <= dense_max) break;
    }
    if (nc == n0 || 10LL * nc > 9LL * n0) break;  // less than 10% fewer rows: stop
    lv.n = nc;
    lv.agg = std::move(comp);
    members(n0, nc, lv.agg, lv.mptr, lv.mem);
    if (levels.empty() && sa_omega > 0.0)
      smoothed_level(*cur, sa_omega, lv);  // P^T A P with the smoothed prolongation
    else
      lv.A = *a;  // pattern (and host values) of the level
    levels.push_back(std::move(lv));
    cur = &levels.back().A;
    if (nc <= dense_max) break;
  }
  return (int)levels.size();
}

}  // namespace ml
}  // namespace fcg

// Host utility: the aggregation of one level (`passes` matching passes on a 0-based CSR
// with ascending columns, stopping once at most dense_max aggregates remain).
extern "C" int fcg_aggregate(int n, const int *ptr, const int *col, const double *val,
                             int passes, int dense_max, int *agg, int *nc) {
  if (n < 0 || !ptr || !agg || !nc || passes < 1 || (n > 0 && (!col || !val)))
    return FCG_ERR_ARG;
  if (ptr[0] != 0) return FCG_ERR_INDEX;
  for (int i = 0; i < n; ++i) {
    if (ptr[i + 1] < ptr[i]) return FCG_ERR_INDEX;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
      if (col[k] < 0 || col[k] >= n || (k > ptr[i] && col[k] <= col[k - 1])) return FCG_ERR_INDEX;
  }
  fcg::ml::HostCsr a;
  a.n = n;
  a.ptr.assign(ptr, ptr + n + 1);
  a.col.assign(col, col + ptr[n]);
  a.val.assign(val, val + ptr[n]);
  std::vector<fcg::ml::HostLevel> lv;
  fcg::ml::build_levels(a, 2, dense_max, passes, lv);
  if (lv.empty()) {
    for (int i = 0; i < n; ++i) agg[i] = i;
    *nc = n;
  } else {
    for (int i = 0; i < n; ++i) agg[i] = lv[0].agg[i];
    *nc = lv[0].n;
  }
  return FCG_OK;
}

// Host utility: P^T A P of the smoothed prolongation P = (I - omega D^-1 A) P_tent of the
// aggregation agg[n] (nc aggregates) of a 0-based CSR with ascending columns, in FP64 in
// the order the hierarchy uses.  With cptr NULL only *nnz is returned; otherwise cptr[nc+1],
// ccol[*nnz] and cval[*nnz] are filled (*nnz must hold their capacity).
extern "C" int fcg_smoothed_level(int n, const int *ptr, const int *col, const double *val,
                                  const int *agg, int nc, double omega, long long *nnz,
                                  int *cptr, int *ccol, double *cval) {
  if (n < 1 || nc < 1 || !ptr || !col || !val || !agg || !nnz || !(omega > 0.0))
    return FCG_ERR_ARG;
  if (ptr[0] != 0) return FCG_ERR_INDEX;
  for (int i = 0; i < n; ++i) {
    if (ptr[i + 1] < ptr[i] || agg[i] < 0 || agg[i] >= nc) return FCG_ERR_INDEX;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
      if (col[k] < 0 || col[k] >= n || (k > ptr[i] && col[k] <= col[k - 1])) return FCG_ERR_INDEX;
  }
  fcg::ml::HostCsr a;
  a.n = n;
  a.ptr.assign(ptr, ptr + n + 1);
  a.col.assign(col, col + ptr[n]);
  a.val.assign(val, val + ptr[n]);
  fcg::ml::HostLevel lv;
  lv.n = nc;
  lv.agg.assign(agg, agg + n);
  fcg::ml::smoothed_level(a, omega, lv);
  const long long m = (long long)lv.A.col.size();
  if (!cptr) {
    *nnz = m;
    return FCG_OK;
  }
  if (!ccol || !cval || *nnz < m) return FCG_ERR_ARG;
  std::copy(lv.A.ptr.begin(), lv.A.ptr.end(), cptr);
  std::copy(lv.A.col.begin(), lv.A.col.end(), ccol);
  std::copy(lv.A.val.begin(), lv.A.val.end(), cval);
  *nnz = m;
  return FCG_OK;
}

