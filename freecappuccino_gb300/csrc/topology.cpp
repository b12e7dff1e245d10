// Bind-time topology of libfcgpu.so, built on the host once per mesh.
//
// * The CSR pattern of create_CSR_matrix_from_mesh_data (src/sparse_matrix.f90:42-172):
//   the reference fills a COO list and heap-sorts it lexically; since the (row, col)
//   pairs are unique the result is the canonical row-sorted, column-ascending CSR, so
//   it is built here directly by counting rows and sorting each (<= 7 entry) row.
//   diag and the two face->slot maps (:153-167) follow.  Bit-exact with the reference.
// * Cell->face incidence lists in the reference's face-loop order, used by the
//   cell-gather kernels so that every per-cell sum adds its terms in the order of the
//   Fortran loops (inner faces ascending, then boundary faces by type).
// * A sliced-ELL (32-row slices) copy of the pattern for the solvers.
// * Level schedules of the lower and upper triangles (row i waits for the rows its
//   lower/upper entries name) for the DIC/DILU sweeps of iccg.f90 / bicgstab.f90.
#include <algorithm>
#include <cstdlib>
#include <string>

#include "fcg_internal.h"
#include "host_util.h"

namespace fcg {

int validate_topology(const fcg_mesh_desc &m, const int cnt[B_NTYPES], const int fst[B_NTYPES],
                      std::string &err) {
  const int n = m.numCells, nf = m.numFaces, nin = m.numInnerFaces;
  for (int f = 0; f < nf; ++f) {
    int o = m.owner[f];
    if (o < 1 || o > n) {
      err = "owner(" + std::to_string(f + 1) + ") = " + std::to_string(o) + " is out of 1.." +
            std::to_string(n);
      return FCG_ERR_INDEX;
    }
  }
  for (int f = 0; f < nin; ++f) {
    int nb = m.neighbour[f];
    if (nb < 1 || nb > n || nb == m.owner[f]) {
      err = "neighbour(" + std::to_string(f + 1) + ") = " + std::to_string(nb) + " is invalid";
      return FCG_ERR_INDEX;
    }
  }
  for (int ty = 0; ty < B_NTYPES; ++ty) {
    if (cnt[ty] < 0 || (cnt[ty] > 0 && (fst[ty] < nin || (long long)fst[ty] + cnt[ty] > nf))) {
      err = "boundary type " + std::to_string(ty) + " face range is outside the boundary faces";
      return FCG_ERR_INDEX;
    }
  }
  return FCG_OK;
}

int build_topology(const fcg_mesh_desc &m, const int cnt[B_NTYPES], const int fst[B_NTYPES],
                   const int bst[B_NTYPES], HostTopology &t, std::string &err, bool csr_given) {
  const int n = m.numCells, nf = m.numFaces, nin = m.numInnerFaces;
  int vrc = validate_topology(m, cnt, fst, err);
  if (vrc) return vrc;
  if (!csr_given) {
    int crc = build_csr(m, t, err);
    if (crc) return crc;
  }
  return build_rest(m, cnt, fst, bst, t);
}

// CSR of create_CSR_matrix_from_mesh_data (sparse_matrix.f90:42-172), 1-based, with the
// face slot maps.
int build_csr(const fcg_mesh_desc &m, HostTopology &t, std::string &err) {
  const int n = m.numCells, nin = m.numInnerFaces;
  t.ioffset.assign(n + 1, 0);
  std::vector<int> rowcnt(n, 1);
  for (int f = 0; f < nin; ++f) {
    rowcnt[m.owner[f] - 1]++;
    rowcnt[m.neighbour[f] - 1]++;
  }
  t.ioffset[0] = 1;
  for (int i = 0; i < n; ++i) {
    long long next = (long long)t.ioffset[i] + rowcnt[i];
    if (next > 0x7fffffffLL) {
      err = "nnz does not fit a 32-bit CSR index";
      return FCG_ERR_ARG;
    }
    t.ioffset[i + 1] = (int)next;
  }
  const long long nnz = (long long)t.ioffset[n] - 1;
  t.ja.assign(nnz, 0);
  {
    std::vector<int> fill(n);
    for (int i = 0; i < n; ++i) {
      fill[i] = t.ioffset[i] - 1;
      t.ja[fill[i]++] = i + 1;
    }
    for (int f = 0; f < nin; ++f) {
      int o = m.owner[f] - 1, nb = m.neighbour[f] - 1;
      t.ja[fill[o]++] = nb + 1;
      t.ja[fill[nb]++] = o + 1;
    }
  }
  bool dup = false;
  parallel_for(n, [&](long long i) {
    int b = t.ioffset[i] - 1, e = t.ioffset[i + 1] - 1;
    std::sort(t.ja.begin() + b, t.ja.begin() + e);
    for (int k = b + 1; k < e; ++k)
      if (t.ja[k] == t.ja[k - 1]) dup = true;
  });
  if (dup) {
    err = "two faces connect the same pair of cells";
    return FCG_ERR_INDEX;
  }
  t.diag.assign(n, 0);
  parallel_for(n, [&](long long i) {
    for (int k = t.ioffset[i] - 1; k < t.ioffset[i + 1] - 1; ++k)
      if (t.ja[k] == i + 1) t.diag[i] = k + 1;
  });
  auto find = [&](int row1, int col1) {  // 1-based position of (row, col), 0 if absent
    int b = t.ioffset[row1 - 1] - 1, e = t.ioffset[row1] - 1;
    auto it = std::lower_bound(t.ja.begin() + b, t.ja.begin() + e, col1);
    return (it != t.ja.begin() + e && *it == col1) ? (int)(it - t.ja.begin()) + 1 : 0;
  };
  t.slot_pn.assign(nin, 0);
  t.slot_np.assign(nin, 0);
  parallel_for(nin, [&](long long f) {
    t.slot_pn[f] = find(m.owner[f], m.neighbour[f]);
    t.slot_np[f] = find(m.neighbour[f], m.owner[f]);
  });
  return FCG_OK;
}

// Everything built from the CSR and the face lists: transpose positions, incidence lists,
// the sliced ELL copy and the level schedules.
int build_rest(const fcg_mesh_desc &m, const int cnt[B_NTYPES], const int fst[B_NTYPES],
               const int bst[B_NTYPES], HostTopology &t) {
  const int n = m.numCells, nf = m.numFaces, nin = m.numInnerFaces;
  const long long nnz = (long long)t.ioffset[n] - 1;
  auto find = [&](int row1, int col1) {  // 1-based position of (row, col), 0 if absent
    int b = t.ioffset[row1 - 1] - 1, e = t.ioffset[row1] - 1;
    auto it = std::lower_bound(t.ja.begin() + b, t.ja.begin() + e, col1);
    return (it != t.ja.begin() + e && *it == col1) ? (int)(it - t.ja.begin()) + 1 : 0;
  };
  t.tpos.assign(nnz, 0);
  parallel_for(n, [&](long long i) {
    for (int k = t.ioffset[i] - 1; k < t.ioffset[i + 1] - 1; ++k)
      t.tpos[k] = find(t.ja[k], (int)i + 1) - 1;
  });

  // --- incidence lists ---------------------------------------------------------
  // The inner faces of cell i are its off-diagonal CSR entries (one per face), so the
  // list is built per row from the CSR: each entry's face (the inverse of the slot
  // maps), sorted by face index -- the order of a face loop over the cell.
  t.cf_ptr.assign(n + 1, 0);
  for (int i = 0; i <= n; ++i) t.cf_ptr[i] = (t.ioffset[i] - 1) - i;
  t.cf_ent.assign(t.cf_ptr[n], 0);
  t.cf_slot.assign(t.cf_ptr[n], 0);
  {
    std::vector<int> face_at(nnz, -1);
    parallel_for(nin, [&](long long f) {
      face_at[t.slot_pn[f] - 1] = (int)f;
      face_at[t.slot_np[f] - 1] = (int)f;
    });
    parallel_for(n, [&](long long i) {
      int e = t.cf_ptr[i];
      for (int k = t.ioffset[i] - 1; k < t.ioffset[i + 1] - 1; ++k) {
        if (k == t.diag[i] - 1) continue;
        const int f = face_at[k];
        int j = e++;
        // insertion into the row's list, ascending face index
        while (j > t.cf_ptr[i] && std::abs(t.cf_ent[j - 1]) > f + 1) {
          t.cf_ent[j] = t.cf_ent[j - 1];
          t.cf_slot[j] = t.cf_slot[j - 1];
          --j;
        }
        t.cf_ent[j] = m.owner[f] == (int)i + 1 ? f + 1 : -(f + 1);
        t.cf_slot[j] = k;
      }
    });
  }
  t.cb_ptr.assign(n + 1, 0);
  for (int ty = 0; ty < B_NTYPES; ++ty)
    for (int i = 0; i < cnt[ty]; ++i) t.cb_ptr[m.owner[fst[ty] + i]]++;
  for (int i = 0; i < n; ++i) t.cb_ptr[i + 1] += t.cb_ptr[i];
  t.cb_face.assign(t.cb_ptr[n], 0);
  t.cb_slot.assign(t.cb_ptr[n], 0);
  t.cb_type.assign(t.cb_ptr[n], 0);
  {
    std::vector<int> fill(t.cb_ptr.begin(), t.cb_ptr.end() - 1);
    for (int ty = 0; ty < B_NTYPES; ++ty)
      for (int i = 0; i < cnt[ty]; ++i) {
        int face = fst[ty] + i, c = m.owner[face] - 1;
        int e = fill[c]++;
        t.cb_face[e] = face;
        t.cb_slot[e] = bst[ty] + i;
        t.cb_type[e] = ty;
      }
  }
  t.cbf_ptr.assign(n + 1, 0);
  for (int f = nin; f < nf; ++f) t.cbf_ptr[m.owner[f]]++;
  for (int i = 0; i < n; ++i) t.cbf_ptr[i + 1] += t.cbf_ptr[i];
  t.cbf_face.assign(t.cbf_ptr[n], 0);
  {
    std::vector<int> fill(t.cbf_ptr.begin(), t.cbf_ptr.end() - 1);
    for (int f = nin; f < nf; ++f) t.cbf_face[fill[m.owner[f] - 1]++] = f;
  }

  // --- sliced ELL with offset-uniform slices ------------------------------------
  // A slice is "uniform" when it is cheaper to store, per slot j, one column offset
  // shared by its 32 rows (slot j of row r reads column r + off[j]; a row without that
  // offset gets the value 0) than 32 explicit columns.  Uniform slots follow the
  // ascending offsets, so every row still meets its entries in CSR column order.  On a
  // hex mesh numbered i-fastest every slice is uniform with the 7 offsets
  // -N^2, -N, -1, 0, 1, N, N^2, and the SpMV reads no column indices at all.
  const int ns = (n + 31) / 32;
  t.sell_ptr.assign(ns + 1, 0);
  t.sell_width.assign(ns, 0);
  t.sell_kind.assign(ns, 0);
  t.sell_offp.assign(ns + 1, 0);
  t.sell_maxw = 0;
  std::vector<std::vector<int>> uoffs(ns);
  std::vector<int> ecols(ns, 0);  // explicit column block size per slice
  parallel_for(ns, [&](long long sl) {
    int wexp = 0;
    thread_local std::vector<int> u;
    u.clear();
    for (long long r = 32 * sl; r < std::min<long long>(n, 32 * sl + 32); ++r) {
      wexp = std::max(wexp, t.ioffset[r + 1] - t.ioffset[r]);
      for (int k = t.ioffset[r] - 1; k < t.ioffset[r + 1] - 1; ++k) u.push_back(t.ja[k] - 1 - (int)r);
    }
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    if (!u.empty() && 2 * (long long)u.size() < 3LL * wexp) {  // 8w_u < 12w_e bytes per row
      t.sell_kind[sl] = 0;
      t.sell_width[sl] = (int)u.size();
      uoffs[sl] = u;
    } else {
      t.sell_kind[sl] = 1;
      t.sell_width[sl] = wexp;
      ecols[sl] = 32 * wexp;
    }
  });
  for (int sl = 0; sl < ns; ++sl) {
    int w = t.sell_width[sl];
    t.sell_maxw = std::max(t.sell_maxw, w);
    t.sell_ptr[sl + 1] = t.sell_ptr[sl] + 32LL * w;
    t.sell_offp[sl + 1] = t.sell_offp[sl] + (t.sell_kind[sl] == 0 ? w : 0);
  }
  // explicit column blocks are stored after the offset table, in one index array
  std::vector<long long> colp(ns + 1, 0);
  for (int sl = 0; sl < ns; ++sl) colp[sl + 1] = colp[sl] + ecols[sl];
  t.sell_off.assign(t.sell_offp[ns] + colp[ns], 0);
  t.sell_src.assign(t.sell_ptr[ns], -1);
  parallel_for(ns, [&](long long sl) {
    int w = t.sell_width[sl];
    if (t.sell_kind[sl] == 0) {
      const std::vector<int> &u = uoffs[sl];
      for (int j = 0; j < w; ++j) t.sell_off[t.sell_offp[sl] + j] = u[j];
    } else {
      t.sell_offp[sl] = (int)(t.sell_offp[ns] + colp[sl]);  // explicit: start of the column block
    }
    for (int lane = 0; lane < 32; ++lane) {
      long long r = 32 * sl + lane;
      int b = r < n ? t.ioffset[r] - 1 : 0, e = r < n ? t.ioffset[r + 1] - 1 : 0;
      for (int j = 0; j < w; ++j) {
        long long pos = t.sell_ptr[sl] + (long long)j * 32 + lane;
        if (t.sell_kind[sl] == 0) {
          int want = (int)r + uoffs[sl][j] + 1;  // 1-based column for this slot
          for (int k = b; k < e; ++k)
            if (t.ja[k] == want) t.sell_src[pos] = k;
        } else {
          long long cpos = t.sell_offp[sl] + (long long)j * 32 + lane;
          if (j < e - b) {
            t.sell_off[cpos] = t.ja[b + j] - 1;
            t.sell_src[pos] = b + j;
          } else {
            t.sell_off[cpos] = (int)std::min<long long>(r, n - 1);
          }
        }
      }
    }
  });
  t.sell_nuniform = 0;
  for (int sl = 0; sl < ns; ++sl) t.sell_nuniform += t.sell_kind[sl] == 0;

  // --- level schedules -----------------------------------------------------------
  std::vector<int> lev(n, 0);
  int nlev = 0;
  for (int i = 0; i < n; ++i) {
    int l = 0;
    for (int k = t.ioffset[i] - 1; k < t.diag[i] - 1; ++k) l = std::max(l, lev[t.ja[k] - 1] + 1);
    lev[i] = l;
    nlev = std::max(nlev, l + 1);
  }
  t.lf_ptr.assign(nlev + 1, 0);
  for (int i = 0; i < n; ++i) t.lf_ptr[lev[i] + 1]++;
  for (int l = 0; l < nlev; ++l) t.lf_ptr[l + 1] += t.lf_ptr[l];
  t.lf_rows.assign(n, 0);
  {
    std::vector<int> fill(t.lf_ptr.begin(), t.lf_ptr.end() - 1);
    for (int i = 0; i < n; ++i) t.lf_rows[fill[lev[i]]++] = i;
  }
  nlev = 0;
  for (int i = n - 1; i >= 0; --i) {
    int l = 0;
    for (int k = t.diag[i]; k < t.ioffset[i + 1] - 1; ++k) l = std::max(l, lev[t.ja[k] - 1] + 1);
    lev[i] = l;
    nlev = std::max(nlev, l + 1);
  }
  t.lb_ptr.assign(nlev + 1, 0);
  for (int i = 0; i < n; ++i) t.lb_ptr[lev[i] + 1]++;
  for (int l = 0; l < nlev; ++l) t.lb_ptr[l + 1] += t.lb_ptr[l];
  t.lb_rows.assign(n, 0);
  {
    std::vector<int> fill(t.lb_ptr.begin(), t.lb_ptr.end() - 1);
    for (int i = 0; i < n; ++i) t.lb_rows[fill[lev[i]]++] = i;
  }
  return FCG_OK;
}

}  // namespace fcg

extern "C" int fcg_csr_build(int numCells, int numInnerFaces, const int *owner,
                             const int *neighbour, int *ioffset, int *ja, int *diag, int *slot_pn,
                             int *slot_np) {
  if (numCells <= 0 || numInnerFaces < 0 || (numInnerFaces > 0 && (!owner || !neighbour)) ||
      !ioffset || !ja || !diag || (numInnerFaces > 0 && (!slot_pn || !slot_np)))
    return FCG_ERR_ARG;
  fcg_mesh_desc m{};
  m.numCells = numCells;
  m.numFaces = numInnerFaces;
  m.numInnerFaces = numInnerFaces;
  m.owner = owner;
  m.neighbour = neighbour;
  const int zero[fcg::B_NTYPES] = {0, 0, 0, 0, 0};
  fcg::HostTopology t;
  std::string err;
  int rc = fcg::build_topology(m, zero, zero, zero, t, err);
  if (rc) return rc;
  std::copy(t.ioffset.begin(), t.ioffset.end(), ioffset);
  std::copy(t.ja.begin(), t.ja.end(), ja);
  std::copy(t.diag.begin(), t.diag.end(), diag);
  std::copy(t.slot_pn.begin(), t.slot_pn.end(), slot_pn);
  std::copy(t.slot_np.begin(), t.slot_np.end(), slot_np);
  return FCG_OK;
}
