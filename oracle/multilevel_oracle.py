"""numpy oracle of the learned FCG's coarse-grid correction (aggregation.cpp and
coarse.cu in libfcgpu.so).

TEST INFRASTRUCTURE ONLY: the checker for the hierarchy and the correction kernels; only
``tests/`` may import it.  The correction has no counterpart in the reference (it
belongs to the learned preconditioner, which preconditions flexible CG in place of the
Jacobi step of dpcg.f90:85-100), so nothing of the reference pins it: this module
restates the algorithm as the library documents it, and tests/test_multilevel.py checks
the restatement itself against scipy's sparse products and a CG it preconditions.

* Aggregation: per level, three passes of pairwise matching.  Rows are visited in
  ascending order; an unmatched row pairs with its unmatched neighbour of most negative
  coupling (strictly below every earlier candidate, so ties keep the lowest column) or
  stays single.  Then every row left single, in ascending order, joins the matched pair
  (as matched, not as grown by earlier joins) it is most negatively coupled to, if any,
  and the aggregates are renumbered in their order.  Between passes the matrix is
  P^T A P summed in a fixed order: member rows ascending, each member row's entries in
  column order, each entry added to the slot of its coarse column in the order the
  slots are first met; rows then sorted by column.  A pass that pairs nothing ends the
  level; a level with more than 90% of the rows above it is dropped; a level with at
  most dense_max rows is the coarsest.
* Device values: level 1 is P^T Ahat P of the fine scaled matrix in FP32
  (FP32((a_ij s_i) s_j), s = 1/sqrt(a_ii)), level l + 1 of level l's device values,
  all with the composite aggregation of the level and the summation order above, every
  sum rounded to FP32 (bit-exact with the GPU).
* Smoothed first level (the default): P = (I - omega D^-1 Ahat) P_tent, its pattern the
  row's own and its neighbours' aggregates; A P and P^T A P summed in the documented
  orders (host FP64, device FP32 with every product and sum rounded).
* Correction: out = z + alpha P V(P^T (r - Ahat z)), V as in coarse.cu (alpha = 1 for
  the smoothed P).
"""
from __future__ import annotations

import numpy as np


def scaled_csr(ioffset, ja, diag, a):
    """0-based (ptr, col, val) of Ahat = D^-1/2 A D^-1/2 from the reference's 1-based CSR."""
    ptr = np.asarray(ioffset, np.int64) - 1
    col = np.asarray(ja, np.int64) - 1
    a = np.asarray(a, np.float64)
    s = 1.0 / np.sqrt(a[np.asarray(diag) - 1])
    rows = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr))
    return ptr, col, (a * s[rows]) * s[col]


def pair_match(ptr, col, val):
    n = len(ptr) - 1
    agg = np.full(n, -1, np.int64)
    nc = 0
    ptr_l, col_l, val_l = ptr.tolist(), col.tolist(), val.tolist()
    ag = agg.tolist()
    paired = []
    for i in range(n):
        if ag[i] >= 0:
            continue
        best, bv = -1, 0.0
        for k in range(ptr_l[i], ptr_l[i + 1]):
            j = col_l[k]
            if j == i or ag[j] >= 0:
                continue
            if val_l[k] < bv:
                bv, best = val_l[k], j
        ag[i] = nc
        if best >= 0:
            ag[best] = nc
        paired.append(best >= 0)
        nc += 1
    moved = False
    for i in range(n):
        if paired[ag[i]]:
            continue
        best, bv = -1, 0.0
        for k in range(ptr_l[i], ptr_l[i + 1]):
            j = col_l[k]
            if j == i or not paired[ag[j]]:
                continue
            if val_l[k] < bv:
                bv, best = val_l[k], j
        if best >= 0:
            ag[i] = ag[best]
            moved = True
    agg = np.array(ag, np.int64)
    if not moved:
        return agg, nc
    used = np.zeros(nc, bool)
    used[agg] = True
    ids = np.cumsum(used) - 1
    return ids[agg], int(used.sum())


def members(agg, nc):
    mptr = np.zeros(nc + 1, np.int64)
    np.add.at(mptr, np.asarray(agg) + 1, 1)
    mptr = np.cumsum(mptr)
    mem = np.argsort(agg, kind="stable")
    return mptr, mem


def galerkin(ptr, col, val, agg, nc, mptr, mem, f32=False):
    """P^T A P in the documented order, in FP64 or (f32) with every sum rounded to FP32;
    returns (ptr, col, val)."""
    ptr_l, col_l = ptr.tolist(), col.tolist()
    val_l = list(np.asarray(val, np.float32)) if f32 else val.tolist()
    agg_l, mptr_l, mem_l = list(agg), mptr.tolist(), mem.tolist()
    optr, ocol, oval = [0], [], []
    for I in range(nc):
        slot = {}
        cols, vals = [], []
        for m in range(mptr_l[I], mptr_l[I + 1]):
            i = mem_l[m]
            for k in range(ptr_l[i], ptr_l[i + 1]):
                J = agg_l[col_l[k]]
                p = slot.get(J)
                if p is None:
                    slot[J] = len(cols)
                    cols.append(J)
                    vals.append(val_l[k])
                else:
                    vals[p] += val_l[k]
        order = sorted(range(len(cols)), key=lambda q: cols[q])
        ocol += [cols[q] for q in order]
        oval += [vals[q] for q in order]
        optr.append(len(ocol))
    return (np.array(optr, np.int64), np.array(ocol, np.int64),
            np.array(oval, np.float32 if f32 else np.float64))


def smoothed_level(ptr, col, val, agg, nc, omega):
    """P = (I - omega D^-1 A) P_tent, A P and P^T A P of the first level in FP64, in the
    host's order; returns the pattern dict (p_ptr, p_col, t_ptr, t_row, t_pos, ap_ptr,
    ap_col) and (ptr, col, val) of P^T A P."""
    n = len(ptr) - 1
    ptr_l, col_l, val_l, agg_l = ptr.tolist(), col.tolist(), val.tolist(), list(agg)
    p_ptr, p_col, pv = [0], [], []
    for i in range(n):
        ks = range(ptr_l[i], ptr_l[i + 1])
        row = sorted({agg_l[i]} | {agg_l[col_l[k]] for k in ks})
        b = len(p_col)
        d = 0.0
        for k in ks:
            if col_l[k] == i:
                d = val_l[k]
        w = omega / d if d > 0.0 else 0.0
        p_col += row
        pv += [1.0 if J == agg_l[i] else 0.0 for J in row]
        for k in ks:
            q = b + row.index(agg_l[col_l[k]])
            pv[q] = pv[q] - w * val_l[k]
        p_ptr.append(len(p_col))
    t_lists = [[] for _ in range(nc)]
    for i in range(n):
        for q in range(p_ptr[i], p_ptr[i + 1]):
            t_lists[p_col[q]].append((i, q))
    t_ptr = np.cumsum([0] + [len(t) for t in t_lists])
    t_row = [i for t in t_lists for i, _ in t]
    t_pos = [q for t in t_lists for _, q in t]
    ap_ptr, ap_col, apv = [0], [], []
    for i in range(n):
        ks = range(ptr_l[i], ptr_l[i + 1])
        row = sorted({p_col[q] for k in ks for q in range(p_ptr[col_l[k]], p_ptr[col_l[k] + 1])})
        b = len(ap_col)
        ap_col += row
        apv += [0.0] * len(row)
        for k in ks:
            j = col_l[k]
            for q in range(p_ptr[j], p_ptr[j + 1]):
                x = b + row.index(p_col[q])
                apv[x] = apv[x] + val_l[k] * pv[q]
        ap_ptr.append(len(ap_col))
    optr, ocol, oval = [0], [], []
    for I in range(nc):
        slot, cols, vals = {}, [], []
        for m in range(t_ptr[I], t_ptr[I + 1]):
            i, p = t_row[m], pv[t_pos[m]]
            for q in range(ap_ptr[i], ap_ptr[i + 1]):
                J = ap_col[q]
                if J in slot:
                    vals[slot[J]] += p * apv[q]
                else:
                    slot[J] = len(cols)
                    cols.append(J)
                    vals.append(p * apv[q])
        order = sorted(range(len(cols)), key=lambda q: cols[q])
        ocol += [cols[q] for q in order]
        oval += [vals[q] for q in order]
        optr.append(len(ocol))
    pat = dict(p_ptr=np.array(p_ptr), p_col=np.array(p_col), t_ptr=np.asarray(t_ptr),
               t_row=np.array(t_row), t_pos=np.array(t_pos), ap_ptr=np.array(ap_ptr),
               ap_col=np.array(ap_col), p_val64=np.array(pv))
    return pat, (np.array(optr, np.int64), np.array(ocol, np.int64), np.array(oval))


def smoothed_values32(pat, fine32, agg, level, omega):
    """The device's FP32 values of the smoothed first level: P, A P and P^T A P, every
    product and sum rounded to FP32 in the host's order; returns (p_val, a1)."""
    f = np.float32
    ptr, col, val = fine32
    ptr_l, col_l = ptr.tolist(), col.tolist()
    val_l = list(np.asarray(val, np.float32))
    n = len(ptr) - 1
    om = f(omega)
    p_ptr, p_col = pat["p_ptr"].tolist(), pat["p_col"].tolist()
    pv = [f(0)] * len(p_col)
    for i in range(n):
        ks = range(ptr_l[i], ptr_l[i + 1])
        d = f(0)
        for k in ks:
            if col_l[k] == i:
                d = val_l[k]
        w = om / d if d > f(0) else f(0)
        row = p_col[p_ptr[i]:p_ptr[i + 1]]
        for q in range(p_ptr[i], p_ptr[i + 1]):
            pv[q] = f(1) if p_col[q] == agg[i] else f(0)
        for k in ks:
            q = p_ptr[i] + row.index(agg[col_l[k]])
            pv[q] = pv[q] - w * val_l[k]
    ap_ptr, ap_col = pat["ap_ptr"].tolist(), pat["ap_col"].tolist()
    apv = [f(0)] * len(ap_col)
    for i in range(n):
        row = ap_col[ap_ptr[i]:ap_ptr[i + 1]]
        for k in range(ptr_l[i], ptr_l[i + 1]):
            j = col_l[k]
            for q in range(p_ptr[j], p_ptr[j + 1]):
                x = ap_ptr[i] + row.index(p_col[q])
                apv[x] = apv[x] + val_l[k] * pv[q]
    t_ptr, t_row, t_pos = pat["t_ptr"].tolist(), pat["t_row"].tolist(), pat["t_pos"].tolist()
    cptr, ccol = level["ptr"].tolist(), level["col"].tolist()
    a1 = [f(0)] * len(ccol)
    for I in range(len(cptr) - 1):
        pos = {J: q for q, J in enumerate(ccol[cptr[I]:cptr[I + 1]], start=cptr[I])}
        for m in range(t_ptr[I], t_ptr[I + 1]):
            i, p = t_row[m], pv[t_pos[m]]
            for q in range(ap_ptr[i], ap_ptr[i + 1]):
                x = pos[ap_col[q]]
                a1[x] = a1[x] + p * apv[q]
    return np.array(pv, np.float32), np.array(a1, np.float32)


def build_levels(ptr, col, val, max_levels=10, dense_max=128, passes=3, sa_omega=0.67):
    """Levels below (ptr, col, val): dicts with n, agg, mptr, mem, ptr, col, hval, and for
    a smoothed first level (sa_omega > 0) the pattern dict "sa"."""
    levels = []
    cur = (ptr, col, val)
    while len(levels) + 1 < max_levels:
        n0 = len(cur[0]) - 1
        if n0 < 2:
            break
        comp = np.arange(n0)
        a = cur
        nc = n0
        for _ in range(passes):
            agg, m = pair_match(*a)
            if m == len(a[0]) - 1:
                break
            mp, me = members(agg, m)
            a = galerkin(*a, agg, m, mp, me)
            comp = agg[comp]
            nc = m
            if nc <= dense_max:
                break
        if nc == n0 or 10 * nc > 9 * n0:
            break
        mp, me = members(comp, nc)
        lv = dict(n=nc, agg=comp, mptr=mp, mem=me, ptr=a[0], col=a[1], hval=a[2])
        if not levels and sa_omega > 0:
            lv["sa"], a = smoothed_level(*cur, comp, nc, sa_omega)
            lv["ptr"], lv["col"], lv["hval"] = a
        levels.append(lv)
        cur = a
        if nc <= dense_max:
            break
    return levels


def level_values(levels, fine, f32=True, omega=0.67):
    """Values of every level as the device computes them: level 1 from the fine scaled
    matrix rounded to FP32, each level from the one above, FP32 sums in order (f32=False:
    the same products in FP64 from the fine values as given).  A smoothed first level
    also gets its FP32 (or FP64) prolongation values in levels[0]["p_val"]."""
    out = []
    above = (fine[0], fine[1], np.asarray(fine[2], np.float32 if f32 else np.float64))
    for lv in levels:
        if "sa" in lv:
            if f32:
                lv["p_val"], v = smoothed_values32(lv["sa"], above, lv["agg"], lv, omega)
            else:
                lv["p_val"], v = lv["sa"]["p_val64"], lv["hval"]
            out.append(v)
            above = (lv["ptr"], lv["col"], v)
            continue
        _, _, v = galerkin(*above, lv["agg"], lv["n"], lv["mptr"], lv["mem"], f32=f32)
        out.append(v)
        above = (lv["ptr"], lv["col"], v)
    return out


def _spmv(ptr, col, val, x):
    rows = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr))
    y = np.zeros(len(ptr) - 1)
    np.add.at(y, rows, val * x[col])
    return y


class Cycle:
    """The V-cycle of coarse.cu in FP64 on the oracle's hierarchy."""

    def __init__(self, fine, levels, values, alpha=1.8, omega=0.67, sweeps=2, dense_max=128):
        self.fine, self.levels, self.values = fine, levels, values
        self.alpha, self.omega, self.sweeps = alpha, omega, sweeps
        self.mats = [(lv["ptr"], lv["col"], np.asarray(v, np.float64))
                     for lv, v in zip(levels, values)]
        self.dinv = []
        for (p, c, v) in self.mats:
            rows = np.repeat(np.arange(len(p) - 1), np.diff(p))
            d = v[rows == c]
            self.dinv.append(np.where(d > 0, 1.0 / d, 0.0))
        last = self.mats[-1] if self.mats else None
        self.dense = None
        if last is not None and len(last[0]) - 1 <= dense_max:
            n = len(last[0]) - 1
            A = np.zeros((n, n))
            rows = np.repeat(np.arange(n), np.diff(last[0]))
            A[rows, last[1]] = last[2]
            self.dense = np.linalg.inv(A)

    def _restrict(self, k, t):
        lv = self.levels[k]
        bc = np.zeros(lv["n"])
        if "sa" in lv:
            sa = lv["sa"]
            rows = np.repeat(np.arange(len(t)), np.diff(sa["p_ptr"]))
            np.add.at(bc, sa["p_col"], np.asarray(lv["p_val"], np.float64) * t[rows])
        else:
            np.add.at(bc, lv["agg"], t)
        return bc

    def _prolong(self, k, e):
        """(P e, scale): the smoothed P (not scaled) or the aggregation (alpha)."""
        lv = self.levels[k]
        if "sa" in lv:
            sa = lv["sa"]
            rows = np.repeat(np.arange(len(lv["agg"])), np.diff(sa["p_ptr"]))
            out = np.zeros(len(lv["agg"]))
            np.add.at(out, rows, np.asarray(lv["p_val"], np.float64) * e[sa["p_col"]])
            return out, 1.0
        return e[lv["agg"]], self.alpha

    def vcycle(self, k, b):
        A, dinv = self.mats[k], self.dinv[k]
        om, al = self.omega, self.alpha
        last = k + 1 == len(self.mats)
        if last and self.dense is not None:
            return self.dense @ b
        x = om * dinv * b
        pre = 2 * self.sweeps + 2 if last else self.sweeps
        for _ in range(pre - 1):
            x = x + om * dinv * (b - _spmv(*A, x))
        if last:
            return x
        bc = self._restrict(k + 1, b - _spmv(*A, x))
        e = self.vcycle(k + 1, bc)
        x = x + al * e[self.levels[k + 1]["agg"]]
        for _ in range(self.sweeps):
            x = x + om * dinv * (b - _spmv(*A, x))
        return x

    def correct(self, r, z):
        """z + alpha P V(P^T (r - Ahat z))."""
        r, z = np.asarray(r, np.float64), np.asarray(z, np.float64)
        if not self.levels:
            return z.copy()
        t = r - _spmv(*self.fine, z)
        e = self.vcycle(0, self._restrict(0, t))
        pe, a = self._prolong(0, e)
        return z + a * pe

    def jacobi_cycle(self, r):
        """The same cycle with Jacobi sweeps (unit diagonal) in place of the network."""
        r = np.asarray(r, np.float64)
        om = self.omega
        z = om * r
        for _ in range(self.sweeps - 1):
            z = z + om * (r - _spmv(*self.fine, z))
        z = self.correct(r, z)
        for _ in range(self.sweeps):
            z = z + om * (r - _spmv(*self.fine, z))
        return z


def hierarchy(ioffset, ja, diag, a, max_levels=10, dense_max=128, passes=3, sa_omega=0.67,
              **cycle):
    """Everything for one scaled matrix: (fine csr, levels, device values, Cycle)."""
    fine = scaled_csr(ioffset, ja, diag, a)
    levels = build_levels(*fine, max_levels=max_levels, dense_max=dense_max, passes=passes,
                          sa_omega=sa_omega)
    values = level_values(levels, fine, omega=sa_omega)
    return fine, levels, values, Cycle(fine, levels, values, dense_max=dense_max, **cycle)
