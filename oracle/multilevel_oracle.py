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
  slots are first met; rows then sorted by column.  A pass that pairs nothing ends the level; a level with more than 90% of the
  rows above it is dropped; a level with at most dense_max rows is the coarsest.
* Device values: level 1 is P^T Ahat P of the fine scaled matrix in FP32
  (FP32((a_ij s_i) s_j), s = 1/sqrt(a_ii)), level l + 1 of level l's device values,
  all with the composite aggregation of the level and the summation order above, every
  sum rounded to FP32 (bit-exact with the GPU).
* Correction: out = z + alpha P V(P^T (r - Ahat z)), V as in coarse.cu.
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


def build_levels(ptr, col, val, max_levels=10, dense_max=128, passes=3):
    """Levels below (ptr, col, val): dicts with n, agg, mptr, mem, ptr, col, hval."""
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
        levels.append(dict(n=nc, agg=comp, mptr=mp, mem=me, ptr=a[0], col=a[1], hval=a[2]))
        cur = a
        if nc <= dense_max:
            break
    return levels


def level_values(levels, fine, f32=True):
    """Values of every level as the device computes them: level 1 from the fine scaled
    matrix rounded to FP32, each level from the one above, FP32 sums in order (f32=False:
    the same products in FP64 from the fine values as given)."""
    out = []
    above = (fine[0], fine[1], np.asarray(fine[2], np.float32 if f32 else np.float64))
    for lv in levels:
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
        np.add.at(bc, lv["agg"], t)
        return bc

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
        return z + self.alpha * e[self.levels[0]["agg"]]

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


def hierarchy(ioffset, ja, diag, a, max_levels=10, dense_max=128, passes=3, **cycle):
    """Everything for one scaled matrix: (fine csr, levels, device values, Cycle)."""
    fine = scaled_csr(ioffset, ja, diag, a)
    levels = build_levels(*fine, max_levels=max_levels, dense_max=dense_max, passes=passes)
    values = level_values(levels, fine)
    return fine, levels, values, Cycle(fine, levels, values, dense_max=dense_max, **cycle)
