"""Coarse-grid correction of the learned FCG (aggregation.cpp, coarse.cu).

CPU: the oracle's Galerkin products against scipy's P^T A P, its aggregates (every
row in one, connected, about eight rows), and CG preconditioned by its cycle against
plain Jacobi.  GPU: the library's hierarchy (aggregation, members, pattern) is the
oracle's element for element and its FP32 level matrices bit for bit; the correction agrees
with the oracle's FP64 cycle to FP32 rounding; the preconditioner is the network
followed by the correction; the flexible CG with the correction converges in a fraction
of the iterations without it, and the trained network beats Jacobi sweeps in the same
cycle; options are checked."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from oracle import multilevel_oracle as mo
from oracle import oracle

from tests.meshes import mesh_by_name, oracle_csr, oracle_mesh


def _system(m, variable=True, seed=3):
    from freecappuccino_gb300.learned import diffusivity_field

    om, csr = oracle_mesh(m), oracle_csr(m)
    gam = diffusivity_field(m, seed) if variable else np.ones(m.numCells)
    su0 = fcg.uniform(seed, 0, m.numCells) * m.vol
    a, su = oracle.laplacian(om, csr, -gam, np.zeros(m.numTotal), su0)
    return csr, a, su


def _scipy(ptr, col, val):
    import scipy.sparse as sp

    n = len(ptr) - 1
    return sp.csr_matrix((val, col, ptr), shape=(n, n))


# ----------------------------------------------------------------------------- CPU
@pytest.mark.parametrize("name", ["cavity", "hex10"])
def test_oracle_galerkin_is_ptap(name):
    sp = pytest.importorskip("scipy.sparse")
    m = mesh_by_name(name)
    csr, a, _ = _system(m)
    fine = mo.scaled_csr(csr.ioffset, csr.ja, csr.diag, a)
    levels = mo.build_levels(*fine)
    vals = mo.level_values(levels, fine)
    above = _scipy(*fine)
    for lv, v in zip(levels, vals):
        n0 = above.shape[0]
        if "sa" in lv:  # the smoothed first level: P = (I - omega D^-1 A) P_tent
            Pt = sp.csr_matrix((np.ones(n0), (np.arange(n0), lv["agg"])), shape=(n0, lv["n"]))
            P = (Pt - 0.67 * sp.diags(1.0 / above.diagonal()) @ (above @ Pt)).tocsr()
            P.sort_indices()
            sa = lv["sa"]
            Pg = sp.csr_matrix((sa["p_val64"], sa["p_col"], sa["p_ptr"]), shape=P.shape)
            assert abs(Pg - P).max() <= 1e-15 * abs(P).max()
            assert np.abs(lv["p_val"] - sa["p_val64"]).max() <= 1e-6
            tol32 = 2e-5  # FP32 P, A P and P^T A P
        else:
            P = sp.csr_matrix((np.ones(n0), (np.arange(n0), lv["agg"])), shape=(n0, lv["n"]))
            tol32 = 2e-6
        ref = (P.T @ above @ P).tocsr()
        ref.sort_indices()
        got = _scipy(lv["ptr"], lv["col"], v.astype(np.float64))
        assert np.array_equal(ref.indptr, got.indptr) and np.array_equal(ref.indices, got.indices)
        # device values: FP32 sums of the FP32-rounded fine matrix
        assert np.abs(ref.data - got.data).max() <= tol32 * np.abs(ref.data).max()
        # the host values that steered the matching: the same product in FP64
        assert np.abs(lv["hval"] - ref.data).max() <= 1e-14 * np.abs(ref.data).max()
        above = _scipy(lv["ptr"], lv["col"], lv["hval"])


def test_oracle_aggregates_are_connected_and_small():
    m = mesh_by_name("hex16")
    csr, a, _ = _system(m)
    fine = mo.scaled_csr(csr.ioffset, csr.ja, csr.diag, a)
    levels = mo.build_levels(*fine)
    assert len(levels) >= 2
    ptr, col = fine[0], fine[1]
    for l, lv in enumerate(levels):
        sizes = np.diff(lv["mptr"])
        assert sizes.min() >= 1 and sizes.max() <= 64 and sizes.sum() == len(lv["agg"])
        if l + 1 < len(levels):  # three full passes: about eight-fold on a hex mesh
            assert lv["n"] < 0.2 * len(lv["agg"])
        for I in range(lv["n"]):  # connected inside the level above
            mem = set(lv["mem"][lv["mptr"][I]:lv["mptr"][I + 1]].tolist())
            seen, stack = set(), [next(iter(mem))]
            while stack:
                i = stack.pop()
                if i in seen:
                    continue
                seen.add(i)
                stack += [j for j in col[ptr[i]:ptr[i + 1]].tolist() if j in mem]
            assert seen == mem
        ptr, col = lv["ptr"], lv["col"]


def test_oracle_cycle_preconditions_cg():
    """CG on the scaled 16^3 system: the oracle's Jacobi cycle needs a fraction of the
    iterations of plain Jacobi, and the network-free correction alone (z = 0) is
    symmetric to FP32 rounding (a valid CG preconditioner)."""
    m = mesh_by_name("hex16")
    csr, a, su = _system(m)
    fine, levels, values, cyc = mo.hierarchy(csr.ioffset, csr.ja, csr.diag, a)
    A = _scipy(*fine)
    s = 1.0 / np.sqrt(a[csr.diag - 1])
    b = s * su

    def pcg(M, tol=1e-8):
        x = np.zeros_like(b)
        r = b.copy()
        r0 = np.abs(r).sum()
        z = M(r)
        p = z.copy()
        rz = r @ z
        for it in range(1, 2000):
            q = A @ p
            al = rz / (p @ q)
            x += al * p
            r -= al * q
            if np.abs(r).sum() / r0 < tol:
                return it
            z = M(r)
            rz2 = r @ z
            p = z + rz2 / rz * p
            rz = rz2
        return 2000

    jac = pcg(lambda r: r.copy())
    cyc_it = pcg(cyc.jacobi_cycle)
    assert cyc_it < jac / 4
    rng = np.random.default_rng(0)
    u, v = rng.standard_normal(m.numCells), rng.standard_normal(m.numCells)
    zero = np.zeros(m.numCells)
    cu, cv = cyc.correct(u, zero), cyc.correct(v, zero)
    # symmetric up to the FP32 rounding of the level matrices ((I,J) and (J,I) add the
    # same terms in different orders)
    assert abs(u @ cv - v @ cu) <= 1e-5 * abs(u @ cv)
    print(f"\n16^3: CG iterations Jacobi {jac}, Jacobi V-cycle {cyc_it}")


def _host_aggregate(ptr, col, val, dense_max=128, passes=3):
    from freecappuccino_gb300 import _lib

    ptr, col = np.ascontiguousarray(ptr, np.int32), np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    n = len(ptr) - 1
    agg = np.zeros(max(n, 1), np.int32)
    nc = np.zeros(1, np.int32)
    rc = _lib.load().fcg_aggregate(n, ptr.ctypes.data, col.ctypes.data, val.ctypes.data,
                                   passes, dense_max, agg.ctypes.data,
                                   nc.ctypes.data_as(np.ctypeslib.ctypes.POINTER(np.ctypeslib.ctypes.c_int)))
    return rc, agg[:n], int(nc[0])


@pytest.mark.parametrize("name", ["cavity", "pitzdaily", "hexmix8", "hex16"])
def test_host_aggregation_matches_oracle(name):
    """The library's host matching and Galerkin passes (fcg_aggregate) against the
    oracle's, level by level, element for element."""
    m = mesh_by_name(name)
    csr, a, _ = _system(m)
    fine = mo.scaled_csr(csr.ioffset, csr.ja, csr.diag, a)
    levels = mo.build_levels(*fine)
    above = fine
    for lv in levels:
        rc, agg, nc = _host_aggregate(*above)
        assert rc == 0 and nc == lv["n"] and np.array_equal(agg, lv["agg"])
        above = (lv["ptr"], lv["col"], lv["hval"])


def _host_smoothed(ptr, col, val, agg, nc, omega=0.67):
    import ctypes as C

    from freecappuccino_gb300 import _lib

    lib = _lib.load()
    ptr, col = np.ascontiguousarray(ptr, np.int32), np.ascontiguousarray(col, np.int32)
    val, agg = np.ascontiguousarray(val, np.float64), np.ascontiguousarray(agg, np.int32)
    n = len(ptr) - 1
    nnz = C.c_longlong(0)
    rc = lib.fcg_smoothed_level(n, ptr.ctypes.data, col.ctypes.data, val.ctypes.data,
                                agg.ctypes.data, nc, omega, C.byref(nnz), None, None, None)
    if rc:
        return rc, None
    out = (np.zeros(nc + 1, np.int32), np.zeros(nnz.value, np.int32), np.zeros(nnz.value))
    rc = lib.fcg_smoothed_level(n, ptr.ctypes.data, col.ctypes.data, val.ctypes.data,
                                agg.ctypes.data, nc, omega, C.byref(nnz),
                                *[o.ctypes.data for o in out])
    return rc, out


@pytest.mark.parametrize("name", ["cavity", "pitzdaily", "hexmix8", "hex16"])
def test_host_smoothed_level_matches_oracle(name):
    """The library's host construction of the smoothed first level (P, A P, P^T A P on
    all host threads, joined in order) against the oracle's, element for element."""
    m = mesh_by_name(name)
    csr, a, _ = _system(m)
    fine = mo.scaled_csr(csr.ioffset, csr.ja, csr.diag, a)
    lv = mo.build_levels(*fine)[0]
    assert "sa" in lv
    rc, (cptr, ccol, cval) = _host_smoothed(*fine, lv["agg"], lv["n"])
    assert rc == 0
    assert np.array_equal(cptr, lv["ptr"]) and np.array_equal(ccol, lv["col"])
    assert np.array_equal(cval, lv["hval"])


def test_host_smoothed_level_rejects_bad_input():
    from freecappuccino_gb300 import _lib

    ptr, col, val = np.array([0, 2, 4]), np.array([0, 1, 0, 1]), np.array([2.0, -1, -1, 2])
    assert _host_smoothed(ptr, col, val, np.array([0, 0]), 1)[0] == 0
    assert _host_smoothed(ptr, col, val, np.array([0, 2]), 1)[0] == _lib.FCG_ERR_INDEX
    assert _host_smoothed(ptr, np.array([0, 1, 1, 0]), val, np.array([0, 0]), 1)[0] == \
        _lib.FCG_ERR_INDEX
    assert _host_smoothed(ptr, col, val, np.array([0, 0]), 1, omega=0.0)[0] == _lib.FCG_ERR_ARG


def test_host_aggregation_rejects_malformed_csr():
    from freecappuccino_gb300 import _lib

    ptr, col, val = np.array([0, 2, 3]), np.array([0, 1, 1]), np.array([2.0, -1.0, 2.0])
    assert _host_aggregate(ptr, col, val)[0] == 0
    for p_, c_ in ((np.array([0, 2, 3]), np.array([0, 5, 1])),   # column out of range
                   (np.array([0, 2, 3]), np.array([1, 0, 1])),   # not ascending
                   (np.array([1, 2, 3]), np.array([0, 1, 1]))):  # ptr[0] != 0
        assert _host_aggregate(p_, c_, val)[0] == _lib.FCG_ERR_INDEX


# ----------------------------------------------------------------------------- GPU
def _gpu(name, variable=True):
    from freecappuccino_gb300.learned import DEFAULT_WEIGHTS, LearnedPreconditioner

    m = mesh_by_name(name)
    csr, a, su = _system(m, variable)
    ctx = fcg.Context(m)
    lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
    lp.set_matrix(ctx, a)
    return m, csr, a, su, ctx, lp


@pytest.mark.gpu
@pytest.mark.parametrize("name,smoothed", [("cavity", 1), ("pitzdaily", 1), ("hexmix8", 1),
                                           ("hex12", 1), ("pitzdaily", 0), ("hex12", 0)])
def test_hierarchy_matches_oracle(name, smoothed):
    m, csr, a, su, ctx, lp = _gpu(name)
    lp.set_multilevel(smoothed=bool(smoothed))
    info = lp.hierarchy(ctx)
    assert info["built_on"] == "device"
    fine = mo.scaled_csr(csr.ioffset, csr.ja, csr.diag, a)
    levels = mo.build_levels(*fine, sa_omega=0.67 if smoothed else 0.0)
    values = mo.level_values(levels, fine)
    assert info["cells"] == [m.numCells] + [lv["n"] for lv in levels]
    for l, (lv, v) in enumerate(zip(levels, values), start=1):
        g = lp.hierarchy_level(ctx, l)
        for k in ("agg", "mptr", "mem", "ptr", "col"):
            assert np.array_equal(g[k], lv[k]), (l, k)
        assert np.array_equal(g["val"], v), l  # FP32 sums in the same order
    ctx.close()
    lp.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name,smoothed", [("pitzdaily", 1), ("hex16", 1), ("hex16", 0)])
def test_correction_matches_oracle(name, smoothed):
    m, csr, a, su, ctx, lp = _gpu(name)
    lp.set_multilevel(smoothed=bool(smoothed))
    _, _, _, cyc = mo.hierarchy(csr.ioffset, csr.ja, csr.diag, a,
                                sa_omega=0.67 if smoothed else 0.0)
    rng = np.random.default_rng(1)
    r = rng.standard_normal(m.numCells).astype(np.float32)
    z = (0.5 * rng.standard_normal(m.numCells)).astype(np.float32)
    got = lp.coarse_correct(ctx, r, z)
    ref = cyc.correct(r.astype(np.float64), z.astype(np.float64))
    assert np.linalg.norm(got - ref) <= 2e-4 * np.linalg.norm(ref)
    lp.set_multilevel(smoother="jacobi")
    got_j = lp.precondition(ctx, r)
    ref_j = cyc.jacobi_cycle(r.astype(np.float64))
    assert np.linalg.norm(got_j - ref_j) <= 2e-4 * np.linalg.norm(ref_j)
    # the network smoother: M(r) is the correction of N(r), the same kernels
    lp.set_multilevel(smoother="network")
    zn = lp.apply(ctx, r)
    assert np.array_equal(lp.precondition(ctx, r), lp.coarse_correct(ctx, r, zn))
    ctx.close()
    lp.close()


class _host_build:
    """FCG_AGG=host while a hierarchy is built: aggregation.cpp instead of the device."""

    def __enter__(self):
        import os

        self.old = os.environ.get("FCG_AGG")
        os.environ["FCG_AGG"] = "host"

    def __exit__(self, *exc):
        import os

        if self.old is None:
            os.environ.pop("FCG_AGG", None)
        else:
            os.environ["FCG_AGG"] = self.old


def _levels(lp, ctx):
    info = lp.hierarchy(ctx)
    return info, [lp.hierarchy_level(ctx, l) for l in range(1, len(info["cells"]))]


@pytest.mark.gpu
@pytest.mark.parametrize("name,smoothed", [("hex32", 1), ("hex32", 0), ("pitzdaily", 1),
                                           ("hexmix8", 1), ("cavity", 0)])
def test_device_hierarchy_equals_host_hierarchy(name, smoothed):
    """The hierarchy built on the device (aggregation_gpu.cu) against the host build
    (aggregation.cpp) on the same matrix: every level's aggregates, members, pattern and
    FP32 values, and (through the smoothed prolongation's patterns) the correction and a
    whole learned solve, bit for bit."""
    from freecappuccino_gb300.learned import DEFAULT_WEIGHTS, LearnedPreconditioner

    m, csr, a, su, ctx, lp = _gpu(name)
    lp.set_multilevel(smoothed=bool(smoothed))
    info_d, lev_d = _levels(lp, ctx)
    rng = np.random.default_rng(2)
    r = rng.standard_normal(m.numCells).astype(np.float32)
    z = (0.5 * rng.standard_normal(m.numCells)).astype(np.float32)
    corr_d = lp.coarse_correct(ctx, r, z)
    x0 = np.zeros(m.numCells)
    sol_d = lp.solve(ctx, a, su, x0, 1e-8, 5000)
    lp.close()
    with _host_build():
        lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
        lp.set_matrix(ctx, a)
        lp.set_multilevel(smoothed=bool(smoothed))
        info_h, lev_h = _levels(lp, ctx)
    assert info_d["built_on"] == "device" and info_h["built_on"] == "host"
    assert info_d["cells"] == info_h["cells"] and info_d["entries"] == info_h["entries"]
    for l, (gd, gh) in enumerate(zip(lev_d, lev_h), start=1):
        for k in ("agg", "mptr", "mem", "ptr", "col", "val"):
            assert np.array_equal(gd[k], gh[k]), (name, l, k)
    assert np.array_equal(lp.coarse_correct(ctx, r, z), corr_d)
    sol_h = lp.solve(ctx, a, su, x0, 1e-8, 5000)
    assert sol_h.fcg_iters == sol_d.fcg_iters and np.array_equal(sol_h.fi, sol_d.fi)
    print(f"\n{name}: levels {info_d['cells']}, set-up device {info_d['setup_seconds']:.3f} s, "
          f"host {info_h['setup_seconds']:.3f} s")
    ctx.close()
    lp.close()


@pytest.mark.gpu
def test_device_hierarchy_in_order_form(monkeypatch, capfd):
    """The coarse levels' passes run in the in-order form (k_pm_cands, k_pm_seq), the fine
    level's in the chained form, and the in-order form's levels equal those of the
    chained form everywhere (FCG_AGG_SEQ=0) element for element."""
    from freecappuccino_gb300.learned import DEFAULT_WEIGHTS, LearnedPreconditioner

    m = mesh_by_name("hex32")
    csr, a, su = _system(m, True)
    ctx = fcg.Context(m)
    out = []
    for seq in ("1", "0"):
        monkeypatch.setenv("FCG_AGG_SEQ", seq)
        monkeypatch.setenv("FCG_AGG_TRACE", "1")
        capfd.readouterr()
        lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
        lp.set_matrix(ctx, a)
        out.append(_levels(lp, ctx))
        lp.close()
        err = capfd.readouterr().err
        in_order = [ln for ln in err.splitlines() if "decided in order" in ln]
        chained = [ln for ln in err.splitlines() if "by the blocking form" in ln]
        if seq == "1":
            # three passes on the fine matrix chained, every later pass in order
            assert len(chained) == 3 and len(in_order) >= 3, err
        else:
            assert not in_order and len(chained) >= 6, err
    (info_s, lev_s), (info_c, lev_c) = out
    assert info_s["built_on"] == "device" and info_c["built_on"] == "device"
    assert info_s["cells"] == info_c["cells"] and info_s["entries"] == info_c["entries"]
    for l, (gs, gc) in enumerate(zip(lev_s, lev_c), start=1):
        for k in ("agg", "mptr", "mem", "ptr", "col", "val"):
            assert np.array_equal(gs[k], gc[k]), (l, k)
    ctx.close()


@pytest.mark.gpu
def test_device_hierarchy_wait_runs_out_and_host_builds():
    """A matching row that never announces its decision (fcg_set_aggregation_wait_test):
    the waits that read it give up after their poll bound, the GPU build returns without
    hanging, the hierarchy is built on the host instead, and the next build runs on the
    device again with the same arrays."""
    from freecappuccino_gb300.learned import DEFAULT_WEIGHTS, LearnedPreconditioner

    m, csr, a, su, ctx, lp = _gpu("hex16")
    lp.close()
    ctx.set_aggregation_wait_test(polls=4096, absent_row=1)
    lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
    lp.set_matrix(ctx, a)
    info_h, lev_h = _levels(lp, ctx)
    lp.close()
    assert info_h["built_on"] == "host"
    ctx.set_aggregation_wait_test(0, 0)
    lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
    lp.set_matrix(ctx, a)
    info_d, lev_d = _levels(lp, ctx)
    assert info_d["built_on"] == "device" and info_d["cells"] == info_h["cells"]
    for l, (gd, gh) in enumerate(zip(lev_d, lev_h), start=1):
        for k in ("agg", "mptr", "mem", "ptr", "col", "val"):
            assert np.array_equal(gd[k], gh[k]), (l, k)
    r = lp.solve(ctx, a, su, np.zeros(m.numCells), 1e-8, 5000)
    assert r.converged and not r.fallback
    ctx.close()
    lp.close()


@pytest.mark.gpu
def test_device_hierarchy_equals_host_hierarchy_128():
    """The same at 128^3 (jittered, variable diffusivity): every level element for
    element, and the set-up times of both builds."""
    from freecappuccino_gb300.learned import DEFAULT_WEIGHTS, LearnedPreconditioner, pressure_system

    sysm = pressure_system(128, 0.2, 2029, variable=True)
    ctx = sysm.ctx
    out = []
    for host in (False, True):
        lp = LearnedPreconditioner(path=DEFAULT_WEIGHTS)
        if host:
            with _host_build():
                lp.set_matrix(ctx, sysm.a)
                out.append(_levels(lp, ctx))
        else:
            lp.set_matrix(ctx, sysm.a)
            out.append(_levels(lp, ctx))
        lp.close()
    (info_d, lev_d), (info_h, lev_h) = out
    assert info_d["built_on"] == "device" and info_h["built_on"] == "host"
    assert info_d["cells"] == info_h["cells"] and info_d["entries"] == info_h["entries"]
    for l, (gd, gh) in enumerate(zip(lev_d, lev_h), start=1):
        for k in ("agg", "mptr", "mem", "ptr", "col", "val"):
            assert np.array_equal(gd[k], gh[k]), (l, k)
    print(f"\n128^3: levels {info_d['cells']}, set-up device {info_d['setup_seconds']:.3f} s, "
          f"host {info_h['setup_seconds']:.3f} s")
    ctx.close()


@pytest.mark.gpu
def test_fcg_with_correction_converges_fast():
    """32^3 jittered, variable diffusivity: the correction cuts the FCG iterations several
    fold, the solution meets the reference's stop test and agrees with DPCG, and the
    trained network beats Jacobi sweeps in the same cycle (what the network gains over the
    method without it)."""
    m, csr, a, su, ctx, lp = _gpu("hex32")
    x0 = np.zeros(m.numCells)
    d = ctx.dpcg(a, su, x0, 1e-12, 20000)
    r = lp.solve(ctx, a, su, x0, 1e-8, 20000)
    assert r.converged and not r.fallback and r.resl / r.res0 < 1e-8 and r.l2_rel < 1e-7
    assert np.linalg.norm(r.fi - d.fi) <= 1e-6 * np.linalg.norm(d.fi)
    lp.set_multilevel(enabled=False)
    plain = lp.solve(ctx, a, su, x0, 1e-8, 20000)
    lp.set_multilevel(enabled=True, smoother="jacobi")
    jac = lp.solve(ctx, a, su, x0, 1e-8, 20000)
    lp.set_multilevel(smoother="network")
    again = lp.solve(ctx, a, su, x0, 1e-8, 20000)
    assert again.fcg_iters == r.fcg_iters and np.array_equal(again.fi, r.fi)
    assert jac.converged and plain.converged
    assert r.fcg_iters * 2 < plain.fcg_iters
    assert r.fcg_iters < jac.fcg_iters
    print(f"\n32^3: DPCG {d.iters} sweeps; FCG network {plain.fcg_iters}, network + coarse "
          f"{r.fcg_iters}, Jacobi + coarse {jac.fcg_iters}; levels "
          f"{lp.hierarchy(ctx)['cells']}")
    ctx.close()
    lp.close()


@pytest.mark.gpu
def test_fcg_with_correction_on_small_and_general_meshes():
    for name in ("cavity", "pitzdaily", "hexmix8"):
        m, csr, a, su, ctx, lp = _gpu(name)
        x0 = np.zeros(m.numCells)
        r = lp.solve(ctx, a, su, x0, 1e-8, 5000)
        assert r.converged and not r.fallback and r.l2_rel < 1e-6, name
        ctx.close()
        lp.close()


@pytest.mark.gpu
def test_multilevel_options():
    from freecappuccino_gb300.learned import LearnedPreconditioner

    lp = LearnedPreconditioner()
    d = lp.multilevel
    assert d == dict(enabled=1, smoother="network", sweeps=2, max_levels=10, dense_max=128,
                     alpha=1.8, omega=0.67, smoothed=1)
    for bad in (dict(sweeps=0), dict(sweeps=9), dict(max_levels=1), dict(max_levels=17),
                dict(dense_max=0), dict(dense_max=161), dict(alpha=0.0), dict(alpha=4.0),
                dict(omega=0.0), dict(omega=2.0)):
        with pytest.raises(fcg._lib.FcgError) as ei:
            lp.set_multilevel(**bad)
        assert ei.value.status == fcg._lib.FCG_ERR_ARG
    assert lp.multilevel == d
    # fewer levels: a deeper coarsest level without a dense inverse still converges
    m, csr, a, su, ctx, lp2 = _gpu("hex16")
    lp2.set_multilevel(max_levels=2, dense_max=8)
    assert len(lp2.hierarchy(ctx)["cells"]) == 2
    r = lp2.solve(ctx, a, su, np.zeros(m.numCells), 1e-8, 5000)
    assert r.converged and not r.fallback
    lp2.set_multilevel(enabled=False)
    with pytest.raises(fcg._lib.FcgError) as ei:
        lp2.hierarchy(ctx)
    assert ei.value.status == fcg._lib.FCG_ERR_STATE
    ctx.close()
    lp2.close()
    lp.close()


@pytest.mark.gpu
def test_cycle_loss_gradient_matches_oracle():
    """The loss through the whole preconditioner (network, then the correction) and its
    gradient against the oracle's network and cycle."""
    from oracle import learned_oracle as lo

    from freecappuccino_gb300.learned import LearnedPreconditioner, dpcg_pairs, pressure_system

    sysm = pressure_system(14, 0.2, 3, variable=True)
    io, ja, dg, _, _ = sysm.ctx.create_csr()
    A = lo.ScaledMatrix(io, ja, dg, sysm.a)
    _, _, _, cyc = mo.hierarchy(io, ja, dg, sysm.a)
    lp = LearnedPreconditioner(seed=1)
    rng = np.random.default_rng(5)
    w = lo.pack(rng.uniform(-1, 1, (lo.C, lo.F)) / np.sqrt(lo.F), rng.uniform(-0.2, 0.2, lo.C),
                [(rng.uniform(-1, 1, (lo.C, 2 * lo.C)) * 2.0 / np.sqrt(2 * lo.C),
                  rng.uniform(-0.2, 0.2, lo.C)) for _ in range(lo.L)],
                rng.uniform(-1, 1, lo.C) / np.sqrt(lo.C), 0.05).astype(np.float32)
    lp.weights = w
    lp.set_loss("cycle")
    lp.set_matrix(sysm.ctx, sysm.a)
    r, e = dpcg_pairs(sysm, [5])[0]
    loss, g = lp.loss_grad(sysm.ctx, r, e)
    feat = lo.features(sysm.mesh, sysm.scale)
    lr_, gr = lo.loss_grad(A, feat, r, e, w, emulate=True, kind="cycle", correct=cyc.correct)
    assert loss == pytest.approx(lr_, rel=5e-3)
    bounds = [0, lo.C * lo.F + lo.C] + [lo.C * lo.F + lo.C + (l + 1) * lo.LAYER
                                         for l in range(lo.L)] + [lo.P]
    for b0, b1 in zip(bounds[:-1], bounds[1:]):
        assert np.linalg.norm(g[b0:b1] - gr[b0:b1]) < 3e-2 * np.linalg.norm(gr[b0:b1]), (b0, b1)
    # the correction off: the cycle loss is refused
    lp.set_multilevel(enabled=False)
    with pytest.raises(fcg._lib.FcgError) as ei:
        lp.loss_grad(sysm.ctx, r, e)
    assert ei.value.status == fcg._lib.FCG_ERR_STATE
    lp.close()
    sysm.ctx.close()

