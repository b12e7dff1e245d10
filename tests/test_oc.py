"""O-C grid cuts and cyclic faces (noc > 0; mesh_geometry_and_topology.f90:453-462, 800-845,
1083-1163; fvm_laplacian.f90:67-86; dpcg.f90:58-61,113-116; iccg.f90:59-62,137-140;
bicgstab.f90:49-52).

The test mesh is an N^3 hex mesh cut into two blocks: the inner faces between two planes
become O-C pairs (tests/meshes.py oc_split_mesh).  The operator of the cut mesh, its CSR
values plus the pairs' ar and al, is then the operator of the uncut mesh up to the
rounding of the pairs' interpolation factor (from the face centres) against the inner
faces' (from the plane intersection), so both meshes give the same solution.

CPU: the oracle's pair geometry, operator and solvers.  GPU: fcg_laplacian bit for bit
against the oracle, fcg_dpcg / fcg_iccg / fcg_bicgstab and fcg_spmv against it (within
the solvers' usual 1e-10), the same solution as on the uncut mesh, and the entry points
that do not take the pairs refusing the mesh."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from oracle import oracle
from tests.meshes import oc_split_mesh, oracle_csr, oracle_mesh


def _fields(m, seed=5):
    mu = -(1.0 + 0.5 * fcg.uniform(seed, 5, m.numCells))
    su = fcg.uniform(seed, 7, m.numCells) * m.vol
    return mu, np.zeros(m.numTotal), su


def _operator(m, csr, a):
    """Dense operator of a (CSR values, then ar and al of the pairs)."""
    n = m.numCells
    A = np.zeros((n, n))
    for i in range(n):
        for k in range(csr.ioffset[i] - 1, csr.ioffset[i + 1] - 1):
            A[i, csr.ja[k] - 1] += a[k]
    if m.noc:
        ijl, ijr, _, _ = oracle.oc_geometry(oracle_mesh(m))
        ar, al = a[csr.nnz:csr.nnz + m.noc], a[csr.nnz + m.noc:]
        for i in range(m.noc):
            A[ijl[i] - 1, ijr[i] - 1] += ar[i]
            A[ijr[i] - 1, ijl[i] - 1] += al[i]
    return A


def _oc(m):
    ijl, ijr, _, _ = oracle.oc_geometry(oracle_mesh(m))
    return ijl, ijr


# ----------------------------------------------------------------------------- CPU
@pytest.mark.parametrize("cyclic", [False, True])
def test_oracle_pair_geometry(cyclic):
    """ijl / ijr are the owners of each pair's faces; foc is the cut faces' interpolation
    factor (1/2 for cyclic pairs) and srdoc |S| / (djn + dpn)."""
    N = 8
    m, u = oc_split_mesh(N, cyclic=cyclic), fcg.hex_mesh(N)
    ijl, ijr, foc, srdoc = oracle.oc_geometry(oracle_mesh(m))
    assert m.noc == N * N
    assert np.array_equal(ijl, m.owner[m.ijlFace - 1]) and np.array_equal(ijr, m.owner[m.ijrFace - 1])
    assert np.all(ijr - ijl == N * N)
    nin = u.numInnerFaces
    cut = ((u.owner[:nin] - 1) // (N * N) == N // 2 - 1) & ((u.neighbour - 1) // (N * N) == N // 2)
    if cyclic:
        assert np.all(foc == 0.5)
    else:
        assert np.abs(foc - u.facint[cut]).max() < 1e-13
    f = np.flatnonzero(cut)
    are = np.sqrt(u.arx[f] ** 2 + u.ary[f] ** 2 + u.arz[f] ** 2)
    assert np.allclose(srdoc, are * N, rtol=1e-12)


@pytest.mark.parametrize("N", [6, 8])
def test_oracle_laplacian_of_the_cut_mesh_is_the_uncut_operator(N):
    m, u = oc_split_mesh(N), fcg.hex_mesh(N)
    mu, phi, su = _fields(m)
    a, su_m = oracle.laplacian(oracle_mesh(m), oracle_csr(m), mu, phi, su)
    b, su_u = oracle.laplacian(oracle_mesh(u), oracle_csr(u), mu, np.zeros(u.numTotal), su)
    assert len(a) == m.nnz + 2 * m.noc
    assert np.array_equal(a[m.nnz:m.nnz + m.noc], a[m.nnz + m.noc:])  # al = ar (:218-219)
    A, B = _operator(m, oracle_csr(m), a), _operator(u, oracle_csr(u), b)
    assert np.abs(A - B).max() <= 1e-13 * np.abs(B).max()
    assert np.array_equal(su_m, su_u)


def test_oracle_solvers_take_the_pairs_where_the_reference_does():
    """dpcg and iccg solve the cut operator; all three start from its residual
    (res0 = sum |su - A fi| with the pairs); bicgstab's sweeps use the CSR part only."""
    m = oc_split_mesh(6)
    csr = oracle_csr(m)
    mu, phi, su = _fields(m)
    a, su = oracle.laplacian(oracle_mesh(m), csr, mu, phi, su)
    A = _operator(m, csr, a)
    fi0 = fcg.uniform(9, 0, m.numCells)
    r0 = np.abs(su - A @ fi0).sum()
    x = np.linalg.solve(A, su)
    for solve in (oracle.dpcg, oracle.iccg):
        r = solve(csr, a, su, fi0, 1e-13, 2000, oc=_oc(m))
        assert r.res0 == pytest.approx(r0, rel=1e-12)
        assert np.abs(r.fi - x).max() <= 1e-8 * np.abs(x).max()
    r = oracle.bicgstab(csr, a, su, fi0, 1e-13, 3, oc=_oc(m))
    assert r.res0 == pytest.approx(r0, rel=1e-12)
    # without the pairs the first residual differs (the pairs carry the cut's couplings)
    r_csr = oracle.bicgstab(csr, a[: m.nnz], su, fi0, 1e-13, 3)
    assert abs(r_csr.res0 - r0) > 1e-6 * r0


def test_oracle_dpcg_on_the_cut_mesh_gives_the_uncut_solution():
    N = 8
    m, u = oc_split_mesh(N), fcg.hex_mesh(N)
    mu, phi, su = _fields(m)
    a, su_m = oracle.laplacian(oracle_mesh(m), oracle_csr(m), mu, phi, su)
    b, su_u = oracle.laplacian(oracle_mesh(u), oracle_csr(u), mu, np.zeros(u.numTotal), su)
    x0 = np.zeros(m.numCells)
    rm = oracle.dpcg(oracle_csr(m), a, su_m, x0, 1e-12, 5000, oc=_oc(m))
    ru = oracle.dpcg(oracle_csr(u), b, su_u, x0, 1e-12, 5000)
    assert abs(rm.iters - ru.iters) <= 2
    assert np.abs(rm.fi - ru.fi).max() <= 1e-9 * np.abs(ru.fi).max()


def test_oracle_gauss_gradient_of_the_cut_mesh_is_the_uncut_one():
    """The pairs carry the cut faces' Gauss terms (grad_gauss.f90:60-67): the gradient of a
    field on the cut mesh is the uncut mesh's up to the rounding of foc; the O-C slots of
    bpres take the owner values (stage 1)."""
    N = 8
    m, u = oc_split_mesh(N), fcg.hex_mesh(N)
    phi_c = fcg.uniform(2, 1, m.numCells)
    pm = np.concatenate([phi_c, np.zeros(m.numTotal - m.numCells)])
    pu = np.concatenate([phi_c, np.zeros(u.numTotal - u.numCells)])
    # boundary values as bpres stage 1 gives them, on both meshes
    pm = oracle.bpres(oracle_mesh(m), pm, None, 1)
    pu = oracle.bpres(oracle_mesh(u), pu, None, 1)
    ocs = m.boundary_slot_start("prOutlet") + m.counts.get("npru", 0)
    assert np.array_equal(pm[ocs:ocs + m.noc], phi_c[m.owner[m.iOCFacesStart:m.iOCFacesStart + m.noc] - 1])
    for nigrad in (1, 2):
        gm = oracle.grad_gauss(oracle_mesh(m), pm, nigrad=nigrad)
        gu = oracle.grad_gauss(oracle_mesh(u), pu, nigrad=nigrad)
        assert np.abs(gm - gu).max() <= 1e-12 * np.abs(gu).max()


def _cell_fields(m, seed=3):
    """Flow fields from cell values only (boundary slots 0), so that the cut and the uncut
    mesh see the same fields."""
    n, nt = m.numCells, m.numTotal
    pad = lambda x: np.concatenate([x, np.zeros(nt - n)])
    f = {k: pad(fcg.uniform(seed, i, n)) for i, k in enumerate(("u", "v", "w", "p"), start=1)}
    for k, name in enumerate(("dUdxi", "dVdxi", "dWdxi", "dPdxi")):
        f[name] = fcg.uniform(seed, 10 + k, 3 * n).reshape(n, 3)
    for k, name in enumerate(("apu", "apv", "apw")):
        f[name] = 1.0 / m.vol * (1.0 + 0.1 * fcg.uniform(seed, 20 + k, n))
    f["den"] = pad(1.0 + 0.2 * fcg.uniform(seed, 30, n))
    return f


def test_oracle_face_fluxes_of_the_cut_mesh_are_the_uncut_ones():
    """calcp on the cut mesh (:34-100, 159-171, 193-215): the pairs' ar / al and fmoc are the
    cut inner faces' coefficients and fluxes, so the p' operator, its source and the mass
    fluxes are the uncut mesh's up to the rounding of foc."""
    N = 8
    m, u = oc_split_mesh(N), fcg.hex_mesh(N)
    fm_, fu_ = _cell_fields(m), _cell_fields(u)
    a, su_m, fl_m = oracle.facefluxmass(oracle_mesh(m), oracle_csr(m), *fm_.values())
    b, su_u, fl_u = oracle.facefluxmass(oracle_mesh(u), oracle_csr(u), *fu_.values())
    assert len(a) == m.nnz + 2 * m.noc and len(fl_m) == m.numInnerFaces + m.noc
    A, B = _operator(m, oracle_csr(m), a), _operator(u, oracle_csr(u), b)
    assert np.abs(A - B).max() <= 1e-12 * np.abs(B).max()
    assert np.abs(su_m - su_u).max() <= 1e-12 * np.abs(su_u).max()
    nin = u.numInnerFaces
    cut = ((u.owner[:nin] - 1) // (N * N) == N // 2 - 1) & ((u.neighbour - 1) // (N * N) == N // 2)
    keep = ~cut
    assert np.abs(fl_m[m.numInnerFaces:] - fl_u[cut]).max() <= 1e-12 * np.abs(fl_u).max()
    assert np.array_equal(fl_m[: m.numInnerFaces], fl_u[keep])
    # the non-orthogonal corrector and the flux correction follow the same faces
    su2_m, fl2_m = oracle.fluxmc(oracle_mesh(m), fm_["dPdxi"], fm_["apu"], fm_["den"], fl_m)
    su2_u, fl2_u = oracle.fluxmc(oracle_mesh(u), fu_["dPdxi"], fu_["apu"], fu_["den"], fl_u)
    assert np.abs(fl2_m[m.numInnerFaces:] - fl2_u[cut]).max() <= 1e-12 * np.abs(fl2_u).max()
    assert np.abs(su2_m - su2_u).max() <= 1e-12 * np.abs(su2_u).max()
    pp_m = np.concatenate([fcg.uniform(6, 1, m.numCells), np.zeros(m.numTotal - m.numCells)])
    pp_u = np.concatenate([pp_m[: m.numCells], np.zeros(u.numTotal - u.numCells)])
    fc_m = oracle.flux_correct(oracle_mesh(m), oracle_csr(m), a, pp_m, fl_m)
    fc_u = oracle.flux_correct(oracle_mesh(u), oracle_csr(u), b, pp_u, fl_u)
    assert np.abs(fc_m[m.numInnerFaces:] - fc_u[cut]).max() <= 1e-12 * np.abs(fc_u).max()


# ----------------------------------------------------------------------------- GPU
def _gpu(N=8, cyclic=False):
    m = oc_split_mesh(N, cyclic=cyclic)
    return m, fcg.Context(m)


@pytest.mark.gpu
@pytest.mark.parametrize("cyclic", [False, True])
def test_laplacian_with_pairs_bit_exact(cyclic):
    m, c = _gpu(8, cyclic)
    mu, _, su = _fields(m)
    phi = fcg.uniform(1, 6, m.numTotal)
    a, su_g = c.laplacian(mu, phi, su)
    a_o, su_o = oracle.laplacian(oracle_mesh(m), oracle_csr(m), mu, phi, su)
    assert len(a) == m.nnz + 2 * m.noc
    assert np.array_equal(a, a_o)
    assert np.array_equal(su_g, su_o)
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["dpcg", "iccg", "bicgstab"])
def test_solvers_with_pairs_against_the_oracle(method):
    """Fixed sweeps from a nonzero start: the solution and the residual norms within
    1e-10 of the oracle's (which applies the pairs where the reference does)."""
    m, c = _gpu(8)
    mu, phi, su = _fields(m)
    a, su = oracle.laplacian(oracle_mesh(m), oracle_csr(m), mu, phi, su)
    fi0 = fcg.uniform(9, 0, m.numCells)
    nsw = 12
    g = getattr(c, method)(a, su, fi0, 0.0, nsw)
    o = getattr(oracle, method)(oracle_csr(m), a, su, fi0, 0.0, nsw, oc=_oc(m))
    assert g.iters == o.iters == nsw
    assert g.res0 == pytest.approx(o.res0, rel=1e-12)
    assert g.resl == pytest.approx(o.resl, rel=1e-8)
    assert np.abs(g.fi - o.fi).max() <= 1e-10 * np.abs(o.fi).max()
    c.close()


@pytest.mark.gpu
def test_dpcg_on_the_cut_mesh_gives_the_uncut_solution_and_spmv():
    N = 16
    m, c = _gpu(N)
    u = fcg.hex_mesh(N)
    cu = fcg.Context(u)
    mu, phi, su = _fields(m)
    a, su_m = c.laplacian(mu, phi, su)
    b, su_u = cu.laplacian(mu, np.zeros(u.numTotal), su)
    x0 = np.zeros(m.numCells)
    rm = c.dpcg(a, su_m, x0, 1e-12, 20000)
    ru = cu.dpcg(b, su_u, x0, 1e-12, 20000)
    assert rm.converged and ru.converged and abs(rm.iters - ru.iters) <= 3
    assert np.abs(rm.fi - ru.fi).max() <= 1e-8 * np.abs(ru.fi).max()
    # y = A x with the pairs, against the operator of the oracle's restatement
    x = fcg.uniform(3, 1, m.numCells)
    y = c.spmv(a, x)
    A = _operator(m, oracle_csr(m), a)
    assert np.abs(y - A @ x).max() <= 1e-13 * np.abs(A @ x).max()
    c.close()
    cu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("cyclic", [False, True])
def test_gradients_and_bpres_with_pairs_bit_exact(cyclic):
    """Gauss (1 and 2 passes), corrected Gauss, least squares and both bpres stages on the
    cut mesh, bit for bit against the oracle."""
    m, c = _gpu(8, cyclic)
    om = oracle_mesh(m)
    phi = fcg.uniform(2, 1, m.numTotal)
    for nigrad in (1, 2):
        assert np.array_equal(c.grad(phi, "gauss", nigrad=nigrad),
                              oracle.grad_gauss(om, phi, nigrad=nigrad))
    g0 = fcg.uniform(2, 3, 3 * m.numCells).reshape(-1, 3)
    assert np.array_equal(c.grad(phi, "gauss_corrected", dphidxi=g0),
                          oracle.grad_gauss(om, phi, corrected=True, dphidxi_in=g0))
    d_o = oracle.grad_lsq_matrix(om)
    assert np.array_equal(c.grad_lsq_matrix(), d_o)
    assert np.array_equal(c.grad(phi, "lsq"), oracle.grad_lsq(om, phi, d_o))
    p = fcg.uniform(3, 1, m.numTotal)
    g = fcg.uniform(3, 2, 3 * m.numCells).reshape(-1, 3)
    for stage in (1, 2):
        assert np.array_equal(c.bpres(p, g, stage), oracle.bpres(om, p, g, stage))
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("cyclic", [False, True])
def test_calcp_face_fluxes_with_pairs_bit_exact(cyclic):
    """facefluxmass, fluxmc, the flux correction and the continuity errors on the cut mesh,
    bit for bit against the oracle (ar, al after the CSR values, fmoc after the inner
    faces' fluxes)."""
    from tests.meshes import seeded_fields

    m, c = _gpu(8, cyclic)
    om, csr = oracle_mesh(m), oracle_csr(m)
    f = seeded_fields(m)
    a, su, fm = c.facefluxmass(**f)
    a_o, su_o, fm_o = oracle.facefluxmass(om, csr, *f.values())
    assert len(fm) == m.numInnerFaces + m.noc
    assert np.array_equal(a, a_o) and np.array_equal(su, su_o) and np.array_equal(fm, fm_o)
    su2, fm2 = c.fluxmc(f["dPdxi"], f["apu"], f["den"], fm)
    su2_o, fm2_o = oracle.fluxmc(om, f["dPdxi"], f["apu"], f["den"], fm_o)
    assert np.array_equal(su2, su2_o) and np.array_equal(fm2, fm2_o)
    pp = fcg.uniform(6, 1, m.numTotal)
    assert np.array_equal(c.flux_correct(a, pp, fm2), oracle.flux_correct(om, csr, a_o, pp, fm2_o))
    r, sl, sg = c.continuity_errors(fm2, np.zeros(0), np.zeros(0))
    r_o, sl_o, sg_o = oracle.continuity_errors(om, fm2_o, np.zeros(0), np.zeros(0))
    assert np.array_equal(r, r_o)
    # the PISO corrector's assembly takes the pairs the same way (PISO :151-174)
    pf = {k: f[k] for k in ("u", "v", "w", "dUdxi", "dVdxi", "dWdxi", "apu", "den")}
    a3, su3, fm3 = c.facefluxmass_piso(**pf)
    a3_o, su3_o, fm3_o = oracle.facefluxmass_piso(om, csr, *pf.values())
    assert np.array_equal(a3, a3_o) and np.array_equal(su3, su3_o) and np.array_equal(fm3, fm3_o)
    c.close()


@pytest.mark.gpu
def test_entry_points_without_pairs_refuse_the_mesh():
    """The mixed and multi-RHS solvers, which have no reference counterpart, do not take
    the pairs: FCG_ERR_UNSUPPORTED (-8), the context still usable."""
    from freecappuccino_gb300._lib import FcgError

    m, c = _gpu(6)
    mu, phi, su = _fields(m)
    a, su = c.laplacian(mu, phi, su)
    with pytest.raises(FcgError) as e:
        c.dpcg_mixed(a, su, np.zeros(m.numCells), 1e-8, 100)
    assert e.value.status == -8
    with pytest.raises(FcgError) as e:
        c.bicgstab_multi(np.stack([a, a]), np.stack([su, su]), np.zeros((2, m.numCells)), 1e-8, 10)
    assert e.value.status == -8
    r = c.dpcg(a, su, np.zeros(m.numCells), 1e-10, 2000)
    assert r.converged
    c.close()


def test_polymesh_round_trip_keeps_the_pairs(tmp_path):
    """A cut mesh written as a polyMesh ('domain' patch pairs in the boundary file) and
    read back: the same pairs, and, with the geometry recomputed from the points, the same
    operator; a 'cyclic' pair of patches reads as cyclic pairs."""
    from freecappuccino_gb300.polymesh import read_polymesh, write_polymesh

    for cyclic in (False, True):
        m = oc_split_mesh(6, cyclic=cyclic)
        d = tmp_path / ("cyc" if cyclic else "oc")
        write_polymesh(m, str(d))
        r = read_polymesh(str(d))
        assert (r.noc, r.ncyc) == (m.noc, m.ncyc)
        assert np.array_equal(r.ijlFace, m.ijlFace) and np.array_equal(r.ijrFace, m.ijrFace)
        assert np.array_equal(r.owner, m.owner) and np.array_equal(r.neighbour, m.neighbour)
        # the reference sets iOCFacesStart from 'domain' patches only
        assert r.iOCFacesStart == (0 if cyclic else m.iOCFacesStart)
        if not cyclic:
            mu, phi, su = _fields(m)
            a, _ = oracle.laplacian(oracle_mesh(m), oracle_csr(m), mu, phi, su)
            b, _ = oracle.laplacian(oracle_mesh(r), oracle_csr(r), mu, phi, su)
            A, B = _operator(m, oracle_csr(m), a), _operator(r, oracle_csr(r), b)
            assert np.abs(A - B).max() <= 1e-12 * np.abs(A).max()


@pytest.mark.gpu
def test_cyclic_only_polymesh_binds_as_the_reference_reads_it(tmp_path):
    """A polyMesh whose only pairs are 'cyclic' keeps iOCFacesStart = 0, as the reference
    leaves it, so the pairs' areas come from faces 1..noc: the library binds it and its
    Laplacian and gradients are the oracle's bit for bit. Those inner faces lie across the
    pairs' direction, so ar and al come out infinite and the wall cells among the pairs' get
    NaN sources, in the oracle as in the library: NaN compares equal here."""
    from freecappuccino_gb300.polymesh import read_polymesh, write_polymesh

    write_polymesh(oc_split_mesh(6, cyclic=True), str(tmp_path))
    m = read_polymesh(str(tmp_path))
    assert m.noc == m.ncyc > 0 and m.iOCFacesStart == 0
    c = fcg.Context(m)
    mu, phi, su = _fields(m)
    a, su_g = c.laplacian(mu, phi, su)
    a_o, su_o = oracle.laplacian(oracle_mesh(m), oracle_csr(m), mu, phi, su)
    assert np.isinf(a_o).any() and np.isnan(su_o).any()
    assert np.array_equal(a, a_o) and np.array_equal(su_g, su_o, equal_nan=True)
    ph = fcg.uniform(2, 1, m.numTotal)
    assert np.array_equal(c.grad(ph, "gauss", nigrad=2),
                          oracle.grad_gauss(oracle_mesh(m), ph, nigrad=2))
    c.close()


def _uvw_fields(m, flmass, seed=5):
    """Momentum inputs from cell values (boundary slots 0) and the given face fluxes."""
    n, nt = m.numCells, m.numTotal
    pad = lambda x: np.concatenate([x, np.zeros(nt - n)])
    f = {k: pad(fcg.uniform(seed, i, n)) for i, k in enumerate(("u", "v", "w", "p"), start=1)}
    f["vis"] = pad(1e-3 * (1.0 + 0.5 * fcg.uniform(seed, 50, n, 0.0, 1.0)))
    f["den"] = 1.0 + 0.2 * fcg.uniform(seed, 30, n)
    for k, name in enumerate(("dUdxi", "dVdxi", "dWdxi", "dPdxi")):
        f[name] = fcg.uniform(seed, 10 + k, 3 * n).reshape(n, 3)
    for k, s in (("t", 54), ("uo", 55), ("vo", 56), ("wo", 57), ("uoo", 58), ("voo", 59),
                 ("woo", 60)):
        f[k] = fcg.uniform(seed, s, n) + (290.0 if k == "t" else 0.0)
    f["flmass"], f["fmi"], f["fmo"] = flmass, np.zeros(0), np.zeros(0)
    return f


def _uvw_oracle(m, kw, f, a):
    from tests.test_momentum import _oracle

    return _oracle(m, oracle_csr(m), kw, f, a)


def test_oracle_momentum_of_the_cut_mesh_is_the_uncut_one():
    """calcuvw's pairs (facefluxuvw_cyclic and presFaceDivInner, calcuvw.f90:186-215,
    fieldManipulation.f90:110-125) carry the cut faces' terms: on the unjittered cut mesh
    the momentum operators, diagonals, sources and ap are the uncut mesh's."""
    N = 6
    m, u = oc_split_mesh(N), fcg.hex_mesh(N)
    nin = u.numInnerFaces
    cut = ((u.owner[:nin] - 1) // (N * N) == N // 2 - 1) & ((u.neighbour - 1) // (N * N) == N // 2)
    fl = 0.05 * fcg.uniform(5, 51, nin)
    fu = _uvw_fields(u, fl)
    fm = _uvw_fields(m, np.concatenate([fl[~cut], fl[cut]]))
    for kw in (dict(scheme="central"), dict(scheme="muscl", bdf=True, timestep=0.01),
               dict(scheme="flux_limiter", limiter="smart")):
        am, dm, rm, pm = _uvw_oracle(m, kw, fm, np.zeros(m.nnz + 2 * m.noc))
        au, du, ru, pu = _uvw_oracle(u, kw, fu, np.zeros(u.nnz))
        A, B = _operator(m, oracle_csr(m), am), _operator(u, oracle_csr(u), au)
        assert np.abs(A - B).max() <= 1e-11 * np.abs(B).max(), kw
        for x, y in ((dm, du), (rm, ru), (pm, pu)):
            assert np.abs(x - y).max() <= 1e-11 * np.abs(y).max(), kw


@pytest.mark.gpu
@pytest.mark.parametrize("cyclic", [False, True])
def test_calcuvw_with_pairs_bit_exact(cyclic):
    """fcg_calcuvw on the cut mesh with every option set of the momentum tests, bit for bit
    against the oracle (ar, al after the CSR values; the pairs' fmoc after the inner
    faces' fluxes)."""
    from tests.test_momentum import OPTS

    m, c = _gpu(8, cyclic)
    f = _uvw_fields(m, 0.05 * fcg.uniform(5, 51, m.numInnerFaces + m.noc))
    a = fcg.uniform(5, 70, m.nnz + 2 * m.noc)
    keys = ("u", "v", "w", "p", "vis", "den", "dUdxi", "dVdxi", "dWdxi", "dPdxi", "flmass")
    for kw in OPTS:
        got = c.calcuvw(*[f[k] for k in keys], a, f["fmi"], f["fmo"], t=f["t"], uo=f["uo"],
                        vo=f["vo"], wo=f["wo"], uoo=f["uoo"], voo=f["voo"], woo=f["woo"], **kw)
        ref = _uvw_oracle(m, kw, f, a)
        for key, r in zip(("a", "diag_vw", "rhs", "ap"), ref):
            assert np.array_equal(got[key], r), (kw, key)
    c.close()
