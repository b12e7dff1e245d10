"""The pressure step of calcp (calcp-multiple_correction_SIMPLE.f90:34-223) chained on
the GPU and on the oracle with the same inputs: assembly by facefluxmass, then per
pressure correction ipcorr = 1..npcor: p' = 0 and ICCG, nipgrad stages of bpres + Gauss
gradient, the Gauss-corrected gradient (:143), the mass-flux correction (:159-171), the
velocity and pressure correction (:184-189) and, between corrections, the
non-orthogonal corrector source from fluxmc (:193-206).

The p' matrix has no Dirichlet row (its right-hand side sums to zero), so p' is fixed
only up to a constant: the comparison uses what does not see that constant -- the
gradient, the fluxes, the corrected velocities and the pressure corrected relative to
pp(pRefCell).  The single steps are compared bit for bit."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from oracle import oracle
from tests.meshes import hex_mesh, oracle_csr, oracle_mesh, seeded_fields

URF, PREF, NIPGRAD = 0.3, 1, 2


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def calcp_gpu(c, m, f, npcor, sor=1e-8, nsw=2000):
    n, nt = m.numCells, m.numTotal
    a, su, flmass = c.facefluxmass(**f)
    u, v, w, p = f["u"], f["v"], f["w"], f["p"]
    dPdxi = f["dPdxi"]
    iters = []
    for ipcorr in range(1, npcor + 1):
        r = c.iccg(a, su, np.zeros(n), sor, nsw)
        iters.append(r.iters)
        pp = np.concatenate([r.fi, np.zeros(nt - n)])
        for istage in range(1, NIPGRAD + 1):
            pp = c.bpres(pp, dPdxi, istage)
            dPdxi = c.grad(pp, "gauss")
        dPdxi = c.grad(pp, "gauss_corrected", dphidxi=np.zeros((n, 3)))
        flmass = c.flux_correct(a, pp, flmass)
        u, v, w, p = c.correct_fields(dPdxi, f["apu"], f["apv"], f["apw"], pp, URF, PREF,
                                      u, v, w, p)
        if ipcorr != npcor:
            su, flmass = c.fluxmc(dPdxi, f["apu"], f["den"], flmass)
    return dict(pp=pp, dPdxi=dPdxi, flmass=flmass, u=u, v=v, w=w, p=p, iters=iters)


def calcp_oracle(m, f, npcor, sor=1e-8, nsw=2000):
    om, csr = oracle_mesh(m), oracle_csr(m)
    n, nt = m.numCells, m.numTotal
    a, su, flmass = oracle.facefluxmass(om, csr, *f.values())
    u, v, w, p = f["u"], f["v"], f["w"], f["p"]
    dPdxi = f["dPdxi"]
    iters = []
    for ipcorr in range(1, npcor + 1):
        r = oracle.iccg(csr, a, su, np.zeros(n), sor, nsw)
        iters.append(r.iters)
        pp = np.concatenate([r.fi, np.zeros(nt - n)])
        for istage in range(1, NIPGRAD + 1):
            pp = oracle.bpres(om, pp, dPdxi, istage)
            dPdxi = oracle.grad_gauss(om, pp, 1)
        dPdxi = oracle.grad_gauss(om, pp, 1, corrected=True, dphidxi_in=np.zeros((n, 3)))
        flmass = oracle.flux_correct(om, csr, a, pp, flmass)
        u, v, w, p = oracle.correct_fields(om, dPdxi, f["apu"], f["apv"], f["apw"], pp, URF,
                                           PREF, u, v, w, p)
        if ipcorr != npcor:
            su, flmass = oracle.fluxmc(om, dPdxi, f["apu"], f["den"], flmass)
    return dict(pp=pp, dPdxi=dPdxi, flmass=flmass, u=u, v=v, w=w, p=p, iters=iters)


@pytest.mark.gpu
@pytest.mark.parametrize("N,npcor", [(10, 2), (12, 3)])
def test_calcp_pressure_step_matches_oracle(N, npcor):
    m = hex_mesh(N, 0.2)
    c = fcg.Context(m)
    f = seeded_fields(m, seed=7)
    g = calcp_gpu(c, m, f, npcor)
    o = calcp_oracle(m, f, npcor)
    assert all(abs(i - j) <= 1 for i, j in zip(g["iters"], o["iters"]))
    n = m.numCells
    for k in ("dPdxi", "flmass", "u", "v", "w"):
        assert _rel(g[k], o[k]) < 1e-8, k
    dp_g = g["p"][:n] - f["p"][:n]
    dp_o = o["p"][:n] - f["p"][:n]
    assert _rel(dp_g, dp_o) < 1e-8
    c.close()


@pytest.mark.gpu
def test_flux_and_field_corrections_bit_exact():
    m = hex_mesh(9, 0.2)
    c = fcg.Context(m)
    om, csr = oracle_mesh(m), oracle_csr(m)
    f = seeded_fields(m, seed=11)
    a, _, flm = c.facefluxmass(**f)
    pp = fcg.uniform(3, 5, m.numTotal)
    assert np.array_equal(c.flux_correct(a, pp, flm), oracle.flux_correct(om, csr, a, pp, flm))
    got = c.correct_fields(f["dPdxi"], f["apu"], f["apv"], f["apw"], pp, 0.7, 5,
                           f["u"], f["v"], f["w"], f["p"])
    ref = oracle.correct_fields(om, f["dPdxi"], f["apu"], f["apv"], f["apw"], pp, 0.7, 5,
                                f["u"], f["v"], f["w"], f["p"])
    for x, y in zip(got, ref):
        assert np.array_equal(x, y)
    # boundary slots are left alone
    assert np.array_equal(got[0][m.numCells:], f["u"][m.numCells:])
    c.close()


def test_oracle_corrections_restate_the_loops():
    """The oracle's correction loops against a direct numpy statement of :159-171 and
    :184-189 (CPU)."""
    m = hex_mesh(5, 0.2)
    om, csr = oracle_mesh(m), oracle_csr(m)
    rng = np.random.default_rng(0)
    a = rng.standard_normal(csr.nnz)
    pp = rng.standard_normal(m.numTotal)
    flm = rng.standard_normal(m.numInnerFaces)
    P, N = m.owner[:m.numInnerFaces] - 1, m.neighbour - 1
    ref = flm + a[csr.slot_pn - 1] * (pp[N] - pp[P])
    assert np.array_equal(oracle.flux_correct(om, csr, a, pp, flm), ref)
    n = m.numCells
    g = rng.standard_normal((n, 3))
    ap = [rng.uniform(0.5, 1, n) for _ in range(3)]
    uvwp = [rng.standard_normal(m.numTotal) for _ in range(4)]
    u, v, w, p = oracle.correct_fields(om, g, *ap, pp, 0.3, 2, *uvwp)
    assert np.array_equal(u[:n], uvwp[0][:n] - g[:, 0] * m.vol * ap[0])
    assert np.array_equal(w[:n], uvwp[2][:n] - g[:, 2] * m.vol * ap[2])
    assert np.array_equal(p[:n], uvwp[3][:n] + 0.3 * (pp[:n] - pp[1]))


@pytest.mark.gpu
def test_boundary_velocity_and_continuity_errors_bit_exact():
    """correctBoundaryConditionsVelocity and continuityErrors.h on the pitzDaily mesh
    (inlet, outlet and walls) and a hex mesh (symmetry patches)."""
    from tests.meshes import fixture_mesh

    from tests.meshes import mixed_patch_mesh

    for m in (fixture_mesh("pitzdaily"), hex_mesh(8, 0.2), mixed_patch_mesh(8)):
        c = fcg.Context(m)
        om = oracle_mesh(m)
        f = seeded_fields(m, seed=5)
        got = c.correct_bc_velocity(f["den"], 0.75, f["u"], f["v"], f["w"])
        ref = oracle.correct_bc_velocity(om, f["den"], 0.75, f["u"], f["v"], f["w"])
        for x, y in zip(got, ref):
            assert np.array_equal(x, y)
        flm = fcg.uniform(9, 1, m.numInnerFaces)
        fmi = fcg.uniform(9, 2, m.counts.get("ninl", 0))
        res, sl, sg = c.continuity_errors(flm, fmi, got[3])
        res_o, sl_o, sg_o = oracle.continuity_errors(om, flm, fmi, ref[3])
        assert np.array_equal(res, res_o)
        assert sl == pytest.approx(sl_o, rel=1e-13) and sg == pytest.approx(sg_o, rel=1e-9, abs=1e-12)
        c.close()
