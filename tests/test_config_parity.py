"""GPU parity on the benchmark configurations themselves, at their full sizes.

- 64^3 uniform hex, unit diffusivity, DPCG: the plain-method case that also runs on a
  CPU.  FP64 DPCG after a fixed 25 sweeps within 1e-10 relative of the oracle
  (dpcg.f90:51-142), and the converged solve (L1 1e-8, at most 2000 sweeps) within one
  sweep of the oracle's count.
- 128^3 hex jittered by +-0.2 h: the CSR pattern and both face-to-slot maps
  (sparse_matrix.f90:42-172), laplacian, facefluxmass, fluxmc, the Gauss, corrected
  Gauss and least-squares gradients and both bpres stages bit-identical to the oracle;
  ICCG after a fixed 20 sweeps within 1e-10 (iccg.f90:77-166).
- the five transport systems (u, v, w, k, eps) on that 128^3 pattern: FP64 BiCGStab(DILU)
  after a fixed 10 sweeps within 1e-10 of the oracle's on every system
  (bicgstab.f90:99-224), and the one-launch multi-RHS solve to 1e-10 checked through the
  oracle's own FP64 product b - A x.

Each case holds well under 2 GB on the device."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from oracle import oracle
from tests.meshes import hex_mesh, oracle_csr, oracle_mesh, poisson_system, seeded_fields

pytestmark = pytest.mark.gpu

_cache = {}


def case(N, jitter):
    key = (N, jitter)
    if key not in _cache:
        _cache.clear()  # keep one large mesh alive at a time
        m = hex_mesh(N, jitter)
        _cache[key] = (m, fcg.Context(m), oracle_csr(m), oracle_mesh(m))
    return _cache[key]


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def poisson(m, c, csr, om):
    mu, phi, su = poisson_system(m)
    a, su_g = c.laplacian(mu, phi, su)
    a_o, su_o = oracle.laplacian(om, csr, mu, phi, su)
    assert np.array_equal(a, a_o) and np.array_equal(su_g, su_o)
    return a, su_g


# --- 64^3 uniform, DPCG --------------------------------------------------------------

def test_64_dpcg_fixed_sweeps_within_1e10():
    m, c, csr, om = case(64, 0.0)
    assert m.numCells == 262144
    a, su = poisson(m, c, csr, om)
    K = 25
    r = c.dpcg(a, su, np.zeros(m.numCells), 0.0, K)
    o = oracle.dpcg(csr, a, su, np.zeros(m.numCells), 0.0, K)
    assert r.iters == o.iters == K
    assert abs(r.res0 - o.res0) <= 1e-13 * o.res0
    assert rel(r.fi, o.fi) < 1e-10
    assert np.abs(r.res - o.res).max() < 1e-10 * np.abs(su).max()


def test_64_dpcg_converged_matches_oracle():
    m, c, csr, om = case(64, 0.0)
    a, su = poisson(m, c, csr, om)
    r = c.dpcg(a, su, np.zeros(m.numCells), 1e-8, 2000)
    o = oracle.dpcg(csr, a, su, np.zeros(m.numCells), 1e-8, 2000)
    assert r.converged and o.iters < 2000
    assert abs(r.iters - o.iters) <= 1
    assert r.resl / r.res0 < 1e-8
    # both stop on the same L1 test: their solutions differ by at most the tolerance
    assert rel(r.fi, o.fi) < (1e-10 if r.iters == o.iters else 1e-6)
    # the FP64 residual of the GPU solution, recomputed by the oracle
    res = su - oracle.spmv(csr, a, r.fi)
    assert np.abs(res).sum() / r.res0 < 1e-8


# --- 128^3 jittered: pattern and face-loop assembly -----------------------------------

def test_128_csr_and_slot_maps_bit_exact():
    m, c, csr, om = case(128, 0.2)
    assert m.numCells == 2097152 and len(csr.ja) == 14581760
    io, ja, dg, spn, snp = c.create_csr()
    for got, exp in ((io, csr.ioffset), (ja, csr.ja), (dg, csr.diag), (spn, csr.slot_pn),
                     (snp, csr.slot_np)):
        assert np.array_equal(got, exp)


def test_128_assembly_bit_exact():
    m, c, csr, om = case(128, 0.2)
    mu = -(1.0 + 0.5 * fcg.uniform(1, 5, m.numCells))
    phi = fcg.uniform(1, 6, m.numTotal)
    su = fcg.uniform(1, 7, m.numCells)
    a, su_g = c.laplacian(mu, phi, su)
    a_o, su_o = oracle.laplacian(om, csr, mu, phi, su)
    assert np.array_equal(a, a_o) and np.array_equal(su_g, su_o)
    f = seeded_fields(m)
    a, su, fm = c.facefluxmass(**f)
    a_o, su_o, fm_o = oracle.facefluxmass(om, csr, *f.values())
    assert np.array_equal(a, a_o) and np.array_equal(su, su_o) and np.array_equal(fm, fm_o)
    flm = fcg.uniform(4, 8, m.numInnerFaces)
    su, fm = c.fluxmc(f["dPdxi"], f["apu"], f["den"], flm)
    su_o, fm_o = oracle.fluxmc(om, f["dPdxi"], f["apu"], f["den"], flm)
    assert np.array_equal(su, su_o) and np.array_equal(fm, fm_o)


def test_128_gradients_and_bpres_bit_exact():
    m, c, csr, om = case(128, 0.2)
    phi = fcg.uniform(2, 1, m.numTotal)
    assert np.array_equal(c.grad(phi, "gauss", nigrad=2), oracle.grad_gauss(om, phi, nigrad=2))
    g0 = fcg.uniform(2, 3, 3 * m.numCells).reshape(-1, 3)
    assert np.array_equal(c.grad(phi, "gauss_corrected", dphidxi=g0),
                          oracle.grad_gauss(om, phi, corrected=True, dphidxi_in=g0))
    d = c.grad_lsq_matrix()
    d_o = oracle.grad_lsq_matrix(om)
    assert np.array_equal(d, d_o)
    assert np.array_equal(c.grad(phi, "lsq"), oracle.grad_lsq(om, phi, d_o))
    p = fcg.uniform(3, 1, m.numTotal)
    for stage in (1, 2):
        assert np.array_equal(c.bpres(p, g0, stage), oracle.bpres(om, p, g0, stage))


def test_128_iccg_fixed_sweeps_within_1e10():
    m, c, csr, om = case(128, 0.2)
    a, su = poisson(m, c, csr, om)
    K = 20
    r = c.iccg(a, su, np.zeros(m.numCells), 0.0, K)
    o = oracle.iccg(csr, a, su, np.zeros(m.numCells), 0.0, K)
    assert r.iters == o.iters == K
    assert abs(r.res0 - o.res0) <= 1e-13 * o.res0
    assert rel(r.fi, o.fi) < 1e-10
    assert np.abs(r.res - o.res).max() < 1e-10 * np.abs(su).max()


# --- the five transport systems on the 128^3 pattern ----------------------------------

def test_128_transport_systems_bicgstab():
    from freecappuccino_gb300.systems import transport_systems

    m, c, csr, om = case(128, 0.2)
    a, su, _ = transport_systems(m, (csr.ioffset, csr.ja, csr.diag, csr.slot_pn, csr.slot_np))
    K = 10
    for k in range(a.shape[0]):
        r = c.bicgstab(a[k], su[k], np.zeros(m.numCells), 0.0, K)
        o = oracle.bicgstab(csr, a[k], su[k], np.zeros(m.numCells), 0.0, K)
        assert r.iters == o.iters == K
        assert rel(r.fi, o.fi) < 1e-10, k
    x, reps = c.bicgstab_multi(a, su, np.zeros_like(su), 1e-10, 2000)
    for k in range(a.shape[0]):
        r_true = su[k] - oracle.spmv(csr, a[k], x[k])
        assert reps[k].converged
        assert np.abs(r_true).sum() / reps[k].res0 < 1e-10, k
        assert reps[k].l2_rel == pytest.approx(np.linalg.norm(r_true) / np.linalg.norm(su[k]),
                                               rel=1e-6, abs=1e-15)
