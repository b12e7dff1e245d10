"""Properties of the oracle on mesh problems (CPU): the assembled Laplacian is the SPD
operator the pressure path expects, the solvers reach the direct solution, and the
gradients are exact where the schemes are exact."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import oracle
from tests.meshes import hex_mesh, mesh_by_name, oracle_csr, oracle_mesh, poisson_system


def _matrix(csr, a):
    n = len(csr.diag)
    rows = np.repeat(np.arange(n), np.diff(csr.ioffset))
    return sp.csr_matrix((a, (rows, csr.ja - 1)), shape=(n, n))


@pytest.mark.parametrize("name", ["hex6", "cavity", "pitzdaily"])
def test_laplacian_is_spd_with_wall_dirichlet(name):
    m = mesh_by_name(name)
    om, csr = oracle_mesh(m), oracle_csr(m)
    mu, phi, su = poisson_system(m)
    a, su2 = oracle.laplacian(om, csr, mu, phi, su)
    A = _matrix(csr, a)
    assert abs(A - A.T).max() == 0.0  # cap == can bitwise
    assert np.all(A.diagonal() > 0)
    assert np.array_equal(su2, su)  # phi = 0 on the wall adds nothing
    if m.counts.get("nwal", 0):
        # rows of cells touching no wall sum to zero (pure diffusion)
        row_sums = np.asarray(A.sum(1)).ravel()
        wall_cells = set(m.owner[m.starts["iWallFacesStart"]:
                                 m.starts["iWallFacesStart"] + m.counts["nwal"]] - 1)
        interior = np.array([i for i in range(m.numCells) if i not in wall_cells])
        assert np.abs(row_sums[interior]).max() < 1e-10 * A.diagonal().max()


@pytest.mark.parametrize("kind", ["dpcg", "iccg", "bicgstab"])
def test_oracle_solvers_reach_direct_solution(kind):
    m = hex_mesh(6)
    om, csr = oracle_mesh(m), oracle_csr(m)
    mu, phi, su = poisson_system(m)
    a, su = oracle.laplacian(om, csr, mu, phi, su)
    x_direct = spla.spsolve(_matrix(csr, a).tocsc(), su)
    # BiCGStab's recursive residual stagnates near 1e-10 on this SPD system
    r = getattr(oracle, kind)(csr, a, su, np.zeros(m.numCells), 1e-10, 2000)
    assert 0 < r.iters < 2000 and r.resl / r.res0 < 1e-10
    assert np.abs(r.fi - x_direct).max() < 1e-8 * np.abs(x_direct).max()


def test_iccg_needs_fewer_sweeps_than_dpcg():
    m = hex_mesh(8)
    om, csr = oracle_mesh(m), oracle_csr(m)
    a, su = oracle.laplacian(om, csr, *poisson_system(m))
    d = oracle.dpcg(csr, a, su, np.zeros(m.numCells), 1e-8, 2000)
    i = oracle.iccg(csr, a, su, np.zeros(m.numCells), 1e-8, 2000)
    assert i.iters < d.iters


def test_early_exit_below_tol_keeps_resor():
    m = hex_mesh(4)
    om, csr = oracle_mesh(m), oracle_csr(m)
    a, su = oracle.laplacian(om, csr, *poisson_system(m))
    r = oracle.dpcg(csr, a, np.zeros(m.numCells), np.zeros(m.numCells), 1e-8, 100)
    assert r.iters == 0 and r.resor is None and r.res0 == 0.0  # dpcg.f90:66-70


def test_gradients_exact_for_linear_field():
    m = hex_mesh(6)
    om = oracle_mesh(m)
    gx, gy, gz = 0.3, -1.7, 2.5
    phi = np.concatenate([gx * m.xc + gy * m.yc + gz * m.zc, np.zeros(m.numTotal - m.numCells)])
    # boundary values: linear field at the face centres
    nb0 = m.numCells
    for t, cnt, st in (("symmetry", m.counts.get("nsym", 0), m.starts.get("iSymmetryFacesStart", 0)),
                       ("wall", m.counts.get("nwal", 0), m.starts.get("iWallFacesStart", 0))):
        s0 = m.boundary_slot_start(t)
        f = np.arange(st, st + cnt)
        phi[s0:s0 + cnt] = gx * m.xf[f] + gy * m.yf[f] + gz * m.zf[f]
    dmat = oracle.grad_lsq_matrix(om)
    g = oracle.grad_lsq(om, phi, dmat)
    # LSQ is exact for linear fields in x and z.  The reference's y row
    # (grad_lsq.f90:303) pairs b1 with the (2,2) cofactor and b2 with the (2,1) one, so
    # its y component is b1*C22 + b2*C21 + b3*C23; the oracle keeps that as written.
    assert np.abs(g[:, 0] - gx).max() < 1e-9 and np.abs(g[:, 2] - gz).max() < 1e-9
    assert np.abs(g[:, 1] - gy).max() > 1e-3
    # with the two coefficients put back in place, y is exact too
    D = dmat
    b = np.linalg.solve(np.stack([D[:, [0, 1, 2]] * [1, -1, 1], D[:, [3, 4, 5]] * [1, -1, -1],
                                  D[:, [6, 7, 8]] * [1, -1, 1]], 1), g[..., None])[..., 0]
    gy_fixed = -D[:, 4] * b[:, 0] + D[:, 3] * b[:, 1] - D[:, 5] * b[:, 2]
    assert np.abs(gy_fixed - gy).max() < 1e-8
    assert nb0 == m.numCells
    # Gauss: inconsistent on skewed cells; the iterative correction (nigrad) shrinks it
    e1 = np.abs(oracle.grad_gauss(om, phi, nigrad=1) - [gx, gy, gz]).mean()
    e3 = np.abs(oracle.grad_gauss(om, phi, nigrad=3) - [gx, gy, gz]).mean()
    assert e3 < e1


def test_bpres_stage1_copies_owner_values():
    m = mesh_by_name("pitzdaily")
    om = oracle_mesh(m)
    p = np.concatenate([np.arange(1.0, m.numCells + 1.0), np.zeros(m.numTotal - m.numCells)])
    p1 = oracle.bpres(om, p, None, 1)
    for t, key, stk in (("inlet", "ninl", "iInletFacesStart"), ("wall", "nwal", "iWallFacesStart"),
                        ("symmetry", "nsym", "iSymmetryFacesStart")):
        s0, cnt, st = m.boundary_slot_start(t), m.counts[key], m.starts[stk]
        assert np.array_equal(p1[s0:s0 + cnt], p[m.owner[st:st + cnt] - 1])
