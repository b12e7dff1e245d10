"""Host-side parts of libfcgpu.so (no GPU needed): mesh generator, geometry and the
CSR construction, each checked bit for bit against the oracle."""
import ctypes as C

import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from freecappuccino_gb300 import _lib
from oracle import oracle
from tests.meshes import hex_mesh, mesh_by_name, oracle_csr

MESHES = ["hex6", "hex5_u", "cavity", "pitzdaily"]


@pytest.mark.parametrize("name", MESHES)
def test_geometry_bit_identical_to_oracle(name):
    m = mesh_by_name(name)
    g = oracle.geometry(m.points[:, 0], m.points[:, 1], m.points[:, 2], m.numCells,
                        m.numInnerFaces, m.face_ptr, m.face_nodes, m.owner, m.neighbour)
    for k, ref in g.items():
        assert np.array_equal(getattr(m, k), ref), k


def _csr_build(m):
    lib = _lib.load()
    n, nin = m.numCells, m.numInnerFaces
    io, ja, dg = np.zeros(n + 1, np.int32), np.zeros(m.nnz, np.int32), np.zeros(n, np.int32)
    spn, snp = np.zeros(nin, np.int32), np.zeros(nin, np.int32)
    rc = lib.fcg_csr_build(n, nin, m.owner.ctypes.data, m.neighbour.ctypes.data, io.ctypes.data,
                           ja.ctypes.data, dg.ctypes.data, spn.ctypes.data, snp.ctypes.data)
    assert rc == 0
    return io, ja, dg, spn, snp


@pytest.mark.parametrize("name", MESHES)
def test_csr_bit_exact_with_reference_construction(name):
    m = mesh_by_name(name)
    ref = oracle_csr(m)
    io, ja, dg, spn, snp = _csr_build(m)
    assert np.array_equal(io, ref.ioffset)
    assert np.array_equal(ja, ref.ja)
    assert np.array_equal(dg, ref.diag)
    assert np.array_equal(spn, ref.slot_pn)
    assert np.array_equal(snp, ref.slot_np)


def test_csr_properties_hex():
    m = hex_mesh(5)
    io, ja, dg, spn, snp = _csr_build(m)
    n = m.numCells
    assert io[0] == 1 and io[-1] == m.nnz + 1  # sparse_matrix.f90:97-104
    assert m.nnz == n + 2 * m.numInnerFaces     # mesh_geometry_and_topology.f90:580
    rows = np.repeat(np.arange(1, n + 1), np.diff(io))
    assert np.all(ja[dg - 1] == np.arange(1, n + 1))
    assert np.all(np.diff(ja)[np.diff(rows) == 0] > 0)  # strictly ascending columns per row
    assert np.all(rows[spn - 1] == m.owner[: m.numInnerFaces]) and np.all(ja[spn - 1] == m.neighbour)
    assert np.all(rows[snp - 1] == m.neighbour) and np.all(ja[snp - 1] == m.owner[: m.numInnerFaces])


def test_csr_rejects_bad_indices():
    lib = _lib.load()
    owner = np.array([1, 2], np.int32)
    bad = np.array([2, 9], np.int32)  # cell 9 does not exist
    out = [np.zeros(16, np.int32) for _ in range(5)]
    rc = lib.fcg_csr_build(3, 2, owner.ctypes.data, bad.ctypes.data, *[o.ctypes.data for o in out])
    assert rc == _lib.FCG_ERR_INDEX
    dup = np.array([2, 2], np.int32)  # two faces between cells 1-2 ... and 2-2
    rc = lib.fcg_csr_build(3, 2, owner.ctypes.data, dup.ctypes.data, *[o.ctypes.data for o in out])
    assert rc == _lib.FCG_ERR_INDEX


@pytest.mark.parametrize("N,n,nin,nb,nnz", [
    (32, 32768, 95232, 6144, 223232),
    (64, 262144, 774144, 24576, 1810432),
    (128, 2097152, 6242304, 98304, 14581760),
    (256, 16777216, 50135040, 393216, 117047296),
])
def test_hex_sizes_table(N, n, nin, nb, nnz):
    lib = _lib.load()
    a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    assert lib.fcg_hex_mesh_sizes(N, C.byref(a), C.byref(b), C.byref(c), C.byref(d)) == 0
    assert (b.value, d.value, c.value - d.value, b.value + 2 * d.value) == (n, nin, nb, nnz)


def test_hex_mesh_is_valid():
    m = hex_mesh(6)
    assert np.isclose(m.vol.sum(), 1.0, rtol=0, atol=1e-13)
    assert np.all(m.vol > 0)
    assert np.all(m.owner[: m.numInnerFaces] < m.neighbour)  # upper-triangular face order
    # area vectors point from owner to neighbour
    d = np.stack([m.xc[m.neighbour - 1] - m.xc[m.owner[: m.numInnerFaces] - 1],
                  m.yc[m.neighbour - 1] - m.yc[m.owner[: m.numInnerFaces] - 1],
                  m.zc[m.neighbour - 1] - m.zc[m.owner[: m.numInnerFaces] - 1]], 1)
    s = np.stack([m.arx, m.ary, m.arz], 1)[: m.numInnerFaces]
    assert np.all((d * s).sum(1) > 0)
    # closed cells: sum of outward area vectors is zero
    acc = np.zeros((m.numCells, 3))
    sa = np.stack([m.arx, m.ary, m.arz], 1)
    np.add.at(acc, m.owner - 1, sa)
    np.add.at(acc, m.neighbour - 1, -sa[: m.numInnerFaces])
    assert np.abs(acc).max() < 1e-15


def test_uniform_generator_is_deterministic():
    a = fcg.uniform(5, 9, 1000)
    b = fcg.uniform(5, 9, 1000)
    c = fcg.uniform(5, 10, 1000)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() >= -1 and a.max() < 1 and abs(a.mean()) < 0.1
