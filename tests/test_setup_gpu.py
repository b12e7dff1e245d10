"""Mesh setup on the GPU: fcg_mesh_geometry_gpu and fcg_csr_build_gpu against the host
forms and the oracle (mesh_geometry_and_topology.f90:859-1079, sparse_matrix.f90:42-172),
bit for bit, plus the index errors they report."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from freecappuccino_gb300 import _lib
from freecappuccino_gb300.mesh import compute_geometry, compute_geometry_gpu, csr_build_gpu
from oracle import oracle
from tests.meshes import fixture_mesh, hex_mesh

pytestmark = pytest.mark.gpu

NAMES = ["cavity", "pitzdaily", "hex10", "hex7_u"]
KEYS = ("arx", "ary", "arz", "xf", "yf", "zf", "xc", "yc", "zc", "vol", "facint")


def _mesh(name):
    if name.startswith("hex"):
        uniform = name.endswith("_u")
        N = int(name[3:].split("_")[0])
        return hex_mesh(N, 0.0 if uniform else 0.2)
    return fixture_mesh(name)


def _host_csr(n, owner, neighbour):
    nin = len(neighbour)
    out = [np.zeros(n + 1, np.int32), np.zeros(n + 2 * nin, np.int32), np.zeros(n, np.int32),
           np.zeros(max(nin, 1), np.int32), np.zeros(max(nin, 1), np.int32)]
    rc = _lib.load().fcg_csr_build(n, nin, np.ascontiguousarray(owner, np.int32).ctypes.data,
                                   np.ascontiguousarray(neighbour, np.int32).ctypes.data,
                                   *[o.ctypes.data for o in out])
    assert rc == 0
    out[3], out[4] = out[3][:nin], out[4][:nin]
    return out


@pytest.mark.parametrize("name", NAMES)
def test_geometry_gpu_bit_exact(name):
    m = _mesh(name)
    args = (m.points, m.face_ptr, m.face_nodes, m.owner, m.neighbour, m.numCells)
    g = compute_geometry_gpu(*args)
    h = compute_geometry(*args)
    o = oracle.geometry(m.points[:, 0], m.points[:, 1], m.points[:, 2], m.numCells,
                        m.numInnerFaces, m.face_ptr, m.face_nodes, m.owner, m.neighbour)
    for k in KEYS:
        assert np.array_equal(g[k], h[k]), k
        assert np.array_equal(g[k], o[k]), k


@pytest.mark.parametrize("name", NAMES)
def test_csr_build_gpu_bit_exact(name):
    m = _mesh(name)
    nin = m.numInnerFaces
    g = csr_build_gpu(m.numCells, m.owner[:nin], m.neighbour)
    h = _host_csr(m.numCells, m.owner[:nin], m.neighbour)
    o = oracle.create_csr(m.numCells, m.owner[:nin], m.neighbour)
    for a, b, c in zip(g, h, (o.ioffset, o.ja, o.diag, o.slot_pn, o.slot_np)):
        assert np.array_equal(a, b) and np.array_equal(a, c)


def test_csr_build_gpu_any_face_order_and_device_arrays():
    """Faces in a shuffled order with owner and neighbour swapped on some: the pattern is
    the same canonical CSR and the slot maps follow the faces (sparse_matrix.f90:77,159-167)."""
    torch = pytest.importorskip("torch")
    m = hex_mesh(9, 0.2)
    nin = m.numInnerFaces
    rng = np.random.default_rng(3)
    perm = rng.permutation(nin)
    own, nb = m.owner[:nin][perm].copy(), m.neighbour[perm].copy()
    swap = rng.random(nin) < 0.3
    own[swap], nb[swap] = nb[swap], own[swap].copy()
    o = oracle.create_csr(m.numCells, own, nb)
    t_own = torch.from_numpy(own.astype(np.int32)).cuda()
    t_nb = torch.from_numpy(nb.astype(np.int32)).cuda()
    g = csr_build_gpu(m.numCells, t_own, t_nb)
    for a, c in zip(g, (o.ioffset, o.ja, o.diag, o.slot_pn, o.slot_np)):
        assert np.array_equal(a, c)


def test_setup_gpu_reports_bad_indices():
    m = hex_mesh(4, 0.0)
    nin = m.numInnerFaces
    own, nb = m.owner[:nin].copy(), m.neighbour.copy()
    dup_o, dup_n = np.append(own, own[0]), np.append(nb, nb[0])  # two faces on one cell pair
    for o_, n_ in ((dup_o, dup_n), (own, np.where(np.arange(nin) == 5, m.numCells + 1, nb)),
                   (own, np.where(np.arange(nin) == 2, own, nb))):
        with pytest.raises(_lib.FcgError) as ei:
            csr_build_gpu(m.numCells, o_, n_)
        assert ei.value.status == _lib.FCG_ERR_INDEX
    fp = m.face_ptr.copy()
    bad_nodes = m.face_nodes.copy()
    bad_nodes[7] = len(m.points) + 3
    short = fp.copy()
    short[1] = 2  # face 0 with two nodes
    for fp_, fn_ in ((fp, bad_nodes), (short, m.face_nodes)):
        with pytest.raises(_lib.FcgError) as ei:
            compute_geometry_gpu(m.points, fp_, fn_, m.owner, m.neighbour, m.numCells)
        assert ei.value.status == _lib.FCG_ERR_INDEX


def test_read_polymesh_on_device_matches_host(tmp_path):
    m = fixture_mesh("pitzdaily")
    fcg.write_polymesh(m, str(tmp_path))
    a = fcg.read_polymesh(str(tmp_path))
    b = fcg.read_polymesh(str(tmp_path), device=0)
    for k in KEYS:
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    c = fcg.hex_mesh(6, jitter=0.2, seed=4, device=0)
    d = fcg.hex_mesh(6, jitter=0.2, seed=4)
    for k in KEYS:
        assert np.array_equal(getattr(c, k), getattr(d, k)), k


def _shuffled(m, seed=5):
    """The same mesh with its inner faces in a shuffled order (boundary faces kept)."""
    nin = m.numInnerFaces
    perm = np.random.default_rng(seed).permutation(nin)
    full = np.concatenate([perm, np.arange(nin, m.numFaces)])
    face = {k: getattr(m, k)[full] for k in ("owner", "arx", "ary", "arz", "xf", "yf", "zf")}
    return fcg.Mesh(m.numCells, m.numFaces, nin, face["owner"].astype(np.int32),
                    m.neighbour[perm].astype(np.int32), face["arx"], face["ary"], face["arz"],
                    face["xf"], face["yf"], face["zf"], m.xc, m.yc, m.zc, m.vol,
                    m.facint[perm], counts=dict(m.counts), starts=dict(m.starts))


@pytest.mark.parametrize("name", ["cavity", "pitzdaily", "hexmix8", "hex10", "hex7_u",
                                  "hex9_shuffled"])
def test_bind_topology_gpu_equals_host(name):
    """fcg_bind_mesh builds its topology with GPU kernels; FCG_TOPOLOGY=host builds the
    same on the host.  Every bound array agrees (digest over all of them), and a solve
    that reads all of them (ICCG: levels, transpose positions, sliced ELL) agrees bit for
    bit."""
    import os

    from tests.meshes import mesh_by_name

    m = _shuffled(hex_mesh(9, 0.2)) if name == "hex9_shuffled" else (
        mesh_by_name(name) if name.startswith("hexmix") else _mesh(name))
    a = fcg.Context(m)
    old = os.environ.get("FCG_TOPOLOGY")
    os.environ["FCG_TOPOLOGY"] = "host"
    try:
        b = fcg.Context(m)
    finally:
        if old is None:
            os.environ.pop("FCG_TOPOLOGY", None)
        else:
            os.environ["FCG_TOPOLOGY"] = old
    assert a.topology_digest() == b.topology_digest()
    mu = -(1.0 + 0.5 * fcg.uniform(3, 1, m.numCells))
    phi, su = np.zeros(m.numTotal), fcg.uniform(3, 2, m.numCells)
    A, S = a.laplacian(mu, phi, su)
    r1 = a.bicgstab(A, S, np.zeros(m.numCells), 0.0, 20)
    r2 = b.bicgstab(A, S, np.zeros(m.numCells), 0.0, 20)
    assert np.array_equal(r1.fi, r2.fi)
    a.close()
    b.close()
