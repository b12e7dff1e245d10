"""polyMesh files (freecappuccino_gb300.polymesh): a jittered hex mesh written in the
reference's polyMesh layout and read back gives the same topology, boundary
bookkeeping and geometry, bit for bit (CPU)."""
import numpy as np
import pytest

import freecappuccino_gb300 as fcg
from freecappuccino_gb300.polymesh import parse_boundary, parse_faces, read_polymesh, write_polymesh


def test_write_read_round_trip(tmp_path):
    m = fcg.hex_mesh(5, jitter=0.2, seed=3, keep_topology=True)
    write_polymesh(m, str(tmp_path))
    r = read_polymesh(str(tmp_path))
    assert (r.numCells, r.numFaces, r.numInnerFaces) == (m.numCells, m.numFaces, m.numInnerFaces)
    assert {k: v for k, v in r.counts.items() if v} == {k: v for k, v in m.counts.items() if v}
    assert r.starts == m.starts
    for k in ("owner", "neighbour", "face_ptr", "face_nodes"):
        assert np.array_equal(getattr(r, k), getattr(m, k)), k
    for k in ("arx", "ary", "arz", "xf", "yf", "zf", "xc", "yc", "zc", "vol", "facint"):
        assert np.array_equal(getattr(r, k), getattr(m, k)), k


def test_parsers_reject_inconsistent_lists():
    with pytest.raises(ValueError):
        parse_faces("2\n(\n3(0 1 2)\n)\n")
    assert parse_boundary("# type nFaces startFace\nwall 4 10\nsymmetry 2 14\n") == \
        [("wall", 4, 10), ("symmetry", 2, 14)]


def test_faces_with_mixed_node_counts():
    ptr, nodes = parse_faces("3\n(\n3(0 1 2)\n4(1 2 3 4)\n5(0 1 2 3 4)\n)\n")
    assert ptr.tolist() == [0, 3, 7, 12]
    assert nodes.tolist() == [1, 2, 3, 2, 3, 4, 5, 1, 2, 3, 4, 5]
    # two errors that cancel in the flat count stream: caught by the per-face check
    with pytest.raises(ValueError):
        parse_faces("2\n(\n3(0 1 2 3)\n3(0 1)\n)\n")
    with pytest.raises(ValueError):  # a group left open
        parse_faces("2\n(\n3(0 1 2\n3(0 1 2)\n)\n")


def test_writer_round_trips_mixed_faces(tmp_path):
    """write_polymesh's face list with mixed node counts reads back unchanged."""
    import os
    from types import SimpleNamespace

    ptr = np.array([0, 3, 7, 12], np.int32)
    nodes = np.array([1, 2, 3, 2, 3, 4, 5, 1, 2, 3, 4, 5], np.int32)
    m = SimpleNamespace(points=np.random.default_rng(0).random((5, 3)), face_ptr=ptr,
                        face_nodes=nodes, owner=np.array([1, 1, 2], np.int32),
                        neighbour=np.array([2], np.int32), numCells=2, numFaces=3,
                        numInnerFaces=1, counts={"nwal": 2}, starts={"iWallFacesStart": 1})
    write_polymesh(m, str(tmp_path))
    with open(os.path.join(str(tmp_path), "faces")) as f:
        p2, n2 = parse_faces(f.read())
    assert np.array_equal(p2, ptr) and np.array_equal(n2, nodes)

