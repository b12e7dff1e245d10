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
