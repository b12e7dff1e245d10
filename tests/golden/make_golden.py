"""Regenerates the golden fixtures in this folder from the freeCappuccino source tree.

Run once with the root of a freeCappuccino source tree (the folder that holds ``src/``,
``tests/`` and ``examples/``):

    python tests/golden/make_golden.py REFERENCE_ROOT

It writes
  * ``sparse_solvers.json``       -- the two 5x5 dense-as-CSR systems of
    tests/test_sparse_solvers.f90:596-655 (matrix, right-hand side and the CSR arrays,
    the numbers kept as the literal strings the Fortran source holds);
  * ``sparse_solvers_output.txt`` -- tests/output.txt, the reference's printed traces of
    those solves (BiCGStab, ICCG, DPCG);
  * ``cavity_mesh.npz`` / ``pitzdaily_mesh.npz`` -- the polyMesh of the cavity and
    pitzDaily examples (points, faces, owner, neighbour, boundary patches), 1-based
    indices as the Fortran reader stores them (mesh_geometry_and_topology.f90:778-797).

Nothing at test time reads the reference tree; the tests read these files.
"""
from __future__ import annotations

import io
import json
import os
import re
import sys
import tarfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _array_literal(src: str, start_marker: str, name: str):
    """Return the list of literal strings of the first ``name = (/ ... /)`` after a marker."""
    pos = src.index(start_marker)
    m = re.compile(rf"\b{name}\s*=\s*\(/(.*?)/\)", re.S).search(src, pos)
    body = m.group(1).replace("&", " ")
    return [t for t in re.split(r"[\s,]+", body) if t]


def sparse_solver_systems(ref: str):
    path = os.path.join(ref, "tests", "test_sparse_solvers.f90")
    src = open(path).read()
    t1 = "Test 1 - Real nonsymmetric 5x5 system.'"
    t2 = "Test 2 - symmetric positive definite 5x5 system.'"
    out = {
        "source": "tests/test_sparse_solvers.f90",
        "note": "literals are default REAL (float32) in the Fortran source, promoted to real(dp)",
        "ja": [int(t) for t in _array_literal(src, t1, "ja")],
        "ioffset": [int(t) for t in _array_literal(src, t1, "ioffset")],
        "diag": [int(t) for t in _array_literal(src, t1, "diag")],
        "test1": {"a": _array_literal(src, t1, "a"), "b": _array_literal(src, t1, "b"),
                  "xa": _array_literal(src, t1, "xa")},
        "test2": {"a": _array_literal(src, t2, "a"), "b": _array_literal(src, t2, "b"),
                  "xa": _array_literal(src, t2, "xa")},
    }
    with open(os.path.join(HERE, "sparse_solvers.json"), "w") as f:
        json.dump(out, f, indent=1)
    with open(os.path.join(ref, "tests", "output.txt")) as fi, \
            open(os.path.join(HERE, "sparse_solvers_output.txt"), "w") as fo:
        fo.write(fi.read())


def _foam_body(text: str):
    """Strip the FoamFile header; return the tokens between the outer parentheses."""
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"FoamFile\s*\{.*?\}", "", text, flags=re.S)
    return text.strip()


def read_polymesh(tf: tarfile.TarFile, prefix: str):
    def get(name):
        return tf.extractfile(prefix + name).read().decode()

    pts_txt = _foam_body(get("points"))
    n = int(pts_txt.split("(", 1)[0])
    pts = np.array(re.findall(r"\(([^()]*)\)", pts_txt.split("(", 1)[1]), dtype=object)
    xyz = np.array([[float(v) for v in p.split()] for p in pts], dtype=np.float64)
    assert xyz.shape == (n, 3)

    faces_txt = _foam_body(get("faces"))
    nf = int(faces_txt.split("(", 1)[0])
    face_ptr = [0]
    nodes = []
    for cnt, body in re.findall(r"(\d+)\(([^()]*)\)", faces_txt.split("(", 1)[1]):
        ids = [int(v) + 1 for v in body.split()]
        assert len(ids) == int(cnt)
        nodes.extend(ids)
        face_ptr.append(len(nodes))
    assert len(face_ptr) == nf + 1

    def labels(name):
        t = _foam_body(get(name))
        cnt = int(t.split("(", 1)[0])
        vals = np.array(t.split("(", 1)[1].rsplit(")", 1)[0].split(), dtype=np.int64) + 1
        assert len(vals) == cnt
        return vals.astype(np.int32)

    owner, neighbour = labels("owner"), labels("neighbour")
    note = re.search(r"nCells:\s*(\d+)", get("owner"))
    ncells = int(note.group(1))
    patches = []
    for line in get("boundary").splitlines():
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        t, cnt, start = line.split()
        patches.append((t, int(cnt), int(start)))
    return dict(points=xyz, face_ptr=np.array(face_ptr, np.int32), face_nodes=np.array(nodes, np.int32),
                owner=owner, neighbour=neighbour, numCells=ncells,
                patch_type=np.array([p[0] for p in patches]),
                patch_nfaces=np.array([p[1] for p in patches], np.int32),
                patch_start=np.array([p[2] for p in patches], np.int32))


def meshes(ref: str):
    for tar, prefix, out in (
        ("examples/cavity/cavity-setup.tar.gz", "polyMesh/", "cavity_mesh.npz"),
        ("examples/pitzDaily/pitzDaily-setup.tar.gz", "polyMesh/", "pitzdaily_mesh.npz"),
    ):
        with tarfile.open(os.path.join(ref, tar)) as tf:
            m = read_polymesh(tf, prefix)
        np.savez_compressed(os.path.join(HERE, out), **m)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_ROOT")
    ref = sys.argv[1]
    sparse_solver_systems(ref)
    meshes(ref)
    print("golden fixtures written to", HERE)
