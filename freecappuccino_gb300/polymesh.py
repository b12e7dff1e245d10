"""polyMesh files of the reference's cases (points, faces, owner, neighbour, boundary).

The reference reads an OpenFOAM-style polyMesh plus its own `boundary` file
(mesh_geometry_and_topology.f90:310-560): ASCII lists with a FoamFile header, faces as
`n(i j k ...)` with 0-based point labels, owner/neighbour as 0-based cell labels (the
cell count in the owner header note `nCells:`), and one `type nFaces startFace` line per
patch in the boundary file.  Indices are returned 1-based, as the reference holds them.
"""
from __future__ import annotations

import os
import re

import numpy as np

from .mesh import Mesh, polymesh_mesh


def _body(text: str) -> str:
    """The list part of a FOAM file: comments and the FoamFile header removed."""
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"FoamFile\s*\{.*?\}", "", text, flags=re.S)
    return text.strip()


_PARENS = str.maketrans("()", "  ")


def _split_list(text: str):
    """(count, the list's text after its opening parenthesis)."""
    t = _body(text)
    head, rest = t.split("(", 1)
    return int(head), rest


def _numbers(rest: str, dtype) -> np.ndarray:
    """Every number of the text, parentheses ignored, parsed in one C pass."""
    return np.fromstring(rest.translate(_PARENS), dtype=dtype, sep=" ")


def _tokens_per_group(rest: str, ngroups: int) -> np.ndarray:
    """The number of unsigned integers between each of the first `ngroups` "(" and the
    ")" that closes it; the groups must follow one another without nesting."""
    b = np.frombuffer(rest.encode("ascii"), dtype=np.uint8)
    op = np.flatnonzero(b == 40)
    cl = np.flatnonzero(b == 41)
    if len(op) != ngroups or len(cl) < ngroups or (
            ngroups and (np.any(op >= cl[:ngroups]) or np.any(cl[:ngroups - 1] >= op[1:]))):
        raise ValueError("faces: the parentheses of the face list do not pair up")
    dig = (b >= 48) & (b <= 57)
    starts = np.flatnonzero(dig[1:] & ~dig[:-1]) + 1  # first digit of every number
    if len(dig) and dig[0]:
        starts = np.concatenate(([0], starts))
    return np.searchsorted(starts, cl[:ngroups]) - np.searchsorted(starts, op)


def parse_points(text: str) -> np.ndarray:
    n, rest = _split_list(text)
    xyz = _numbers(rest, np.float64)
    if xyz.size != 3 * n or rest.count("(") != n:
        raise ValueError(f"points: expected {n} x 3 values, found {xyz.size} values")
    return xyz.reshape(n, 3)


def parse_faces(text: str):
    """(face_ptr, face_nodes), 1-based node labels."""
    nf, rest = _split_list(text)
    flat = _numbers(rest, np.int64)
    inside = _tokens_per_group(rest, nf)  # labels inside each face's parentheses
    c0 = int(flat[0]) if flat.size else 0
    if nf and flat.size == nf * (c0 + 1) and np.all(flat[::c0 + 1] == c0):
        counts = np.full(nf, c0, np.int64)  # every face has c0 nodes
        nodes = flat.reshape(nf, c0 + 1)[:, 1:].ravel()
    else:
        lst = flat.tolist()
        pos = np.zeros(nf, np.int64)
        at = 0
        for f in range(nf):
            if at >= len(lst):
                raise ValueError(f"faces: expected {nf} faces, the list ends early")
            pos[f] = at
            at += int(lst[at]) + 1
        if at != len(lst):
            raise ValueError("faces: the counts do not match the node lists")
        counts = flat[pos]
        keep = np.ones(flat.size, bool)
        keep[pos] = False
        nodes = flat[keep]
    if not np.array_equal(counts + 1, inside + 1) or np.any(counts < 1):
        raise ValueError("faces: a face lists a wrong number of nodes")
    ptr = np.zeros(nf + 1, np.int64)
    np.cumsum(counts, out=ptr[1:])
    return ptr.astype(np.int32), (nodes + 1).astype(np.int32)


def parse_labels(text: str) -> np.ndarray:
    """A label list as 1-based int32."""
    cnt, rest = _split_list(text)
    vals = _numbers(rest, np.int64) + 1
    if len(vals) != cnt:
        raise ValueError(f"labels: expected {cnt}, found {len(vals)}")
    return vals.astype(np.int32)


def parse_ncells(owner_text: str) -> int:
    m = re.search(r"nCells:\s*(\d+)", owner_text)
    if not m:
        raise ValueError("owner: the header note carries no nCells")
    return int(m.group(1))


def parse_boundary(text: str):
    """[(type, nFaces, startFace)] from the reference's boundary file."""
    out = []
    for line in text.splitlines():
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        t, cnt, start = line.split()
        out.append((t, int(cnt), int(start)))
    return out


def read_polymesh(path: str, device: int | None = None) -> Mesh:
    """The mesh of a polyMesh directory, with the reference's geometry and boundary
    bookkeeping (mesh.polymesh_mesh); with `device` set, the geometry is computed by the
    GPU kernels on that device."""
    def get(name):
        with open(os.path.join(path, name)) as f:
            return f.read()

    owner_text = get("owner")
    face_ptr, face_nodes = parse_faces(get("faces"))
    patches = parse_boundary(get("boundary"))
    return polymesh_mesh(parse_points(get("points")), face_ptr, face_nodes,
                         parse_labels(owner_text), parse_labels(get("neighbour")),
                         parse_ncells(owner_text), np.array([p[0] for p in patches]),
                         np.array([p[1] for p in patches], np.int32),
                         np.array([p[2] for p in patches], np.int32), device=device)


_HEADER = """FoamFile
{{
    version     2.0;
    format      ascii;
    class       {cls};
    note        "{note}";
    location    "constant/polyMesh";
    object      {obj};
}}
"""


def write_polymesh(m: Mesh, path: str):
    """Writes points, faces, owner, neighbour and boundary of a mesh that keeps its
    topology (hex_mesh(..., keep_topology=True) or read_polymesh)."""
    if m.points is None or m.face_ptr is None:
        raise ValueError("the mesh keeps no points/faces (build it with keep_topology=True)")
    os.makedirs(path, exist_ok=True)
    note = f"nPoints:{len(m.points)} nCells:{m.numCells} nFaces:{m.numFaces} " \
           f"nInternalFaces:{m.numInnerFaces}"

    def write(name, cls, lines):
        with open(os.path.join(path, name), "w") as f:
            f.write(_HEADER.format(cls=cls, note=note, obj=name))
            f.write(f"\n{len(lines)}\n(\n")
            f.write("\n".join(lines))
            f.write("\n)\n")

    write("points", "vectorField",
          ["(%r %r %r)" % (x, y, z) for x, y, z in np.asarray(m.points, np.float64).tolist()])
    fp = np.asarray(m.face_ptr, np.int64)
    fn = (np.asarray(m.face_nodes, np.int64) - 1).tolist()
    cnt = np.diff(fp)
    if len(cnt) and np.all(cnt == cnt[0]):  # one node count: fixed-width rows
        c = int(cnt[0])
        fmt = f"{c}(" + " ".join(["%d"] * c) + ")"
        rows = [fmt % tuple(fn[b:b + c]) for b in range(0, len(fn), c)]
    else:
        fpl = fp.tolist()
        rows = [f"{fpl[i + 1] - fpl[i]}(" + " ".join(map(str, fn[fpl[i]:fpl[i + 1]])) + ")"
                for i in range(len(fpl) - 1)]
    write("faces", "faceList", rows)
    write("owner", "labelList", list(map(str, (np.asarray(m.owner, np.int64) - 1).tolist())))
    write("neighbour", "labelList",
          list(map(str, (np.asarray(m.neighbour, np.int64) - 1).tolist())))
    names = {"nsym": "symmetry", "nwal": "wall", "ninl": "inlet", "nout": "outlet",
             "npru": "prOutlet"}
    start_key = {"nsym": "iSymmetryFacesStart", "nwal": "iWallFacesStart",
                 "ninl": "iInletFacesStart", "nout": "iOutletFacesStart",
                 "npru": "iPressOutletFacesStart"}
    rows = sorted((m.starts[start_key[k]], names[k], c) for k, c in m.counts.items() if c)
    with open(os.path.join(path, "boundary"), "w") as f:
        f.write("# type nFaces startFace\n")
        for st, t, c in rows:
            f.write(f"{t} {c} {st}\n")
        for t, st, st_friend, c in _pair_patches(m):
            f.write(f"{t} {c} {st}\n{t} {c} {st_friend}\n")


def _pair_patches(m: Mesh):
    """The O-C and cyclic pairs of a mesh as patch pairs (type, start, friend start, count):
    runs of pairs whose faces and friend faces are both consecutive."""
    if not getattr(m, "noc", 0):
        return []
    ijl = np.asarray(m.ijlFace, np.int64) - 1
    ijr = np.asarray(m.ijrFace, np.int64) - 1
    out, i = [], 0
    while i < m.noc:
        t = "domain" if i < m.noc - m.ncyc else "cyclic"
        j = i + 1
        while (j < m.noc and (j < m.noc - m.ncyc) == (i < m.noc - m.ncyc)
               and ijl[j] == ijl[j - 1] + 1 and ijr[j] == ijr[j - 1] + 1):
            j += 1
        out.append((t, int(ijl[i]), int(ijr[i]), j - i))
        i = j
    return out
