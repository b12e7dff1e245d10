"""Meshes for the pressure-correction path: the arrays of the reference's module
``geometry`` (src/mesh_geometry_and_topology.f90:12-98).

Two sources:
  * ``hex_mesh(N, jitter, seed)`` -- the N^3 jittered hex mesh of the unit cube made
    by libfcgpu.so (host code, every thread), with its geometry computed the way
    ``mesh_geometry`` computes it;
  * ``polymesh_mesh(points, face_ptr, face_nodes, owner, neighbour, patches)`` -- a mesh
    read from polyMesh files (the test fixtures), with the boundary patches mapped to
    the reference's boundary types as mesh_geometry_and_topology.f90:409-472 does.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib

BOUNDARY_TYPES = ("inlet", "outlet", "symmetry", "wall", "prOutlet")
_WALL_ALIASES = ("wall", "wallIsoth", "wallAdiab", "wallQFlux")


@dataclass
class Mesh:
    numCells: int
    numFaces: int
    numInnerFaces: int
    owner: np.ndarray
    neighbour: np.ndarray
    arx: np.ndarray
    ary: np.ndarray
    arz: np.ndarray
    xf: np.ndarray
    yf: np.ndarray
    zf: np.ndarray
    xc: np.ndarray
    yc: np.ndarray
    zc: np.ndarray
    vol: np.ndarray
    facint: np.ndarray
    counts: dict = field(default_factory=dict)  # ninl, nout, nsym, nwal, npru
    starts: dict = field(default_factory=dict)  # i*FacesStart (0-based)
    points: np.ndarray | None = None
    face_ptr: np.ndarray | None = None
    face_nodes: np.ndarray | None = None
    # O-C grid cut and cyclic pairs (mesh_geometry_and_topology.f90:453-462, 800-845):
    # pair i joins the owners of boundary faces ijlFace[i] and ijrFace[i] (1-based); the
    # last ncyc pairs are cyclic; the O-C loops take pair i's area from face
    # iOCFacesStart + i (0-based start, i 1-based)
    noc: int = 0
    ncyc: int = 0
    iOCFacesStart: int = 0
    ijlFace: np.ndarray | None = None
    ijrFace: np.ndarray | None = None

    @property
    def numTotal(self) -> int:
        return self.numCells + self.numFaces - self.numInnerFaces

    @property
    def nnz(self) -> int:
        return self.numCells + 2 * self.numInnerFaces

    @property
    def a_len(self) -> int:
        """Values of a matrix on this mesh: the CSR values, then ar and al of the O-C pairs."""
        return self.nnz + 2 * self.noc

    def boundary_slot_start(self, btype: str) -> int:
        """0-based offset of a boundary type's slots in a numTotal field (:593-605)."""
        off = self.numCells
        for t, key in zip(BOUNDARY_TYPES, ("ninl", "nout", "nsym", "nwal", "npru")):
            if t == btype:
                return off
            off += self.counts.get(key, 0)
        raise KeyError(btype)

    def desc(self) -> _lib.MeshDesc:
        d = _lib.MeshDesc()
        d.numCells, d.numFaces, d.numInnerFaces = self.numCells, self.numFaces, self.numInnerFaces
        for k in ("ninl", "nout", "nsym", "nwal", "npru"):
            setattr(d, k, int(self.counts.get(k, 0)))
        for k in ("iInletFacesStart", "iOutletFacesStart", "iSymmetryFacesStart",
                  "iWallFacesStart", "iPressOutletFacesStart"):
            setattr(d, k, int(self.starts.get(k, 0)))
        d.noc, d.ncyc, d.iOCFacesStart = int(self.noc), int(self.ncyc), int(self.iOCFacesStart)
        for k in ("owner", "neighbour", "arx", "ary", "arz", "xf", "yf", "zf", "xc", "yc", "zc",
                  "vol", "facint"):
            setattr(d, k, getattr(self, k).ctypes.data)
        if self.noc:
            self.ijlFace = np.ascontiguousarray(self.ijlFace, dtype=np.int32)
            self.ijrFace = np.ascontiguousarray(self.ijrFace, dtype=np.int32)
            d.ijlFace, d.ijrFace = self.ijlFace.ctypes.data, self.ijrFace.ctypes.data
        return d

    def oracle_kwargs(self) -> dict:
        """Keyword arguments for the oracle's mesh wrapper (tests only)."""
        kw = {k: getattr(self, k) for k in ("numCells", "numFaces", "numInnerFaces", "owner",
                                             "neighbour", "arx", "ary", "arz", "xf", "yf", "zf",
                                             "xc", "yc", "zc", "vol", "facint")}
        kw.update(self.counts)
        kw.update(self.starts)
        if self.noc:
            kw.update(noc=self.noc, ncyc=self.ncyc, iOCFacesStart=self.iOCFacesStart,
                      ijlFace=self.ijlFace, ijrFace=self.ijrFace)
        return kw


def _p(a):
    return a.ctypes.data


def compute_geometry(points, face_ptr, face_nodes, owner, neighbour, numCells):
    """mesh_geometry's geometric part (:859-1079), run by libfcgpu.so on the host."""
    lib = _lib.load()
    x, y, z = (np.ascontiguousarray(points[:, i], dtype=np.float64) for i in range(3))
    face_ptr = np.ascontiguousarray(face_ptr, dtype=np.int32)
    face_nodes = np.ascontiguousarray(face_nodes, dtype=np.int32)
    owner = np.ascontiguousarray(owner, dtype=np.int32)
    neighbour = np.ascontiguousarray(neighbour, dtype=np.int32)
    nf, nin = len(face_ptr) - 1, len(neighbour)
    g = {k: np.zeros(nf) for k in ("arx", "ary", "arz", "xf", "yf", "zf")}
    g.update({k: np.zeros(numCells) for k in ("xc", "yc", "zc", "vol")})
    g["facint"] = np.zeros(max(nin, 1))
    rc = lib.fcg_mesh_geometry(len(x), _p(x), _p(y), _p(z), numCells, nf, nin, _p(face_ptr),
                               _p(face_nodes), _p(owner), _p(neighbour if nin else g["facint"]),
                               *[_p(g[k]) for k in ("arx", "ary", "arz", "xf", "yf", "zf", "xc",
                                                    "yc", "zc", "vol", "facint")])
    if rc != 0:
        raise _lib.FcgError(rc, "fcg_mesh_geometry")
    g["facint"] = g["facint"][:nin]
    return g


class _Device:
    """A libfcgpu context that is not bound to a mesh: the device and stream the setup
    kernels (fcg_mesh_geometry_gpu, fcg_csr_build_gpu) run on."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        self.h = C.c_void_p()
        rc = self.lib.fcg_create(C.byref(self.h), int(device))
        if rc != 0:
            raise _lib.FcgError(rc, "fcg_create", "no usable sm_103a CUDA device")

    def check(self, rc, what):
        if rc != 0:
            raise _lib.FcgError(rc, what, self.lib.fcg_last_error(self.h).decode())

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.lib.fcg_destroy(self.h)
        self.h = None


def _ptr(x):
    if hasattr(x, "data_ptr"):  # a CUDA tensor, used in place
        return x.data_ptr()
    return x.ctypes.data


def compute_geometry_gpu(points, face_ptr, face_nodes, owner, neighbour, numCells,
                         device: int = 0):
    """mesh_geometry's geometric part (:859-1079) by the GPU kernels of
    fcg_mesh_geometry_gpu; the same results as compute_geometry, bit for bit."""
    x, y, z = (np.ascontiguousarray(points[:, i], dtype=np.float64) for i in range(3))
    face_ptr = np.ascontiguousarray(face_ptr, dtype=np.int32)
    face_nodes = np.ascontiguousarray(face_nodes, dtype=np.int32)
    owner = np.ascontiguousarray(owner, dtype=np.int32)
    neighbour = np.ascontiguousarray(neighbour, dtype=np.int32)
    nf, nin = len(face_ptr) - 1, len(neighbour)
    g = {k: np.zeros(nf) for k in ("arx", "ary", "arz", "xf", "yf", "zf")}
    g.update({k: np.zeros(numCells) for k in ("xc", "yc", "zc", "vol")})
    g["facint"] = np.zeros(max(nin, 1))
    with _Device(device) as d:
        d.check(d.lib.fcg_mesh_geometry_gpu(
            d.h, len(x), _p(x), _p(y), _p(z), int(numCells), nf, nin, _p(face_ptr),
            _p(face_nodes), _p(owner), _p(neighbour if nin else g["facint"]),
            *[_p(g[k]) for k in ("arx", "ary", "arz", "xf", "yf", "zf", "xc", "yc", "zc", "vol",
                                 "facint")]), "fcg_mesh_geometry_gpu")
    g["facint"] = g["facint"][:nin]
    return g


def csr_build_gpu(numCells: int, owner, neighbour, device: int = 0):
    """create_CSR_matrix_from_mesh_data (sparse_matrix.f90:42-172) by the GPU kernels of
    fcg_csr_build_gpu: (ioffset, ja, diag, slot_pn, slot_np), 1-based int32.  owner and
    neighbour may be numpy arrays or CUDA int32 tensors; the results come back as numpy."""
    nin = len(neighbour)
    if not hasattr(owner, "data_ptr"):
        owner = np.ascontiguousarray(owner, dtype=np.int32)
        neighbour = np.ascontiguousarray(neighbour, dtype=np.int32)
    nnz = numCells + 2 * nin
    io, ja = np.zeros(numCells + 1, np.int32), np.zeros(nnz, np.int32)
    dg = np.zeros(numCells, np.int32)
    spn, snp = np.zeros(max(nin, 1), np.int32), np.zeros(max(nin, 1), np.int32)
    with _Device(device) as d:
        d.check(d.lib.fcg_csr_build_gpu(d.h, int(numCells), nin, _ptr(owner), _ptr(neighbour),
                                        _p(io), _p(ja), _p(dg), _p(spn), _p(snp)),
                "fcg_csr_build_gpu")
    return io, ja, dg, spn[:nin], snp[:nin]


def hex_mesh(N: int, jitter: float = 0.0, seed: int = 0, keep_topology: bool = False,
             device: int | None = None) -> Mesh:
    """N^3 hex mesh of the unit cube: wall at x=0, symmetry on the other five faces.
    With `device` set, the geometry is computed by the GPU kernels on that device."""
    lib = _lib.load()
    nn, nc, nf, nin = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    rc = lib.fcg_hex_mesh_sizes(N, C.byref(nn), C.byref(nc), C.byref(nf), C.byref(nin))
    if rc != 0:
        raise _lib.FcgError(rc, "fcg_hex_mesh_sizes")
    nn, nc, nf, nin = nn.value, nc.value, nf.value, nin.value
    pts = np.zeros((3, nn))
    face_ptr = np.zeros(nf + 1, np.int32)
    face_nodes = np.zeros(4 * nf, np.int32)
    owner = np.zeros(nf, np.int32)
    neighbour = np.zeros(max(nin, 1), np.int32)
    patches = np.zeros(4, np.int32)
    rc = lib.fcg_hex_mesh_build(N, float(jitter), int(seed), _p(pts[0]), _p(pts[1]), _p(pts[2]),
                                _p(face_ptr), _p(face_nodes), _p(owner), _p(neighbour),
                                _p(patches))
    if rc != 0:
        raise _lib.FcgError(rc, "fcg_hex_mesh_build")
    neighbour = neighbour[:nin]
    points = np.ascontiguousarray(pts.T)
    if device is None:
        g = compute_geometry(points, face_ptr, face_nodes, owner, neighbour, nc)
    else:
        g = compute_geometry_gpu(points, face_ptr, face_nodes, owner, neighbour, nc, device)
    m = Mesh(nc, nf, nin, owner, neighbour, **g,
             counts=dict(nsym=int(patches[0]), nwal=int(patches[2])),
             starts=dict(iSymmetryFacesStart=int(patches[1]), iWallFacesStart=int(patches[3])))
    if keep_topology:
        m.points, m.face_ptr, m.face_nodes = points, face_ptr, face_nodes
    return m


def polymesh_mesh(points, face_ptr, face_nodes, owner, neighbour, numCells, patch_type,
                  patch_nfaces, patch_start, device: int | None = None) -> Mesh:
    """A polyMesh (1-based arrays) with the reference's boundary bookkeeping; with
    `device` set, the geometry is computed by the GPU kernels on that device."""
    counts = {k: 0 for k in ("ninl", "nout", "nsym", "nwal", "npru")}
    starts = {}
    key = {"inlet": ("ninl", "iInletFacesStart"), "outlet": ("nout", "iOutletFacesStart"),
           "symmetry": ("nsym", "iSymmetryFacesStart"), "prOutlet": ("npru", "iPressOutletFacesStart")}
    for t in _WALL_ALIASES:
        key[t] = ("nwal", "iWallFacesStart")
    # 'domain' (O-C grid cut) and 'cyclic' patches come in pairs of lines, a patch and its
    # friend of as many faces; face k of one is matched with face k of the other
    # (mesh_geometry_and_topology.f90:453-462, 800-845).  The O-C pairs come first, then
    # the cyclic ones (:1163); iOCFacesStart is the start of the first 'domain' patch.
    pairs = {"domain": [], "cyclic": []}
    pend, oc_start = None, None
    for t, cnt, st in zip(patch_type, patch_nfaces, patch_start):
        t = str(t)
        if t in pairs:
            if pend is None:
                pend = (t, int(cnt), int(st))
                if t == "domain" and oc_start is None:
                    oc_start = int(st)
            else:
                if pend[0] != t or pend[1] != int(cnt):
                    raise ValueError(f"a {pend[0]!r} patch of {pend[1]} faces is followed by "
                                     f"{t!r} of {int(cnt)}, not by its friend")
                pairs[t].append((pend[2], int(st), pend[1]))
                pend = None
            continue
        if t not in key:
            raise ValueError(f"boundary type {t!r} is not supported")
        c, s = key[t]
        if counts[c] == 0:
            starts[s] = int(st)
        counts[c] += int(cnt)
    if pend is not None:
        raise ValueError(f"a {pend[0]!r} patch without its friend")
    runs = pairs["domain"] + pairs["cyclic"]
    ijl = [s0 + 1 + k for s0, _, c in runs for k in range(c)]
    ijr = [s1 + 1 + k for _, s1, c in runs for k in range(c)]
    geo = compute_geometry if device is None else (
        lambda *a: compute_geometry_gpu(*a, device=device))
    g = geo(points, face_ptr, face_nodes, owner, neighbour, int(numCells))
    return Mesh(int(numCells), len(face_ptr) - 1, len(neighbour),
                np.ascontiguousarray(owner, np.int32), np.ascontiguousarray(neighbour, np.int32),
                **g, counts=counts, starts=starts, points=np.asarray(points),
                face_ptr=np.asarray(face_ptr, np.int32), face_nodes=np.asarray(face_nodes, np.int32),
                noc=len(ijl), ncyc=sum(c for _, _, c in pairs["cyclic"]),
                iOCFacesStart=oc_start or 0,
                ijlFace=np.array(ijl, np.int32) if ijl else None,
                ijrFace=np.array(ijr, np.int32) if ijr else None)


def uniform(seed: int, stream: int, count: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    """Counter-based U(lo, hi) numbers keyed by (seed, stream)."""
    out = np.zeros(count)
    rc = _lib.load().fcg_uniform_fill(int(seed), int(stream), int(count), float(lo), float(hi), _p(out))
    if rc != 0:
        raise _lib.FcgError(rc, "fcg_uniform_fill")
    return out
