"""Mesh fixtures shared by the tests: jittered hex meshes from libfcgpu.so's generator
and the reference's cavity and pitzDaily polyMeshes (tests/golden/*.npz)."""
from __future__ import annotations

import functools
import os

import numpy as np

import freecappuccino_gb300 as fcg
from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@functools.lru_cache(maxsize=None)
def fixture_mesh(name: str) -> fcg.Mesh:
    d = np.load(os.path.join(GOLDEN, f"{name}_mesh.npz"))
    return fcg.polymesh_mesh(d["points"], d["face_ptr"], d["face_nodes"], d["owner"],
                             d["neighbour"], int(d["numCells"]), d["patch_type"],
                             d["patch_nfaces"], d["patch_start"])


@functools.lru_cache(maxsize=None)
def hex_mesh(N: int, jitter: float = 0.2, seed: int = 7) -> fcg.Mesh:
    return fcg.hex_mesh(N, jitter=jitter, seed=seed, keep_topology=True)


@functools.lru_cache(maxsize=None)
def oc_split_mesh(N: int, kc: int | None = None, jitter: float = 0.0, seed: int = 7,
                  cyclic: bool = False) -> fcg.Mesh:
    """The N^3 hex mesh with the inner faces between planes kc - 1 and kc (default N/2)
    made O-C pairs, as a mesh cut into two blocks reads them ('domain' patches, or
    'cyclic' with cyclic=True): every cut face becomes a left face owned by the cell
    below and a friend face owned by the cell above (area reversed), both after the other
    boundary faces, left faces first (iOCFacesStart)."""
    m = fcg.hex_mesh(N, jitter=jitter, seed=seed, keep_topology=True)
    nin, nf = m.numInnerFaces, m.numFaces
    own0, nb0 = m.owner[:nin] - 1, m.neighbour - 1
    kc = N // 2 if kc is None else kc
    cut = (own0 // (N * N) == kc - 1) & (nb0 // (N * N) == kc)
    keep = np.flatnonzero(~cut)
    ci = np.flatnonzero(cut)
    bnd = np.arange(nin, nf)
    noc = len(ci)
    src = np.concatenate([keep, bnd, ci, ci])  # the old face each new face copies
    flip = np.concatenate([np.ones(len(keep) + len(bnd) + noc), -np.ones(noc)])
    owner = np.concatenate([m.owner[keep], m.owner[bnd], m.owner[ci], m.neighbour[ci]])
    geo = {k: getattr(m, k)[src] * (flip if k.startswith("ar") else 1.0)
           for k in ("arx", "ary", "arz", "xf", "yf", "zf")}
    start = nf - noc  # 0-based: the left faces follow the old boundary faces
    out = fcg.Mesh(m.numCells, nf + noc, nin - noc, owner.astype(np.int32),
                   m.neighbour[keep].astype(np.int32), xc=m.xc, yc=m.yc, zc=m.zc, vol=m.vol,
                   facint=m.facint[keep], counts=dict(m.counts),
                   starts={k: v - noc for k, v in m.starts.items()}, **geo)
    out.noc, out.ncyc, out.iOCFacesStart = noc, noc if cyclic else 0, start
    out.ijlFace = (start + 1 + np.arange(noc)).astype(np.int32)
    out.ijrFace = (start + 1 + noc + np.arange(noc)).astype(np.int32)
    # the faces' nodes in the new order, the friend faces' reversed
    fp, fn = m.face_ptr, m.face_nodes
    rows = [fn[fp[f]:fp[f + 1]][::int(s)] for f, s in zip(src, flip)]
    out.points = m.points
    out.face_ptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    out.face_nodes = np.concatenate(rows).astype(np.int32)
    return out


@functools.lru_cache(maxsize=None)
def mixed_patch_mesh(N: int = 8) -> fcg.Mesh:
    """A jittered N^3 hex mesh whose boundary faces carry all five boundary types: the
    symmetry faces relabelled in four runs as inlet, outlet, pressure outlet and symmetry,
    the x = 0 faces kept as wall."""
    m = hex_mesh(N, 0.2)
    ns, ss = m.counts["nsym"], m.starts["iSymmetryFacesStart"]
    q = ns // 4
    types = ["inlet", "outlet", "prOutlet", "symmetry", "wall"]
    nfaces = [q, q, q, ns - 3 * q, m.counts["nwal"]]
    starts = [ss, ss + q, ss + 2 * q, ss + 3 * q, m.starts["iWallFacesStart"]]
    return fcg.polymesh_mesh(m.points, m.face_ptr, m.face_nodes, m.owner, m.neighbour,
                             m.numCells, types, nfaces, starts)


def mesh_by_name(name: str) -> fcg.Mesh:
    if name.startswith("hexmix"):
        return mixed_patch_mesh(int(name[6:]))
    if name.startswith("hex"):
        # hexN or hexN_u (uniform)
        body = name[3:]
        uniform = body.endswith("_u")
        N = int(body[:-2] if uniform else body)
        return hex_mesh(N, 0.0 if uniform else 0.2)
    return fixture_mesh(name)


def oracle_mesh(m: fcg.Mesh) -> oracle.Mesh:
    return oracle.Mesh(**m.oracle_kwargs())


def oracle_csr(m: fcg.Mesh) -> oracle.CSR:
    return oracle.create_csr(m.numCells, m.owner, m.neighbour)


def seeded_fields(m: fcg.Mesh, seed: int = 3):
    """Seeded flow fields for facefluxmass / fluxmc / gradient parity."""
    from freecappuccino_gb300.systems import flow_fields

    return flow_fields(m, seed)


def poisson_system(m: fcg.Mesh, seed: int = 11, mu_value: float = -1.0):
    """The pressure Poisson system of the benchmark: mu = -1, su = U(-1,1)*vol, phi = 0."""
    mu = np.full(m.numCells, mu_value)
    phi = np.zeros(m.numTotal)
    su = fcg.uniform(seed, 0, m.numCells) * m.vol
    return mu, phi, su
