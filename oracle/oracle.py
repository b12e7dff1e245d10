"""ctypes front end of the CPU oracle (``oracle/_build/liboracle.so``).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA library.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
this module.  Every function restates a freeCappuccino subroutine; the C source
(``fcg_oracle.c``) cites the Fortran file and line of each loop.

Index values (owner, neighbour, ioffset, ja, diag, slot maps) are 1-based, as the
Fortran arrays hold them.  Gradients are ``(n, 3)`` arrays (component fastest in
memory, the reference's ``dPhidxi(3, numCells)``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc -O2 -ffp-contract=off)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("fcg_oracle.c", "fcg_oracle.h")
    ):
        subprocess.run(["make", "-s", "-C", _HERE, "-B"], check=True)
    return _LIB_PATH


class _Mesh(C.Structure):
    _fields_ = [
        ("numCells", C.c_int), ("numFaces", C.c_int), ("numInnerFaces", C.c_int),
        ("ninl", C.c_int), ("nout", C.c_int), ("nsym", C.c_int), ("nwal", C.c_int),
        ("npru", C.c_int),
        ("iInletFacesStart", C.c_int), ("iOutletFacesStart", C.c_int),
        ("iSymmetryFacesStart", C.c_int), ("iWallFacesStart", C.c_int),
        ("iPressOutletFacesStart", C.c_int),
        ("owner", _ip), ("neighbour", _ip),
        ("arx", _dp), ("ary", _dp), ("arz", _dp), ("xf", _dp), ("yf", _dp), ("zf", _dp),
        ("xc", _dp), ("yc", _dp), ("zc", _dp), ("vol", _dp), ("facint", _dp),
        ("noc", C.c_int), ("ncyc", C.c_int), ("iOCFacesStart", C.c_int),
        ("ijlFace", _ip), ("ijrFace", _ip),
    ]


class _Opts(C.Structure):
    _fields_ = [("resmax", C.c_double), ("nsw", C.c_int), ("small", C.c_double),
                ("early_exit", C.c_int), ("trace", _dp),
                ("noc", C.c_int), ("ijl", _ip), ("ijr", _ip), ("ar", _dp), ("al", _dp)]


class _Out(C.Structure):
    _fields_ = [("res0", C.c_double), ("resl", C.c_double), ("resor", C.c_double),
                ("iters", C.c_int), ("resor_written", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        for name in ("orc_const_small_src", "orc_const_small_test", "orc_const_tol"):
            getattr(_lib, name).restype = C.c_double
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def small_src() -> float:
    return lib().orc_const_small_src()


def small_test() -> float:
    return lib().orc_const_small_test()


def tol() -> float:
    return lib().orc_const_tol()


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Mesh:
    """Holds the arrays of module ``geometry`` and exposes them as an ``orc_mesh``."""

    def __init__(self, numCells, numFaces, numInnerFaces, owner, neighbour, arx, ary, arz,
                 xf, yf, zf, xc, yc, zc, vol, facint, ninl=0, nout=0, nsym=0, nwal=0, npru=0,
                 iInletFacesStart=0, iOutletFacesStart=0, iSymmetryFacesStart=0,
                 iWallFacesStart=0, iPressOutletFacesStart=0, noc=0, ncyc=0, iOCFacesStart=0,
                 ijlFace=None, ijrFace=None):
        self.numCells, self.numFaces, self.numInnerFaces = numCells, numFaces, numInnerFaces
        self.numTotal = numCells + numFaces - numInnerFaces
        self.arrays = dict(owner=_i32(owner), neighbour=_i32(neighbour), arx=_f64(arx),
                           ary=_f64(ary), arz=_f64(arz), xf=_f64(xf), yf=_f64(yf), zf=_f64(zf),
                           xc=_f64(xc), yc=_f64(yc), zc=_f64(zc), vol=_f64(vol),
                           facint=_f64(facint))
        self.counts = dict(ninl=ninl, nout=nout, nsym=nsym, nwal=nwal, npru=npru)
        self.starts = dict(iInletFacesStart=iInletFacesStart, iOutletFacesStart=iOutletFacesStart,
                           iSymmetryFacesStart=iSymmetryFacesStart, iWallFacesStart=iWallFacesStart,
                           iPressOutletFacesStart=iPressOutletFacesStart)
        s = _Mesh()
        s.numCells, s.numFaces, s.numInnerFaces = numCells, numFaces, numInnerFaces
        for k, v in {**self.counts, **self.starts}.items():
            setattr(s, k, int(v))
        for k, v in self.arrays.items():
            setattr(s, k, _i(v) if v.dtype == np.int32 else _d(v))
        # O-C grid cuts and cyclic pairs (1-based face indices of each pair's two faces)
        self.noc, self.ncyc, self.iOCFacesStart = int(noc), int(ncyc), int(iOCFacesStart)
        if self.noc:
            self.arrays["ijlFace"], self.arrays["ijrFace"] = _i32(ijlFace), _i32(ijrFace)
            s.ijlFace, s.ijrFace = _i(self.arrays["ijlFace"]), _i(self.arrays["ijrFace"])
        s.noc, s.ncyc, s.iOCFacesStart = self.noc, self.ncyc, self.iOCFacesStart
        self.struct = s

    def __getattr__(self, k):
        arrays = self.__dict__.get("arrays", {})
        if k in arrays:
            return arrays[k]
        raise AttributeError(k)


def geometry(x, y, z, numCells, numInnerFaces, face_ptr, face_nodes, owner, neighbour):
    """mesh_geometry_and_topology.f90:859-1079 on a face list (1-based node ids)."""
    x, y, z = _f64(x), _f64(y), _f64(z)
    face_ptr, face_nodes = _i32(face_ptr), _i32(face_nodes)
    owner, neighbour = _i32(owner), _i32(neighbour)
    nf = len(face_ptr) - 1
    out = {k: np.zeros(nf) for k in ("arx", "ary", "arz", "xf", "yf", "zf")}
    out.update({k: np.zeros(numCells) for k in ("xc", "yc", "zc", "vol")})
    out["facint"] = np.zeros(max(numInnerFaces, 1))
    rc = lib().orc_geometry(len(x), _d(x), _d(y), _d(z), numCells, nf, numInnerFaces,
                            _i(face_ptr), _i(face_nodes), _i(owner), _i(neighbour),
                            *[_d(out[k]) for k in ("arx", "ary", "arz", "xf", "yf", "zf", "xc",
                                                   "yc", "zc", "vol", "facint")])
    assert rc == 0
    out["facint"] = out["facint"][:numInnerFaces]
    return out


@dataclass
class CSR:
    ioffset: np.ndarray
    ja: np.ndarray
    diag: np.ndarray
    slot_pn: np.ndarray
    slot_np: np.ndarray

    @property
    def nnz(self):
        return len(self.ja)


def create_csr(numCells, owner, neighbour) -> CSR:
    """sparse_matrix.f90:42-172."""
    owner, neighbour = _i32(owner), _i32(neighbour)
    nin = len(neighbour)
    nnz = numCells + 2 * nin
    c = CSR(np.zeros(numCells + 1, np.int32), np.zeros(nnz, np.int32), np.zeros(numCells, np.int32),
            np.zeros(max(nin, 1), np.int32), np.zeros(max(nin, 1), np.int32))
    assert lib().orc_create_csr(numCells, nin, _i(owner), _i(neighbour), _i(c.ioffset), _i(c.ja),
                                _i(c.diag), _i(c.slot_pn), _i(c.slot_np)) == 0
    c.slot_pn, c.slot_np = c.slot_pn[:nin], c.slot_np[:nin]
    return c


def oc_geometry(m: Mesh):
    """ijl, ijr (1-based cells), foc and srdoc of the mesh's O-C and cyclic pairs
    (mesh_geometry_and_topology.f90:814-845, 1083-1152)."""
    ijl, ijr = np.zeros(max(m.noc, 1), np.int32), np.zeros(max(m.noc, 1), np.int32)
    foc, srdoc = np.zeros(max(m.noc, 1)), np.zeros(max(m.noc, 1))
    assert lib().orc_oc_geometry(C.byref(m.struct), _i(ijl), _i(ijr), _d(foc), _d(srdoc)) == 0
    return ijl[: m.noc], ijr[: m.noc], foc[: m.noc], srdoc[: m.noc]


def laplacian(m: Mesh, csr: CSR, mu, phi, su):
    """fvm_laplacian.f90:1-163. Returns (a, su) with su updated by the wall terms; with O-C
    pairs a holds nnz + 2 noc values (the CSR values, then ar, then al)."""
    mu, phi, su = _f64(mu), _f64(phi), _f64(su).copy()
    a = np.zeros(csr.nnz + 2 * m.noc)
    assert lib().orc_laplacian(C.byref(m.struct), _i(csr.ioffset), _i(csr.diag), _i(csr.slot_pn),
                               _i(csr.slot_np), _d(mu), _d(phi), _d(a), _d(su)) == 0
    return a, su


def facefluxmass(m: Mesh, csr: CSR, u, v, w, p, dUdxi, dVdxi, dWdxi, dPdxi, apu, apv, apw, den):
    """calcp-multiple_correction_SIMPLE.f90:34-100 with facefluxmass.f90:34-199.  With O-C
    pairs a holds ar, al after the CSR values and flmass the pairs' fmoc after the inner
    faces' fluxes."""
    args = [_f64(t) for t in (u, v, w, p, dUdxi, dVdxi, dWdxi, dPdxi, apu, apv, apw, den)]
    a = np.zeros(csr.nnz + 2 * m.noc)
    su = np.zeros(m.numCells)
    flmass = np.zeros(max(m.numInnerFaces + m.noc, 1))
    assert lib().orc_facefluxmass(C.byref(m.struct), _i(csr.diag), _i(csr.slot_pn), _i(csr.slot_np),
                                  *[_d(t) for t in args], csr.nnz, _d(a), _d(su), _d(flmass)) == 0
    return a, su, flmass[:m.numInnerFaces + m.noc]


def fluxmc(m: Mesh, dPdxi, apu, den, flmass):
    """calcp-multiple_correction_SIMPLE.f90:193-206 with fluxmc facefluxmass.f90:520-607."""
    dPdxi, apu, den = _f64(dPdxi), _f64(apu), _f64(den)
    flmass = _f64(flmass).copy()
    su = np.zeros(m.numCells)
    assert lib().orc_fluxmc(C.byref(m.struct), _d(dPdxi), _d(apu), _d(den), _d(su), _d(flmass)) == 0
    return su, flmass


def flux_correct(m: Mesh, csr: CSR, a, pp, flmass):
    """calcp-multiple_correction_SIMPLE.f90:159-171 (mass-flux correction by p')."""
    flmass = _f64(flmass).copy()
    assert lib().orc_flux_correct(C.byref(m.struct), _i(_i32(csr.slot_pn)), _d(_f64(a)),
                                  _d(_f64(pp)), _d(flmass)) == 0
    return flmass


def correct_fields(m: Mesh, dPdxi, apu, apv, apw, pp, urf, pRefCell, u, v, w, p):
    """calcp-multiple_correction_SIMPLE.f90:184-189 (velocity and pressure correction)."""
    u, v, w, p = (_f64(x).copy() for x in (u, v, w, p))
    assert lib().orc_correct_fields(C.byref(m.struct), _d(_f64(dPdxi)), _d(_f64(apu)),
                                    _d(_f64(apv)), _d(_f64(apw)), _d(_f64(pp)), C.c_double(urf),
                                    int(pRefCell), _d(u), _d(v), _d(w), _d(p)) == 0
    return u, v, w, p


class UvwParams(C.Structure):
    """orc_uvw_params (calcuvw's parameters)."""
    _fields_ = [("scheme", C.c_int), ("limiter", C.c_int), ("gds", C.c_double),
                ("viscos", C.c_double), ("urfr", C.c_double * 3), ("urfm", C.c_double * 3),
                ("bdf", C.c_int), ("cn", C.c_int), ("timestep", C.c_double),
                ("btime", C.c_double), ("const_mflux", C.c_int), ("gradPcmf", C.c_double),
                ("buoyancy", C.c_int), ("boussinesq", C.c_int), ("beta", C.c_double),
                ("densit", C.c_double), ("tref", C.c_double), ("gravx", C.c_double),
                ("gravy", C.c_double), ("gravz", C.c_double)]


def calcuvw(m: Mesh, csr: CSR, prm: UvwParams, a, u, v, w, p, vis, den, dUdxi, dVdxi, dWdxi,
            dPdxi, flmass, fmi=None, fmo=None, t=None, uo=None, vo=None, wo=None, uoo=None,
            voo=None, woo=None):
    """calcuvw.f90:48-438 without its solves: returns (a, diag_vw (2,n), rhs (3,n), ap (3,n))."""
    n = m.numCells
    a = _f64(a).copy()
    dvw, rhs, ap = np.zeros((2, n)), np.zeros((3, n)), np.zeros((3, n))
    fmi = _f64(fmi) if fmi is not None and len(fmi) else np.zeros(1)
    fmo = _f64(fmo) if fmo is not None and len(fmo) else np.zeros(1)
    rc = lib().orc_calcuvw(
        C.byref(m.struct), _i(csr.ioffset), _i(csr.diag), _i(csr.slot_pn), _i(csr.slot_np),
        C.byref(prm), *[_d(_f64(x)) for x in (u, v, w, p, vis, den)], _opt(t, n), _opt(uo, n),
        _opt(vo, n), _opt(wo, n), _opt(uoo, n), _opt(voo, n), _opt(woo, n),
        *[_d(_f64(x)) for x in (dUdxi, dVdxi, dWdxi, dPdxi, flmass)], _d(fmi), _d(fmo), _d(a),
        _d(dvw), _d(rhs), _d(ap))
    assert rc == 0
    return a, dvw, rhs, ap


class HbyaParams(C.Structure):
    """Parameters read by get_rAU_x_UEqnH (modules_allocatable.f90:40-106)."""
    _fields_ = [("timestep", C.c_double), ("btime", C.c_double), ("bdf", C.c_int),
                ("cn", C.c_int), ("buoyancy", C.c_int), ("boussinesq", C.c_int),
                ("beta", C.c_double), ("densit", C.c_double), ("tref", C.c_double),
                ("gravx", C.c_double), ("gravy", C.c_double), ("gravz", C.c_double)]


def _opt(a, n):
    return _d(_f64(a)) if a is not None else _d(np.zeros(max(n, 1)))


def piso_hbya(m: Mesh, csr: CSR, prm: HbyaParams, h, den, apu, apv, apw, u, v, w,
              t=None, uo=None, vo=None, wo=None, uoo=None, voo=None, woo=None):
    """get_rAU_x_UEqnH.f90:3-208. Returns (u, v, w, su, sv, sw); the cell part of u, v, w
    is overwritten with apu*su etc."""
    n = m.numCells
    u, v, w = (_f64(x).copy() for x in (u, v, w))
    su, sv, sw = np.zeros(n), np.zeros(n), np.zeros(n)
    assert lib().orc_piso_hbya(
        C.byref(m.struct), _i(csr.ioffset), _i(csr.diag), _i(csr.slot_pn), _i(csr.slot_np),
        C.byref(prm), _d(_f64(h)), _opt(den, n), _opt(t, n), _opt(uo, n), _opt(vo, n),
        _opt(wo, n), _opt(uoo, n), _opt(voo, n), _opt(woo, n), _d(_f64(apu)), _d(_f64(apv)),
        _d(_f64(apw)), _d(u), _d(v), _d(w), _d(su), _d(sv), _d(sw)) == 0
    return u, v, w, su, sv, sw


def facefluxmass_piso(m: Mesh, csr: CSR, u, v, w, dUdxi, dVdxi, dWdxi, apu, den):
    """PISO_multiple_correction.f90:109-148 with facefluxmass_piso (facefluxmass.f90:294-358).
    Returns (a, su, flmass)."""
    args = [_f64(t) for t in (u, v, w, dUdxi, dVdxi, dWdxi, apu, den)]
    a = np.zeros(csr.nnz + 2 * m.noc)
    su = np.zeros(m.numCells)
    flmass = np.zeros(max(m.numInnerFaces + m.noc, 1))
    assert lib().orc_facefluxmass_piso(C.byref(m.struct), _i(csr.diag), _i(csr.slot_pn),
                                       _i(csr.slot_np), *[_d(t) for t in args], csr.nnz, _d(a),
                                       _d(su), _d(flmass)) == 0
    return a, su, flmass[:m.numInnerFaces + m.noc]


def adjust_mass_flow(m: Mesh, den, flomas, fmi, u, v, w, su):
    """adjustMassFlow.f90:1-71. Returns (u, v, w, fmo, su)."""
    u, v, w, su = (_f64(x).copy() for x in (u, v, w, su))
    fmo = np.zeros(max(m.struct.nout, 1))
    fmi = _f64(fmi) if len(fmi) else np.zeros(1)
    assert lib().orc_adjust_mass_flow(C.byref(m.struct), _d(_f64(den)), C.c_double(flomas),
                                      _d(fmi), _d(u), _d(v), _d(w), _d(fmo), _d(su)) == 0
    return u, v, w, fmo[:m.struct.nout], su


def set_reference_pressure(csr: CSR, pRefCell, p, a, su):
    """PISO_multiple_correction.f90:188-192. Returns (a, su)."""
    a, su = _f64(a).copy(), _f64(su).copy()
    assert lib().orc_set_reference_pressure(_i(csr.ioffset), _i(csr.diag), int(pRefCell),
                                            _d(_f64(p)), _d(a), _d(su)) == 0
    return a, su


def correct_velocity_piso(m: Mesh, dPdxi, apu, apv, apw, u, v, w):
    """PISO_multiple_correction.f90:300-304. Returns (u, v, w)."""
    u, v, w = (_f64(x).copy() for x in (u, v, w))
    assert lib().orc_correct_velocity_piso(C.byref(m.struct), _d(_f64(dPdxi)), _d(_f64(apu)),
                                           _d(_f64(apv)), _d(_f64(apw)), _d(u), _d(v), _d(w)) == 0
    return u, v, w


def correct_bc_velocity(m: Mesh, den, flomas, u, v, w):
    """correctBoundaryConditionsVelocity.f90:1-80: returns (u, v, w, fmo)."""
    u, v, w = (_f64(x).copy() for x in (u, v, w))
    fmo = np.zeros(max(m.struct.nout, 1))
    assert lib().orc_correct_bc_velocity(C.byref(m.struct), _d(_f64(den)), C.c_double(flomas),
                                         _d(u), _d(v), _d(w), _d(fmo)) == 0
    return u, v, w, fmo[:m.struct.nout]


def continuity_errors(m: Mesh, flmass, fmi, fmo):
    """continuityErrors.h:1-52: returns (res, sumLocalContErr, globalContErr)."""
    res = np.zeros(m.struct.numCells)
    sl, sg = C.c_double(), C.c_double()
    fmi = _f64(fmi) if len(fmi) else np.zeros(1)
    fmo = _f64(fmo) if len(fmo) else np.zeros(1)
    assert lib().orc_continuity_errors(C.byref(m.struct), _d(_f64(flmass)), _d(fmi), _d(fmo),
                                       _d(res), C.byref(sl), C.byref(sg)) == 0
    return res, sl.value, sg.value


def grad_gauss(m: Mesh, phi, nigrad=1, corrected=False, dphidxi_in=None):
    """grad_gauss.f90 (nigrad passes) or grad_gauss_corrected.f90 (one pass, old = incoming)."""
    phi = _f64(phi)
    g = np.zeros((m.numCells, 3)) if dphidxi_in is None else _f64(dphidxi_in).copy()
    assert lib().orc_grad_gauss(C.byref(m.struct), _d(phi), int(nigrad), int(bool(corrected)),
                                _d(g)) == 0
    return g


def grad_lsq_matrix(m: Mesh):
    """grad_lsq.f90 stage 1 (:50-165). Returns dmat as (n, 9)."""
    d = np.zeros((m.numCells, 9))
    assert lib().orc_grad_lsq_matrix(C.byref(m.struct), _d(d)) == 0
    return d


def grad_lsq(m: Mesh, phi, dmat):
    """grad_lsq.f90 stage 2 (:168-306)."""
    phi, dmat = _f64(phi), _f64(dmat)
    g = np.zeros((m.numCells, 3))
    assert lib().orc_grad_lsq(C.byref(m.struct), _d(phi), _d(dmat), _d(g)) == 0
    return g


def bpres(m: Mesh, p, dPdxi, istage):
    """bpres.f90:3-152. Returns the updated p(numTotal)."""
    p = _f64(p).copy()
    dPdxi = _f64(dPdxi) if dPdxi is not None else np.zeros((m.numCells, 3))
    assert lib().orc_bpres(C.byref(m.struct), _d(p), _d(dPdxi), int(istage)) == 0
    return p


@dataclass
class SolveResult:
    fi: np.ndarray
    res: np.ndarray
    res0: float
    resl: float
    iters: int
    resor: float | None
    trace: np.ndarray


def _solve(fn, csr: CSR, a, su, fi, sor, nsw, small=None, early_exit=True,
           oc=None) -> SolveResult:
    """oc = (ijl, ijr), 1-based: the O-C pairs, whose ar and al follow the CSR values in a."""
    n = len(csr.diag)
    a, su = _f64(a), _f64(su)
    fi = _f64(fi).copy()
    res = np.zeros(n)
    trace = np.zeros(2 * max(nsw, 1))
    o = _Opts(float(sor), int(nsw), small_src() if small is None else float(small),
              int(bool(early_exit)), _d(trace))
    if oc is not None and len(oc[0]):
        ijl, ijr = _i32(oc[0]), _i32(oc[1])
        noc, nnz = len(ijl), csr.nnz
        ar, al = np.ascontiguousarray(a[nnz:nnz + noc]), np.ascontiguousarray(a[nnz + noc:nnz + 2 * noc])
        assert len(a) == nnz + 2 * noc
        o.noc, o.ijl, o.ijr, o.ar, o.al = noc, _i(ijl), _i(ijr), _d(ar), _d(al)
        keep = (ijl, ijr, ar, al)  # noqa: F841 (alive across the call)
    out = _Out()
    assert fn(n, _i(csr.ioffset), _i(csr.ja), _i(csr.diag), _d(a), _d(su), _d(fi), _d(res),
              C.byref(o), C.byref(out)) == 0
    return SolveResult(fi, res, out.res0, out.resl, out.iters,
                       out.resor if out.resor_written else None,
                       trace[: 2 * out.iters].reshape(-1, 2))


def dpcg(csr, a, su, fi, sor, nsw, **kw) -> SolveResult:
    """dpcg.f90:3-154."""
    return _solve(lib().orc_dpcg, csr, a, su, fi, sor, nsw, **kw)


def iccg(csr, a, su, fi, sor, nsw, **kw) -> SolveResult:
    """iccg.f90:3-177 (DIC preconditioner)."""
    return _solve(lib().orc_iccg, csr, a, su, fi, sor, nsw, **kw)


def bicgstab(csr, a, su, fi, sor, nsw, **kw) -> SolveResult:
    """bicgstab.f90:1-231 (DILU preconditioner)."""
    return _solve(lib().orc_bicgstab, csr, a, su, fi, sor, nsw, **kw)


def spmv(csr: CSR, a, x):
    a, x = _f64(a), _f64(x)
    y = np.zeros(len(csr.diag))
    assert lib().orc_spmv(len(csr.diag), _i(csr.ioffset), _i(csr.ja), _d(a), _d(x), _d(y)) == 0
    return y
