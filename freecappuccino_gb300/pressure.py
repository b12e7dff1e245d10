"""Python face of the pressure-correction path, mirroring the reference's Fortran calls.

The reference calls ``laplacian(mu,phi)``, ``facefluxmass(...)`` (inside ``calcp``),
``fluxmc``, ``grad(phi,dPhidxi[,option])``, ``bpres(p,istage)`` and
``dpcg/iccg/bicgstab(fi,ifi)`` on module-global arrays.  ``Context`` holds that state for
one mesh on one GPU and exposes the same operations with the arrays passed explicitly.
Arrays may be numpy arrays (host; copied in and out inside each call) or CUDA tensors
(used in place).  Every call goes through libfcgpu.so; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .mesh import Mesh

_GRAD = {"gauss": _lib.FCG_GRAD_GAUSS, "gauss_corrected": _lib.FCG_GRAD_GAUSS_CORRECTED,
         "lsq": _lib.FCG_GRAD_LSQ}


def _is_torch(x) -> bool:
    return hasattr(x, "data_ptr") and hasattr(x, "is_cuda")


def _ptr(x):
    if x is None:
        return None
    if _is_torch(x):
        return x.data_ptr()
    return x.ctypes.data


def _like(ref, shape, dtype=np.float64):
    """A zero array on the same side (host or device) as `ref`."""
    if _is_torch(ref):
        import torch

        tdt = {np.float64: torch.float64, np.int32: torch.int32}[dtype]
        return torch.zeros(shape, dtype=tdt, device=ref.device)
    return np.zeros(shape, dtype=dtype)


def _host(x, dtype=np.float64):
    if _is_torch(x):
        return x
    return np.ascontiguousarray(x, dtype=dtype)


@dataclass
class SolveResult:
    fi: object
    res: object
    res0: float
    resl: float
    iters: int
    converged: bool
    resor: float | None
    l2_rel: float
    seconds: float
    trace: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))


# Log-line names of the reference solvers (dpcg.f90:150, iccg.f90:328, bicgstab.f90:227).
SOLVER_NAMES = {"dpcg": "PCG(Jacobi):  ", "iccg": "  PCG(IC0):  ", "bicgstab": "  BiCGStab(ILU(0)):  ",
                "dpcg_mixed": "PCG(Jacobi, FP32 sweeps + FP64 updates):  "}


def solver_log(kind: str, var: str, r: SolveResult) -> str:
    """The reference's one-line solver report, format '(3a,1PE10.3,a,1PE10.3,a,I0)'."""
    return (f"{SOLVER_NAMES[kind]}Solving for {var}, Initial residual = {r.res0:10.3E}, "
            f"Final residual = {r.resl:10.3E}, No Iterations {r.iters}")


class Context:
    """An fcg_context bound to one mesh."""

    def __init__(self, mesh: Mesh, device: int = 0):
        self.lib = _lib.load()
        self.mesh = mesh
        h = C.c_void_p()
        rc = self.lib.fcg_create(C.byref(h), int(device))
        if rc != 0:
            raise _lib.FcgError(rc, "fcg_create", "no usable sm_103a CUDA device")
        self.h = h
        self._stream, self._pinned = None, False
        self._desc = mesh.desc()  # keeps the pointers alive for the call
        self._check(self.lib.fcg_bind_mesh(self.h, C.byref(self._desc)), "fcg_bind_mesh")
        self.n, self.nnz, self.ntot = mesh.numCells, mesh.nnz, mesh.numTotal

    # -- plumbing -------------------------------------------------------------
    def _check(self, rc, where):
        if rc != 0:
            raise _lib.FcgError(rc, where, self.lib.fcg_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fcg_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        """Queue the context's work on this CUDA stream from now on (and stop following
        torch's current stream)."""
        self._check(self.lib.fcg_set_stream(self.h, stream_handle), "fcg_set_stream")
        self._stream, self._pinned = stream_handle, True

    def _follow(self, *xs):
        """With CUDA tensors among the arguments, queue the library's work on torch's
        current stream (unless a stream was set explicitly): the work is then ordered
        after the kernels that produced the tensors and before those that read the
        results."""
        if self._pinned:
            return
        for x in xs:
            if _is_torch(x) and x.is_cuda:
                import torch

                # handle 0 is the legacy default stream, while the library reads NULL as
                # the context's own stream: pass cudaStreamLegacy (1) for it
                s = torch.cuda.current_stream(x.device).cuda_stream or 1
                if s != self._stream:
                    self._check(self.lib.fcg_set_stream(self.h, s), "fcg_set_stream")
                    self._stream = s
                return

    def topology_digest(self) -> int:
        """64-bit digest of every topology array bound to the device."""
        d = C.c_ulonglong()
        self._check(self.lib.fcg_topology_digest(self.h, C.byref(d)), "fcg_topology_digest")
        return d.value

    def synchronize(self):
        self._check(self.lib.fcg_synchronize(self.h), "fcg_synchronize")

    # -- a1 -----------------------------------------------------------------------
    def create_csr(self):
        """(ioffset, ja, diag, slot_pn, slot_np), 1-based (sparse_matrix.f90:42-172)."""
        n, nin = self.n, self.mesh.numInnerFaces
        io, ja, dg = np.zeros(n + 1, np.int32), np.zeros(self.nnz, np.int32), np.zeros(n, np.int32)
        spn, snp = np.zeros(max(nin, 1), np.int32), np.zeros(max(nin, 1), np.int32)
        self._check(self.lib.fcg_create_csr(self.h, _ptr(io), _ptr(ja), _ptr(dg), _ptr(spn),
                                            _ptr(snp)), "fcg_create_csr")
        return io, ja, dg, spn[:nin], snp[:nin]

    # -- a2-a4 ----------------------------------------------------------------------
    def laplacian(self, mu, phi, su):
        """fvm_laplacian.f90 laplacian(mu,phi): returns (a, su)."""
        self._follow(mu, phi, su)
        mu, phi = _host(mu), _host(phi)
        su = su.clone() if _is_torch(su) else np.array(su, dtype=np.float64)
        a = _like(mu, self.mesh.a_len)  # with O-C pairs: ar and al after the CSR values
        self._check(self.lib.fcg_laplacian(self.h, _ptr(mu), _ptr(phi), _ptr(a), _ptr(su)),
                    "fcg_laplacian")
        return a, su

    def facefluxmass(self, u, v, w, p, dUdxi, dVdxi, dWdxi, dPdxi, apu, apv, apw, den):
        """calcp's assembly loop with facefluxmass: returns (a, su, flmass)."""
        self._follow(u, v, w, p, dUdxi, dVdxi, dWdxi, dPdxi, apu, apv, apw, den)
        arrs = [_host(t) for t in (u, v, w, p, dUdxi, dVdxi, dWdxi, dPdxi, apu, apv, apw, den)]
        ff = _lib.FlowFields(*[_ptr(t) for t in arrs])
        # with O-C pairs: ar, al after the CSR values, fmoc after the inner faces' fluxes
        nfl = self.mesh.numInnerFaces + self.mesh.noc
        a = _like(arrs[0], self.mesh.a_len)
        su = _like(arrs[0], self.n)
        fm = _like(arrs[0], max(nfl, 1))
        self._check(self.lib.fcg_facefluxmass(self.h, C.byref(ff), _ptr(a), _ptr(su), _ptr(fm)),
                    "fcg_facefluxmass")
        return a, su, fm[:nfl]

    def fluxmc(self, dPdxi, apu, den, flmass):
        """calcp's non-orthogonal corrector with fluxmc: returns (su, flmass)."""
        self._follow(dPdxi, apu, den, flmass)
        dPdxi, apu, den = _host(dPdxi), _host(apu), _host(den)
        fm = flmass.clone() if _is_torch(flmass) else np.array(flmass, dtype=np.float64)
        su = _like(apu, self.n)
        self._check(self.lib.fcg_fluxmc(self.h, _ptr(dPdxi), _ptr(apu), _ptr(den), _ptr(su),
                                        _ptr(fm)), "fcg_fluxmc")
        return su, fm

    # -- a5-a8 ----------------------------------------------------------------------
    def flux_correct(self, a, pp, flmass):
        """calcp :159-171: flmass += a(slot_PN) * (pp(N) - pp(P)); returns flmass."""
        self._follow(a, pp, flmass)
        a, pp = _host(a), _host(pp)
        flmass = flmass.clone() if _is_torch(flmass) else np.array(flmass, dtype=np.float64)
        self._check(self.lib.fcg_flux_correct(self.h, _ptr(a), _ptr(pp), _ptr(flmass)),
                    "fcg_flux_correct")
        return flmass

    def correct_fields(self, dPdxi, apu, apv, apw, pp, urf, pRefCell, u, v, w, p):
        """calcp :147,184-189: corrected (u, v, w, p); pRefCell is 1-based."""
        self._follow(dPdxi, apu, apv, apw, pp, u, v, w, p)
        ins = [_host(x) for x in (dPdxi, apu, apv, apw, pp)]
        outs = [x.clone() if _is_torch(x) else np.array(x, dtype=np.float64) for x in (u, v, w, p)]
        self._check(self.lib.fcg_correct_fields(self.h, *[_ptr(x) for x in ins], float(urf),
                                                int(pRefCell), *[_ptr(x) for x in outs]),
                    "fcg_correct_fields")
        return tuple(outs)

    def correct_bc_velocity(self, den, flomas, u, v, w):
        """correctBoundaryConditionsVelocity: returns (u, v, w, fmo)."""
        self._follow(den, u, v, w)
        den = _host(den)
        outs = [x.clone() if _is_torch(x) else np.array(x, dtype=np.float64) for x in (u, v, w)]
        nout = self.mesh.counts.get("nout", 0)
        fmo = _like(den, max(nout, 1))
        self._check(self.lib.fcg_correct_bc_velocity(self.h, _ptr(den), float(flomas),
                                                     *[_ptr(x) for x in outs], _ptr(fmo)),
                    "fcg_correct_bc_velocity")
        return (*outs, fmo[:nout])

    def continuity_errors(self, flmass, fmi, fmo):
        """continuityErrors.h: returns (res, sumLocalContErr, globalContErr)."""
        self._follow(flmass, fmi, fmo)
        flmass = _host(flmass)
        fmi = _host(fmi) if len(fmi) else _like(flmass, 1)
        fmo = _host(fmo) if len(fmo) else _like(flmass, 1)
        res = _like(flmass, self.n)
        sl, sg = C.c_double(), C.c_double()
        self._check(self.lib.fcg_continuity_errors(self.h, _ptr(flmass), _ptr(fmi), _ptr(fmo),
                                                   _ptr(res), C.byref(sl), C.byref(sg)),
                    "fcg_continuity_errors")
        return res, sl.value, sg.value

    # -- momentum assembly (calcuvw.f90:48-438) ------------------------------------------
    def calcuvw(self, u, v, w, p, vis, den, dUdxi, dVdxi, dWdxi, dPdxi, flmass, a,
                fmi=None, fmo=None, *, scheme="muscl", limiter="uds", gds=1.0, viscos=1e-3,
                urf=(0.7, 0.7, 0.7), urfr=None, urfm=None, bdf=False, cn=False, timestep=1.0,
                btime=0.0, const_mflux=False, gradPcmf=0.0, buoyancy=False, boussinesq=False,
                beta=0.0, densit=1.0, tref=0.0, grav=(0.0, 0.0, 0.0), t=None, uo=None,
                vo=None, wo=None, uoo=None, voo=None, woo=None):
        """calcuvw without its solves.  `a` carries the diagonal the reference finds in
        its module array (it is subtracted from the row sums).  Returns a dict: `a` (the
        off-diagonals and the u diagonal), `diag_vw` (2, n), `rhs` (3, n), `ap` (3, n).
        urfr/urfm default to 1/urf and 1-urf."""
        urfr = [1.0 / x for x in urf] if urfr is None else list(urfr)
        urfm = [1.0 - x for x in urf] if urfm is None else list(urfm)
        prm = _lib.UvwParams(_lib.CONV_SCHEMES[scheme], _lib.LIMITERS[limiter], float(gds),
                             float(viscos), (C.c_double * 3)(*urfr), (C.c_double * 3)(*urfm),
                             int(bool(bdf)), int(bool(cn)), float(timestep), float(btime),
                             int(bool(const_mflux)), float(gradPcmf), int(bool(buoyancy)),
                             int(bool(boussinesq)), float(beta), float(densit), float(tref),
                             *[float(g) for g in grav])
        vals = dict(u=u, v=v, w=w, p=p, vis=vis, den=den, t=t, uo=uo, vo=vo, wo=wo, uoo=uoo,
                    voo=voo, woo=woo, dUdxi=dUdxi, dVdxi=dVdxi, dWdxi=dWdxi, dPdxi=dPdxi,
                    flmass=flmass, fmi=fmi, fmo=fmo)
        self._follow(*[x for x in vals.values() if x is not None], a)
        ins = {k: (None if x is None or (k in ("fmi", "fmo") and len(x) == 0) else _host(x))
               for k, x in vals.items()}
        fl = _lib.UvwFields(*[_ptr(ins[k]) for k in _lib.UVW_FIELDS])
        a = a.clone() if _is_torch(a) else np.array(a, dtype=np.float64)
        dvw = _like(a, (2, self.n))
        rhs = _like(a, (3, self.n))
        ap = _like(a, (3, self.n))
        self._check(self.lib.fcg_calcuvw(self.h, C.byref(prm), C.byref(fl), _ptr(a), _ptr(dvw),
                                         _ptr(rhs), _ptr(ap)), "fcg_calcuvw")
        return dict(a=a, diag_vw=dvw, rhs=rhs, ap=ap)

    def uvw_systems(self, asm):
        """The three systems of a calcuvw result as the planar values (3, nnz) and
        right-hand sides (3, n) that bicgstab_multi takes: the off-diagonals shared, each
        with its own diagonal."""
        a = asm["a"]
        lib = a if _is_torch(a) else np
        a3 = lib.stack([a, a.clone() if _is_torch(a) else a.copy(),
                        a.clone() if _is_torch(a) else a.copy()])
        d = self._diag0()
        a3[1, d] = asm["diag_vw"][0]
        a3[2, d] = asm["diag_vw"][1]
        return a3, asm["rhs"]

    def _diag0(self):
        if getattr(self, "_diag_cache", None) is None:
            self._diag_cache = self.create_csr()[2].astype(np.int64) - 1
        return self._diag_cache

    # -- PISO pressure path (PISO_multiple_correction.f90:83-307) -----------------------
    def piso_hbya(self, h, u, v, w, apu, apv, apw, den=None, *, timestep=1.0, btime=0.0,
                  bdf=False, cn=False, buoyancy=False, boussinesq=False, beta=0.0, densit=1.0,
                  tref=0.0, grav=(0.0, 0.0, 0.0), t=None, uo=None, vo=None, wo=None,
                  uoo=None, voo=None, woo=None):
        """get_rAU_x_UEqnH: returns (u, v, w, su, sv, sw) with the cell part of u, v, w
        replaced by HbyA = apu*H(U) (and the volume and old-level sources)."""
        opt = (den, t, uo, vo, wo, uoo, voo, woo)
        self._follow(h, u, v, w, apu, apv, apw, *opt)
        prm = _lib.HbyaParams(float(timestep), float(btime), int(bool(bdf)), int(bool(cn)),
                              int(bool(buoyancy)), int(bool(boussinesq)), float(beta),
                              float(densit), float(tref), *[float(g) for g in grav])
        ins = [None if x is None else _host(x) for x in opt + (apu, apv, apw)]
        fl = _lib.HbyaFields(*[_ptr(x) for x in ins])
        h = _host(h)
        outs = [x.clone() if _is_torch(x) else np.array(x, dtype=np.float64) for x in (u, v, w)]
        srcs = [_like(outs[0], self.n) for _ in range(3)]
        self._check(self.lib.fcg_piso_hbya(self.h, C.byref(prm), C.byref(fl), _ptr(h),
                                           *[_ptr(x) for x in outs], *[_ptr(x) for x in srcs]),
                    "fcg_piso_hbya")
        return (*outs, *srcs)

    def facefluxmass_piso(self, u, v, w, dUdxi, dVdxi, dWdxi, apu, den):
        """The PISO corrector's assembly with facefluxmass_piso: returns (a, su, flmass)."""
        self._follow(u, v, w, dUdxi, dVdxi, dWdxi, apu, den)
        u, v, w, dU, dV, dW, apu, den = (_host(t) for t in (u, v, w, dUdxi, dVdxi, dWdxi, apu,
                                                            den))
        ff = _lib.FlowFields(_ptr(u), _ptr(v), _ptr(w), None, _ptr(dU), _ptr(dV), _ptr(dW), None,
                             _ptr(apu), None, None, _ptr(den))
        nfl = self.mesh.numInnerFaces + self.mesh.noc  # fmoc after the inner faces' fluxes
        a = _like(u, self.mesh.a_len)
        su = _like(u, self.n)
        fm = _like(u, max(nfl, 1))
        self._check(self.lib.fcg_facefluxmass_piso(self.h, C.byref(ff), _ptr(a), _ptr(su),
                                                   _ptr(fm)), "fcg_facefluxmass_piso")
        return a, su, fm[:nfl]

    def adjust_mass_flow(self, den, flomas, fmi, u, v, w, su):
        """adjustMassFlow: returns (u, v, w, fmo, su)."""
        self._follow(den, u, v, w, su)
        den = _host(den)
        fmi = _host(fmi) if len(fmi) else _like(den, 1)
        outs = [x.clone() if _is_torch(x) else np.array(x, dtype=np.float64)
                for x in (u, v, w, su)]
        nout = self.mesh.counts.get("nout", 0)
        fmo = _like(den, max(nout, 1))
        self._check(self.lib.fcg_adjust_mass_flow(self.h, _ptr(den), float(flomas), _ptr(fmi),
                                                  *[_ptr(x) for x in outs[:3]], _ptr(fmo),
                                                  _ptr(outs[3])), "fcg_adjust_mass_flow")
        return (*outs[:3], fmo[:nout], outs[3])

    def set_reference_pressure(self, pRefCell, p, a, su):
        """PISO :188-192, row pRefCell (1-based) of a set to the identity row and
        su(pRefCell) = p(pRefCell): returns (a, su)."""
        self._follow(p, a, su)
        p = _host(p)
        a, su = (x.clone() if _is_torch(x) else np.array(x, dtype=np.float64) for x in (a, su))
        self._check(self.lib.fcg_set_reference_pressure(self.h, int(pRefCell), _ptr(p), _ptr(a),
                                                        _ptr(su)), "fcg_set_reference_pressure")
        return a, su

    def correct_velocity_piso(self, dPdxi, apu, apv, apw, u, v, w):
        """PISO :300-304: returns the corrected (u, v, w)."""
        self._follow(dPdxi, apu, apv, apw, u, v, w)
        ins = [_host(x) for x in (dPdxi, apu, apv, apw)]
        outs = [x.clone() if _is_torch(x) else np.array(x, dtype=np.float64) for x in (u, v, w)]
        self._check(self.lib.fcg_correct_velocity_piso(self.h, *[_ptr(x) for x in ins],
                                                       *[_ptr(x) for x in outs]),
                    "fcg_correct_velocity_piso")
        return tuple(outs)

    def grad(self, phi, option: str = "gauss", nigrad: int = 1, dphidxi=None):
        """grad(phi,dPhidxi[,option]) without limiter: returns dPhidxi as (n, 3)."""
        self._follow(phi, dphidxi)
        phi = _host(phi)
        if option == "gauss_corrected" and dphidxi is not None:
            g = dphidxi.clone() if _is_torch(dphidxi) else np.array(dphidxi, dtype=np.float64)
        else:
            g = _like(phi, (self.n, 3))
        self._check(self.lib.fcg_grad(self.h, _ptr(phi), _ptr(g), _GRAD[option], int(nigrad)),
                    "fcg_grad")
        return g

    def grad_lsq_matrix(self):
        d = np.zeros((self.n, 9))
        self._check(self.lib.fcg_grad_lsq_matrix(self.h, _ptr(d)), "fcg_grad_lsq_matrix")
        return d

    def bpres(self, p, dPdxi, istage: int):
        """bpres(p,istage): returns the updated p(numTotal)."""
        self._follow(p, dPdxi)
        p = p.clone() if _is_torch(p) else np.array(p, dtype=np.float64)
        g = _host(dPdxi) if dPdxi is not None else _like(p, (self.n, 3))
        self._check(self.lib.fcg_bpres(self.h, _ptr(p), _ptr(g), int(istage)), "fcg_bpres")
        return p

    # -- a9-a11 ----------------------------------------------------------------------
    def set_solver_options(self, small: float, early_exit: bool):
        self._check(self.lib.fcg_set_solver_options(self.h, float(small), int(bool(early_exit))),
                    "fcg_set_solver_options")

    def trace(self, max_count: int = 1 << 20) -> np.ndarray:
        cnt = C.c_int()
        self._check(self.lib.fcg_get_solver_trace(self.h, None, 0, C.byref(cnt)), "trace")
        m = min(cnt.value, max_count)
        out = np.zeros((max(m, 1), 2))
        self._check(self.lib.fcg_get_solver_trace(self.h, _ptr(out), m, C.byref(cnt)), "trace")
        return out[: cnt.value]

    def _solve(self, fn, name, a, su, fi, sor, nsw, want_res=True, want_trace=False):
        self._follow(a, su, fi)
        a, su = _host(a), _host(su)
        fi = fi.clone() if _is_torch(fi) else np.array(fi, dtype=np.float64)
        res = _like(su, self.n) if want_res else None
        resor = C.c_double(float("nan"))
        rep = _lib.SolveReport()
        self._check(fn(self.h, _ptr(a), _ptr(su), _ptr(fi), _ptr(res), float(sor), int(nsw),
                       C.byref(resor), C.byref(rep)), name)
        r = SolveResult(fi, res, rep.res0, rep.resl, rep.iters, bool(rep.converged),
                        None if rep.iters == 0 else resor.value, rep.l2_rel, rep.seconds)
        if want_trace:
            r.trace = self.trace()
        return r

    def dpcg(self, a, su, fi, sor, nsw, **kw) -> SolveResult:
        """dpcg(fi,ifi) (dpcg.f90:3-154)."""
        return self._solve(self.lib.fcg_dpcg, "fcg_dpcg", a, su, fi, sor, nsw, **kw)

    def dpcg_mixed(self, a, su, fi, sor, nsw, **kw) -> SolveResult:
        """dpcg with FP32 sweeps under FP64 reliable updates (same stop test)."""
        return self._solve(self.lib.fcg_dpcg_mixed, "fcg_dpcg_mixed", a, su, fi, sor, nsw, **kw)

    def bicgstab_multi(self, a, su, fi, sor, nsw):
        """Several systems on this pattern in one solve: a[nsys, nnz], su and fi[nsys, n].
        Returns (fi, list of SolveResult)."""
        self._follow(a, su, fi)
        a, su = _host(a), _host(su)
        fi = fi.clone() if _is_torch(fi) else np.array(fi, dtype=np.float64)
        ns = a.shape[0]
        resor = (C.c_double * ns)(*([float("nan")] * ns))
        reps = (_lib.SolveReport * ns)()
        self._check(self.lib.fcg_bicgstab_multi(self.h, ns, _ptr(a), _ptr(su), _ptr(fi), float(sor),
                                                int(nsw), resor, reps), "fcg_bicgstab_multi")
        out = [SolveResult(fi[k], None, reps[k].res0, reps[k].resl, reps[k].iters,
                           bool(reps[k].converged), None if reps[k].iters == 0 else resor[k],
                           reps[k].l2_rel, reps[k].seconds) for k in range(ns)]
        return fi, out

    def iccg(self, a, su, fi, sor, nsw, **kw) -> SolveResult:
        """iccg(fi,ifi) (iccg.f90:3-177)."""
        return self._solve(self.lib.fcg_iccg, "fcg_iccg", a, su, fi, sor, nsw, **kw)

    def bicgstab(self, a, su, fi, sor, nsw, **kw) -> SolveResult:
        """bicgstab(fi,ifi) (bicgstab.f90:1-231)."""
        return self._solve(self.lib.fcg_bicgstab, "fcg_bicgstab", a, su, fi, sor, nsw, **kw)

    def set_sweep_wait_test(self, polls: int = 0, absent_row: int = 0):
        """Timeout diagnostics of the one-launch DIC/DILU sweeps: every dependency wait
        gives up after `polls` polls and row `absent_row` (1-based) never announces its
        forward result.  (0, 0) restores normal runs."""
        self._check(self.lib.fcg_set_sweep_wait_test(self.h, int(polls), int(absent_row)),
                    "fcg_set_sweep_wait_test")

    def set_aggregation_wait_test(self, polls: int = 0, absent_row: int = 0):
        """Timeout diagnostics of the GPU build of the learned FCG's coarse hierarchy:
        every matching wait gives up after `polls` polls and row `absent_row` (1-based) of
        the first pass never announces its decision, so the build falls back to the host.
        (0, 0) restores normal runs."""
        self._check(self.lib.fcg_set_aggregation_wait_test(self.h, int(polls), int(absent_row)),
                    "fcg_set_aggregation_wait_test")

    def profile_sweeps(self, reps: int = 10) -> dict:
        """Mean milliseconds per kernel unit of the last solve's sweep (changes its state)."""
        ms = (C.c_double * 32)()
        nu = C.c_int()
        self._check(self.lib.fcg_profile_sweeps(self.h, int(reps), ms, 32, C.byref(nu)),
                    "fcg_profile_sweeps")
        out = {}
        for i in range(nu.value):
            name = self.lib.fcg_profile_unit_name(self.h, i).decode()
            key, j = name, 2
            while key in out:
                key, j = f"{name}#{j}", j + 1
            out[key] = ms[i]
        return out

    def spmv(self, a, x, y=None):
        self._follow(a, x, y)
        x = _host(x)
        y = _like(x, self.n) if y is None else y
        self._check(self.lib.fcg_spmv(self.h, _ptr(_host(a)) if a is not None else None, _ptr(x),
                                      _ptr(y)), "fcg_spmv")
        return y


class Batch:
    """An fcg_batch: independent DPCG solves on several contexts in one persistent
    launch (fcg_batch_dpcg).  Arrays may be numpy arrays or CUDA tensors."""

    def __init__(self, contexts):
        self.lib = _lib.load()
        self.contexts = list(contexts)
        arr = (C.c_void_p * len(self.contexts))(*[c.h.value for c in self.contexts])
        h = C.c_void_p()
        rc = self.lib.fcg_batch_create(arr, len(self.contexts), C.byref(h))
        if rc != 0:
            raise _lib.FcgError(rc, "fcg_batch_create", "contexts must be bound, distinct, one device")
        self.h = h

    def _check(self, rc, where):
        if rc != 0:
            raise _lib.FcgError(rc, where, self.lib.fcg_batch_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.fcg_batch_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _ptrs(xs):
        if xs is None:
            return None
        return (C.c_void_p * len(xs))(*[_ptr(x) for x in xs])

    @property
    def params(self):
        spi, bps, mx = C.c_int(), C.c_int(), C.c_int()
        self._check(self.lib.fcg_batch_get_params(self.h, C.byref(spi), C.byref(bps), C.byref(mx)),
                    "fcg_batch_get_params")
        return {"slices_per_item": spi.value, "blocks_per_sm": bps.value,
                "max_blocks_per_sm": mx.value}

    def set_params(self, slices_per_item: int, blocks_per_sm: int):
        self._check(self.lib.fcg_batch_set_params(self.h, int(slices_per_item), int(blocks_per_sm)),
                    "fcg_batch_set_params")

    def set_wait_test(self, polls: int = 0, absent_block: int = -1):
        """Diagnostics: shorten the grid-barrier waits and keep one CTA away from them,
        so that a solve ends with FCG_ERR_TIMEOUT; (0, -1) restores normal runs."""
        self._check(self.lib.fcg_batch_set_wait_test(self.h, int(polls), int(absent_block)),
                    "fcg_batch_set_wait_test")

    def autotune(self, a, su, sweeps: int = 20) -> float:
        for k, c in enumerate(self.contexts):
            c._follow(None if a is None else a[k], su[k])
        a = None if a is None else [_host(x) for x in a]
        su = [_host(x) for x in su]
        best = C.c_double()
        self._check(self.lib.fcg_batch_autotune(self.h, self._ptrs(a), self._ptrs(su), int(sweeps),
                                                C.byref(best)), "fcg_batch_autotune")
        return best.value

    def dpcg(self, a, su, fi, sor, nsw):
        """Returns (fi list, list of SolveResult); `a` may be None (matrices loaded last)."""
        for k, c in enumerate(self.contexts):
            c._follow(None if a is None else a[k], su[k], fi[k])
        a = None if a is None else [_host(x) for x in a]
        su = [_host(x) for x in su]
        fi = [x.clone() if _is_torch(x) else np.array(x, dtype=np.float64) for x in fi]
        ns = len(fi)
        resor = (C.c_double * ns)(*([float("nan")] * ns))
        reps = (_lib.SolveReport * ns)()
        self._check(self.lib.fcg_batch_dpcg(self.h, self._ptrs(a), self._ptrs(su), self._ptrs(fi),
                                            float(sor), int(nsw), resor, reps), "fcg_batch_dpcg")
        out = [SolveResult(fi[k], None, reps[k].res0, reps[k].resl, reps[k].iters,
                           bool(reps[k].converged), None if reps[k].iters == 0 else resor[k],
                           reps[k].l2_rel, reps[k].seconds) for k in range(ns)]
        return fi, out
