"""ctypes binding of libfcgpu.so (the C ABI declared in include/fcgpu.h and
include/fcgpu_meshgen.h).  Loading fails loudly when the library has not been built:
there is no Python or CPU fallback for any compute entry point."""
from __future__ import annotations

import ctypes as C
import os

from . import _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

FCG_OK = 0
FCG_ERR_ARG = -1
FCG_ERR_STATE = -2
FCG_ERR_CUDA = -3
CONV_SCHEMES = {"cds": 0, "cds_corrected": 1, "central": 2, "second_upwind": 3, "muscl": 4,
                "flux_limiter": 5}
LIMITERS = {"smart": 0, "avl": 1, "muscl": 2, "umist": 3, "koren": 4, "charm": 5, "ospre": 6,
            "uds": 7}
FCG_ERR_INDEX = -4
FCG_ERR_PIVOT = -5
FCG_ERR_STALL = -6
FCG_ERR_TIMEOUT = -7
FCG_ERR_UNSUPPORTED = -8
FCG_ERR_NOMEM = -9
FCG_ERR_NONFINITE = -10

FCG_GRAD_GAUSS = 1
FCG_GRAD_GAUSS_CORRECTED = 2
FCG_GRAD_LSQ = 3


class MeshDesc(C.Structure):
    _fields_ = [
        ("numCells", C.c_int), ("numFaces", C.c_int), ("numInnerFaces", C.c_int),
        ("ninl", C.c_int), ("nout", C.c_int), ("nsym", C.c_int), ("nwal", C.c_int),
        ("npru", C.c_int),
        ("iInletFacesStart", C.c_int), ("iOutletFacesStart", C.c_int),
        ("iSymmetryFacesStart", C.c_int), ("iWallFacesStart", C.c_int),
        ("iPressOutletFacesStart", C.c_int), ("noc", C.c_int),
        ("owner", _vp), ("neighbour", _vp),
        ("arx", _vp), ("ary", _vp), ("arz", _vp), ("xf", _vp), ("yf", _vp), ("zf", _vp),
        ("xc", _vp), ("yc", _vp), ("zc", _vp), ("vol", _vp), ("facint", _vp),
        ("ncyc", C.c_int), ("iOCFacesStart", C.c_int), ("ijlFace", _vp), ("ijrFace", _vp),
    ]


class FlowFields(C.Structure):
    _fields_ = [(k, _vp) for k in ("u", "v", "w", "p", "dUdxi", "dVdxi", "dWdxi", "dPdxi",
                                   "apu", "apv", "apw", "den")]


class HbyaParams(C.Structure):
    """fcg_hbya_params: the parameters get_rAU_x_UEqnH reads."""
    _fields_ = [("timestep", C.c_double), ("btime", C.c_double), ("bdf", C.c_int),
                ("cn", C.c_int), ("buoyancy", C.c_int), ("boussinesq", C.c_int),
                ("beta", C.c_double), ("densit", C.c_double), ("tref", C.c_double),
                ("gravx", C.c_double), ("gravy", C.c_double), ("gravz", C.c_double)]


class HbyaFields(C.Structure):
    _fields_ = [(k, _vp) for k in ("den", "t", "uo", "vo", "wo", "uoo", "voo", "woo",
                                   "apu", "apv", "apw")]


class UvwParams(C.Structure):
    """fcg_uvw_params: the parameters calcuvw reads."""
    _fields_ = [("scheme", C.c_int), ("limiter", C.c_int), ("gds", C.c_double),
                ("viscos", C.c_double), ("urfr", C.c_double * 3), ("urfm", C.c_double * 3),
                ("bdf", C.c_int), ("cn", C.c_int), ("timestep", C.c_double),
                ("btime", C.c_double), ("const_mflux", C.c_int), ("gradPcmf", C.c_double),
                ("buoyancy", C.c_int), ("boussinesq", C.c_int), ("beta", C.c_double),
                ("densit", C.c_double), ("tref", C.c_double), ("gravx", C.c_double),
                ("gravy", C.c_double), ("gravz", C.c_double)]


UVW_FIELDS = ("u", "v", "w", "p", "vis", "den", "t", "uo", "vo", "wo", "uoo", "voo", "woo",
              "dUdxi", "dVdxi", "dWdxi", "dPdxi", "flmass", "fmi", "fmo")


class UvwFields(C.Structure):
    _fields_ = [(k, _vp) for k in UVW_FIELDS]


class Multilevel(C.Structure):
    """fcg_lp_multilevel: options of the learned FCG's coarse-grid correction."""
    _fields_ = [("enabled", C.c_int), ("smoother", C.c_int), ("sweeps", C.c_int),
                ("max_levels", C.c_int), ("dense_max", C.c_int), ("alpha", C.c_double),
                ("omega", C.c_double), ("smoothed", C.c_int)]


SMOOTH_NETWORK, SMOOTH_JACOBI, MAX_LEVELS = 0, 1, 16


class SolveReport(C.Structure):
    _fields_ = [("res0", C.c_double), ("resl", C.c_double), ("iters", C.c_int),
                ("converged", C.c_int), ("l2_rel", C.c_double), ("seconds", C.c_double)]


_CTX = C.c_void_p
_LP = C.c_void_p
_BATCH = C.c_void_p

# name -> (restype, argtypes)
_PROTOS = {
    "fcg_abi_version": (C.c_int, []),
    "fcg_status_string": (C.c_char_p, [C.c_int]),
    "fcg_last_error": (C.c_char_p, [_CTX]),
    "fcg_create": (C.c_int, [C.POINTER(_CTX), C.c_int]),
    "fcg_destroy": (C.c_int, [_CTX]),
    "fcg_set_stream": (C.c_int, [_CTX, _vp]),
    "fcg_synchronize": (C.c_int, [_CTX]),
    "fcg_bind_mesh": (C.c_int, [_CTX, C.POINTER(MeshDesc)]),
    "fcg_mesh_sizes": (C.c_int, [_CTX, _ip, _ip, _ip, C.POINTER(C.c_longlong), _ip]),
    "fcg_create_csr": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, _vp]),
    "fcg_csr_build": (C.c_int, [C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fcg_topology_digest": (C.c_int, [_CTX, C.POINTER(C.c_ulonglong)]),
    "fcg_csr_build_gpu": (C.c_int, [_CTX, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fcg_mesh_geometry_gpu": (C.c_int, [_CTX, C.c_int, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int,
                                        _vp, _vp, _vp, _vp] + [_vp] * 11),
    "fcg_laplacian": (C.c_int, [_CTX, _vp, _vp, _vp, _vp]),
    "fcg_facefluxmass": (C.c_int, [_CTX, C.POINTER(FlowFields), _vp, _vp, _vp]),
    "fcg_fluxmc": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, _vp]),
    "fcg_flux_correct": (C.c_int, [_CTX, _vp, _vp, _vp]),
    "fcg_correct_bc_velocity": (C.c_int, [_CTX, _vp, C.c_double, _vp, _vp, _vp, _vp]),
    "fcg_continuity_errors": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, _dp, _dp]),
    "fcg_correct_fields": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, _vp, C.c_double, C.c_int, _vp,
                                     _vp, _vp, _vp]),
    "fcg_set_sweep_wait_test": (C.c_int, [_CTX, C.c_int, C.c_int]),
    "fcg_set_aggregation_wait_test": (C.c_int, [_CTX, C.c_int, C.c_int]),
    "fcg_calcuvw": (C.c_int, [_CTX, C.POINTER(UvwParams), C.POINTER(UvwFields), _vp, _vp, _vp,
                              _vp]),
    "fcg_piso_hbya": (C.c_int, [_CTX, C.POINTER(HbyaParams), C.POINTER(HbyaFields), _vp, _vp,
                                _vp, _vp, _vp, _vp, _vp]),
    "fcg_facefluxmass_piso": (C.c_int, [_CTX, C.POINTER(FlowFields), _vp, _vp, _vp]),
    "fcg_adjust_mass_flow": (C.c_int, [_CTX, _vp, C.c_double, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fcg_set_reference_pressure": (C.c_int, [_CTX, C.c_int, _vp, _vp, _vp]),
    "fcg_correct_velocity_piso": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fcg_grad": (C.c_int, [_CTX, _vp, _vp, C.c_int, C.c_int]),
    "fcg_grad_lsq_matrix": (C.c_int, [_CTX, _vp]),
    "fcg_bpres": (C.c_int, [_CTX, _vp, _vp, C.c_int]),
    "fcg_dpcg": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, C.c_double, C.c_int, _dp,
                           C.POINTER(SolveReport)]),
    "fcg_iccg": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, C.c_double, C.c_int, _dp,
                           C.POINTER(SolveReport)]),
    "fcg_bicgstab": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, C.c_double, C.c_int, _dp,
                               C.POINTER(SolveReport)]),
    "fcg_dpcg_mixed": (C.c_int, [_CTX, _vp, _vp, _vp, _vp, C.c_double, C.c_int, _dp,
                                 C.POINTER(SolveReport)]),
    "fcg_bicgstab_multi": (C.c_int, [_CTX, C.c_int, _vp, _vp, _vp, C.c_double, C.c_int, _dp,
                                     C.POINTER(SolveReport)]),
    "fcg_set_solver_options": (C.c_int, [_CTX, C.c_double, C.c_int]),
    "fcg_get_solver_trace": (C.c_int, [_CTX, _vp, C.c_int, _ip]),
    "fcg_spmv": (C.c_int, [_CTX, _vp, _vp, _vp]),
    "fcg_profile_sweeps": (C.c_int, [_CTX, C.c_int, _dp, C.c_int, _ip]),
    "fcg_profile_unit_name": (C.c_char_p, [_CTX, C.c_int]),
    "fcg_dpcg_noalloc": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_double,
                                   C.c_int, _dp, C.POINTER(SolveReport), _vp]),
    # batched DPCG
    "fcg_batch_create": (C.c_int, [_vp, C.c_int, C.POINTER(_BATCH)]),
    "fcg_batch_destroy": (C.c_int, [_BATCH]),
    "fcg_batch_last_error": (C.c_char_p, [_BATCH]),
    "fcg_batch_set_params": (C.c_int, [_BATCH, C.c_int, C.c_int]),
    "fcg_batch_get_params": (C.c_int, [_BATCH, _ip, _ip, _ip]),
    "fcg_batch_dpcg": (C.c_int, [_BATCH, _vp, _vp, _vp, C.c_double, C.c_int, _dp,
                                 C.POINTER(SolveReport)]),
    "fcg_batch_autotune": (C.c_int, [_BATCH, _vp, _vp, C.c_int, _dp]),
    "fcg_batch_set_wait_test": (C.c_int, [_BATCH, C.c_longlong, C.c_int]),
    # learned preconditioner and flexible CG
    "fcg_lp_create": (C.c_int, [C.c_int, C.c_ulonglong, C.POINTER(_LP)]),
    "fcg_lp_destroy": (C.c_int, [_LP]),
    "fcg_lp_last_error": (C.c_char_p, [_LP]),
    "fcg_lp_get_weights": (C.c_int, [_LP, _vp, C.c_int]),
    "fcg_lp_set_weights": (C.c_int, [_LP, _vp, C.c_int]),
    "fcg_lp_save": (C.c_int, [_LP, C.c_char_p]),
    "fcg_lp_load": (C.c_int, [_LP, C.c_char_p]),
    "fcg_lp_set_matrix": (C.c_int, [_LP, _CTX, _vp]),
    "fcg_lp_features": (C.c_int, [_LP, _CTX, _vp]),
    "fcg_lp_apply": (C.c_int, [_LP, _CTX, _vp, _vp]),
    "fcg_lp_loss_grad": (C.c_int, [_LP, _CTX, _vp, _vp, C.POINTER(C.c_float), _vp]),
    "fcg_lp_train_step": (C.c_int, [_LP, _CTX, _vp, _vp, C.c_float, C.POINTER(C.c_float)]),
    "fcg_lp_set_loss": (C.c_int, [_LP, C.c_int]),
    "fcg_lp_last_solve_stats": (C.c_int, [_LP, _ip, _ip]),
    "fcg_lp_profile": (C.c_int, [_LP, _CTX, _vp, C.c_int, _dp, C.c_int, _ip]),
    "fcg_lp_layer_form": (C.c_int, [_LP, _CTX, _ip, _ip]),
    "fcg_lp_set_fcg_options": (C.c_int, [_LP, C.c_int, C.c_int, C.c_int, C.c_double]),
    "fcg_lp_set_multilevel": (C.c_int, [_LP, C.POINTER(Multilevel)]),
    "fcg_lp_get_multilevel": (C.c_int, [_LP, C.POINTER(Multilevel)]),
    "fcg_lp_hierarchy_info": (C.c_int, [_LP, _CTX, _ip, _ip, C.POINTER(C.c_longlong), _dp]),
    "fcg_lp_hierarchy_built_on": (C.c_int, [_LP, _CTX, _ip]),
    "fcg_lp_hierarchy_level": (C.c_int, [_LP, _CTX, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fcg_lp_precondition": (C.c_int, [_LP, _CTX, _vp, _vp]),
    "fcg_lp_coarse_correct": (C.c_int, [_LP, _CTX, _vp, _vp, _vp]),
    "fcg_aggregate": (C.c_int, [C.c_int, _vp, _vp, _vp, C.c_int, C.c_int, _vp, _ip]),
    "fcg_smoothed_level": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, C.c_int, C.c_double,
                                     C.POINTER(C.c_longlong), _vp, _vp, _vp]),
    "fcg_fcg_learned": (C.c_int, [_CTX, _LP, _vp, _vp, _vp, _vp, C.c_double, C.c_int, _dp,
                                  C.POINTER(SolveReport), _ip, _ip]),
    # synthetic inputs (include/fcgpu_meshgen.h)
    "fcg_hex_mesh_sizes": (C.c_int, [C.c_int, _ip, _ip, _ip, _ip]),
    "fcg_hex_mesh_build": (C.c_int, [C.c_int, C.c_double, C.c_ulonglong, _vp, _vp, _vp, _vp,
                                     _vp, _vp, _vp, _vp]),
    "fcg_mesh_geometry": (C.c_int, [C.c_int, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp,
                                    _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    _vp, _vp, _vp]),
    "fcg_uniform_fill": (C.c_int, [C.c_ulonglong, C.c_ulonglong, C.c_longlong, C.c_double,
                                   C.c_double, _vp]),
}

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads libfcgpu.so (building it first if asked).  Raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libfcgpu.so is not built ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_PROTOS)


class FcgError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        lib = load(build_if_missing=False)
        name = lib.fcg_status_string(status).decode()
        super().__init__(f"{where}: status {status} ({name}){': ' + detail if detail else ''}")
        self.status = status
