"""The C ABI: libfcgpu.so loads and exports every function include/*.h declares; without
a GPU the compute entry points refuse to run (there is no CPU fallback)."""
import ctypes as C
import glob
import os
import re

import pytest

from freecappuccino_gb300 import _lib
from tests.conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(fcg_\w+)\s*\(", text))
    return sorted(names)


def test_headers_declare_the_path():
    names = declared_functions()
    for must in ("fcg_bind_mesh", "fcg_create_csr", "fcg_laplacian", "fcg_facefluxmass",
                 "fcg_fluxmc", "fcg_grad", "fcg_bpres", "fcg_dpcg", "fcg_iccg", "fcg_bicgstab"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(_lib.load().__getattribute__("_name"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding knows every one of them
    assert set(declared_functions()) <= set(_lib.exported_symbols())


def test_abi_version_and_status_strings():
    lib = _lib.load()
    assert lib.fcg_abi_version() == 2
    assert lib.fcg_status_string(0) == b"ok"
    assert lib.fcg_status_string(_lib.FCG_ERR_PIVOT) == b"zero or non-finite pivot"


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU refusal")
def test_no_cpu_fallback_without_gpu():
    lib = _lib.load()
    h = C.c_void_p()
    assert lib.fcg_create(C.byref(h), 0) == _lib.FCG_ERR_CUDA
    assert not h.value


def test_null_context_is_rejected():
    lib = _lib.load()
    assert lib.fcg_dpcg(None, None, None, None, None, 1e-8, 10, None, None) == _lib.FCG_ERR_ARG
    assert lib.fcg_laplacian(None, None, None, None, None) == _lib.FCG_ERR_ARG


def test_ctypes_structs_match_the_header():
    """Member order and types of the ctypes mirrors of the header's option structs."""
    import ctypes as C
    import os
    import re

    from freecappuccino_gb300 import _lib

    txt = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "include", "fcgpu.h")).read()
    body = re.search(r"typedef struct fcg_lp_multilevel \{(.*?)\} fcg_lp_multilevel;", txt, re.S)
    assert body
    fields = []
    for line in body.group(1).splitlines():
        m = re.match(r"\s*(int|double)\s+(\w+);", line)
        if m:
            fields.append((m.group(2), C.c_int if m.group(1) == "int" else C.c_double))
    assert [(n, t) for n, t in _lib.Multilevel._fields_] == fields

