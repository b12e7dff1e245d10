"""GB300-native (sm_103a) pressure-correction path of freeCappuccino.

libfcgpu.so (C ABI: include/fcgpu.h) holds the face-loop assembly, gradients and the
DPCG / ICCG / BiCGStab solvers; this package builds it in-tree and binds it.
"""
from . import _build, _lib  # noqa: F401
from .mesh import Mesh, hex_mesh, polymesh_mesh, uniform  # noqa: F401
from .polymesh import read_polymesh, write_polymesh  # noqa: F401
from .pressure import Batch, Context, SolveResult, solver_log  # noqa: F401

__all__ = ["Mesh", "hex_mesh", "polymesh_mesh", "read_polymesh", "write_polymesh", "uniform",
           "Batch", "Context", "SolveResult", "solver_log"]
