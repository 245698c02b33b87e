"""GB300 (sm_103a) implementation of Curvami's per-Gauss-point hot path.

Stage A (RKPM shape functions with crease visibility) and stage B (Kirchhoff-Love
residual + tangent with the elastic hinge, scattered into the CSC stiffness) run as
hand-written CUDA kernels in ``libcurvami_gb300.so`` behind the C ABI of
``include/curvami_gb300.h``; this package is the host-side mirror of the reference's
interface over that ABI (ctypes). There is no CPU fallback.
"""
from ._lib import (CGBError, DETERMINISTIC, HINGE, HINGE_EXACT, MIXED, TANGENT,  # noqa: F401
                   TANGENT_CORES, TANGENT_TENSOR, load_library, LIB_PATH)
from .api import (AssemblyGraph, Context, NonLinearAssembler, PlateBatch, PlateModel, ShapeSet,  # noqa: F401
                  abd_isotropic, abd_laminate, concat_shapes, shape_from_host, shape_functions)
from . import synth  # noqa: F401
