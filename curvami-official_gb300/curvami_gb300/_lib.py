"""ctypes declarations of the C ABI in include/curvami_gb300.h.

The shared library is built in-tree (``build.py``) and loaded from this directory;
there is no CPU fallback — a missing library or GPU raises."""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcurvami_gb300.so")

CGB_OK = 0
CGB_ERR_INVALID = 1
CGB_ERR_CUDA = 2
CGB_ERR_SINGULAR = 3
CGB_ERR_PIVOT = 4
CGB_ERR_MAPPING = 5
CGB_ERR_CAPACITY = 6
CGB_ERR_DEVICE = 7

TANGENT = 0x1
HINGE = 0x2
MIXED = 0x4
DETERMINISTIC = 0x8
HINGE_EXACT = 0x10

# Every symbol the header declares, with (restype, argtypes).
vp, i32, i64, dbl, cp = C.c_void_p, C.c_int, C.c_int64, C.c_double, C.c_char_p
SIGNATURES = {
    "cgb_create": (i32, [i32, C.POINTER(vp)]),
    "cgb_destroy": (i32, [vp]),
    "cgb_last_error": (cp, [vp]),
    "cgb_set_stream": (i32, [vp, vp]),
    "cgb_synchronize": (i32, [vp]),
    "cgb_set_nodes": (i32, [vp, vp, i32]),
    "cgb_set_natural_curvature": (i32, [vp, vp]),
    "cgb_shape_build": (i32, [vp, vp, i32, vp, vp, i32, C.POINTER(vp)]),
    "cgb_shape_rebuild": (i32, [vp, vp, i32]),
    "cgb_shape_from_host": (i32, [vp, i32, vp, vp, vp, vp, vp, C.POINTER(vp)]),
    "cgb_shape_size": (i32, [vp, C.POINTER(i32), C.POINTER(i64), C.POINTER(i32)]),
    "cgb_shape_download": (i32, [vp, vp, vp, vp, vp, vp, vp]),
    "cgb_shape_device": (i32, [vp, vp, vp, vp, vp, vp]),
    "cgb_shape_destroy": (i32, [vp]),
    "cgb_assembler_create": (i32, [vp, vp, vp, vp, i32, C.POINTER(vp)]),
    "cgb_assembler_destroy": (i32, [vp]),
    "cgb_assembler_pattern": (i32, [vp, C.POINTER(i32), C.POINTER(i64)]),
    "cgb_assembler_download_pattern": (i32, [vp, vp, vp]),
    "cgb_assembler_download_map": (i32, [vp, vp, i64]),
    "cgb_assembler_stats": (i32, [vp, vp]),
    "cgb_assembler_tensor_stats": (i32, [vp, vp]),
    "cgb_shape_concat": (i32, [vp, vp, vp, i32, vp]),
    "cgb_assembler_set_tuning": (i32, [vp, vp]),
    "cgb_graph_create": (i32, [vp, vp, vp, vp, i32, vp]),
    "cgb_graph_launch": (i32, [vp]),
    "cgb_graph_destroy": (i32, [vp]),
    "cgb_test_stage_timeout": (i32, [vp, i32]),
    "cgb_assembler_set_fold_state": (i32, [vp, i32, dbl, vp, vp]),
    "cgb_set_material": (i32, [vp, vp, vp, vp]),
    "cgb_assemble": (i32, [vp, vp, vp, vp, i32]),
    "cgb_assemble_device": (i32, [vp, vp, vp, vp, i32]),
    "cgb_energies": (i32, [vp, vp, C.POINTER(dbl), C.POINTER(dbl), C.POINTER(dbl)]),
    "cgb_assemble_face_noalloc": (i32, [vp, vp, vp, vp, vp]),
    "cgb_point_state": (i32, [vp, vp, vp, vp, vp, vp, vp]),
    "cgb_point_state_device": (i32, [vp, vp, vp, vp, vp, vp, vp]),
    "cgb_profile_enable": (i32, [vp, i32]),
    "cgb_profile_read": (i32, [vp, vp, vp, i32]),
}

PHASES = ("h2d", "zero", "face", "hinge", "reduce", "d2h", "tangent", "frnn", "crease", "rkpm")


class Crease(C.Structure):
    _fields_ = [("xy", vp), ("n_vertices", i32), ("extend_start", i32), ("extend_end", i32),
                ("is_closed", i32)]


class ShapeParams(C.Structure):
    _fields_ = [("rho", dbl), ("rho_node", vp), ("order", i32), ("kernel", i32), ("precision", i32)]


TANGENT_CORES = 0
TANGENT_TENSOR = 1


class NaturalCurvature(C.Structure):
    """cgb_natural_curvature: the band of Kinematics::NaturalCurvature (theta0 in radians,
    sign -1 mountain / +1 valley)."""
    _fields_ = [("active", i32), ("x0", dbl), ("width", dbl), ("theta0", dbl), ("sign", dbl)]


class Tuning(C.Structure):
    _fields_ = [("n_chunks", i32), ("residual_threads", i32), ("tangent_ctas_per_sm", i32),
                ("tangent_kind", i32)]


class Fold(C.Structure):
    _fields_ = [("left", vp), ("right", vp), ("weight", vp), ("tangent", vp), ("Kt", dbl),
                ("theta0", dbl), ("theta0_gp", vp), ("active", vp)]


NOALLOC_MAX_BLOCKS = 699050
POINT_STATE_COLS = 33


class FaceProblem(C.Structure):
    """cgb_face_problem: device pointers of the allocation-free face assembly."""
    _fields_ = [("n_gp", i32), ("n_nodes", i32), ("max_neighbours", i32), ("nnz", i64),
                ("nbr_ptr", vp), ("nbr_idx", vp), ("dpsi", vp), ("ddpsi", vp), ("weight", vp),
                ("map_ptr", vp), ("csr_map", vp), ("outer", vp),
                ("A", dbl * 9), ("B", dbl * 9), ("D", dbl * 9)]


class CGBError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


_lock = threading.Lock()
_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load the in-tree library (build it first with build.py / __graft_entry__.build)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise CGBError(CGB_ERR_INVALID,
                           f"{p} is missing: build it with curvami-official_gb300/build.py")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib
