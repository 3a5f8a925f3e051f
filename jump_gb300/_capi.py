"""ctypes mirror of include/jump_mpm.h and the loader of the CUDA library.

The structures here are the boundary a Julia ``ccall`` shim would fill from
jump's Grid/Solid/Material objects (SolveExplicitSolidMechanics2D.jl:335,
SolveExplicitSolidMechanics3D.jl:230).  The product library is
``jump_gb300/lib/libjumpmpm.so``; importing this module never falls back to a
CPU implementation: when the library is missing, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

ABI_VERSION = 10  # JUMP_MPM_ABI_VERSION of the structures below

MPM_OK = 0
MPM_ERR_ARG = 1
MPM_ERR_CUDA = 2
MPM_ERR_NEGATIVE_J = 3
MPM_ERR_NONFINITE = 4
MPM_ERR_OUT_OF_GRID = 5
MPM_ERR_UNSUPPORTED = 7
MPM_ERR_SOLVER = 8

ERR_NAMES = {
    MPM_ERR_ARG: "MPM_ERR_ARG",
    MPM_ERR_CUDA: "MPM_ERR_CUDA",
    MPM_ERR_NEGATIVE_J: "MPM_ERR_NEGATIVE_J",
    MPM_ERR_NONFINITE: "MPM_ERR_NONFINITE",
    MPM_ERR_OUT_OF_GRID: "MPM_ERR_OUT_OF_GRID",
    MPM_ERR_UNSUPPORTED: "MPM_ERR_UNSUPPORTED",
    MPM_ERR_SOLVER: "MPM_ERR_SOLVER",
}

MPM_MAT_ELASTIC = 0
MPM_MAT_NEOHOOKEAN = 1
MPM_MAT_J2 = 2
MPM_MAT_JOHNSON_COOK = 3
MPM_MAT_VOCE = 4
MPM_MAT_JOHNSON_COOK_DAMAGE = 5
MPM_MAT_RIGID = 6
MPM_MAX_RIGID_BODIES = 32

MPM_PREC_F64 = 0
MPM_PREC_F32 = 1
MPM_PREC_DW = 2

# double-word operations of mpm_probe_dw
MPM_DW_OP_FROM_F64 = 0
MPM_DW_OP_ADD = 1
MPM_DW_OP_SUB = 2
MPM_DW_OP_MUL = 3
MPM_DW_OP_MUL_FLOAT = 4
MPM_DW_OP_FMA = 5
MPM_DW_OP_SQR = 6
MPM_DW_OP_SQRT = 7
MPM_DW_OP_RECIP = 8
MPM_DW_OP_ONE_MINUS = 9
MPM_DW_OP_TO_F64 = 10

MPM_ALG_USL = 0
MPM_ALG_MUSL = 1

MPM_BASIS_LINEAR = 0
MPM_BASIS_QUAD_BSPLINE = 1
MPM_BASIS_CUBIC_BSPLINE = 2

MPM_TUNE_CANDIDATES = 49
MPM_P2G_ATOMIC = 0
MPM_P2G_WARP = 1
MPM_P2G_TILE = 2
MPM_P2G_TILE_WARP = 3
MPM_P2G_FUSED = 4
MPM_FUSED_MAX_PARTICLES = 2048

MPM_BATCH_PERSISTENT = 0
MPM_BATCH_WIDE = 1
MPM_BATCH_MAX_BODIES = 4

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)


class GridDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("reserved", C.c_int32),
        ("xmin", C.c_double * 3),
        ("xmax", C.c_double * 3),
        ("nodes", C.c_int64 * 3),
        ("fixed_nodes", _ip),
    ]


class MaterialDesc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("reserved", C.c_int32),
        ("E", C.c_double),
        ("nu", C.c_double),
        ("density", C.c_double),
        ("fy", C.c_double),
        ("k1", C.c_double),
        ("A", C.c_double),
        ("B", C.c_double),
        ("C", C.c_double),
        ("n", C.c_double),
        ("epsdot0", C.c_double),
        ("cellsize", C.c_double),
        ("m", C.c_double),
        ("chi", C.c_double),
        ("Cp", C.c_double),
        ("d1", C.c_double),
        ("d2", C.c_double),
        ("d3", C.c_double),
        ("d4", C.c_double),
        ("d5", C.c_double),
        ("depsdot0", C.c_double),
        ("Tr", C.c_double),
        ("Tm", C.c_double),
        ("v_rigid", C.c_double * 3),
        ("fixed", C.c_int32),
        ("reserved2", C.c_int32),
    ]


class BodyDesc(C.Structure):
    _fields_ = [
        ("count", C.c_int64),
        ("mat", MaterialDesc),
        ("pos", _dp),
        ("velocity", _dp),
        ("mass", _dp),
        ("volume", _dp),
        ("volume_initial", _dp),
        ("F", _dp),
        ("strain", _dp),
        ("stress", _dp),
        ("alpha", _dp),
        ("pstrain", _dp),
        ("youngs", _dp),
        ("alphadot", _dp),
        ("damage_init", _dp),
        ("damage", _dp),
        ("temperature", _dp),
        ("vmstr", _dp),
    ]


class BodyView(C.Structure):
    _fields_ = [
        ("pos", _dp),
        ("velocity", _dp),
        ("volume", _dp),
        ("F", _dp),
        ("strain", _dp),
        ("stress", _dp),
        ("alpha", _dp),
        ("pstrain", _dp),
        ("vmstr", _dp),
        ("alphadot", _dp),
        ("damage_init", _dp),
        ("damage", _dp),
        ("temperature", _dp),
    ]


class Params(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("tolerance", C.c_double),
        ("body_force", C.c_double * 3),
        ("precision", C.c_int32),
        ("contact", C.c_int32),
        ("friction", C.c_double),
        ("sort_interval", C.c_int32),
        ("flags", C.c_int32),
        ("algorithm", C.c_int32),
        ("basis", C.c_int32),
        ("alpha", C.c_double),
    ]


def dptr(a: np.ndarray | None):
    """Pointer to a C-contiguous float64 array (None -> NULL)."""
    if a is None:
        return _dp()
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "need C-contiguous float64"
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray | None):
    if a is None:
        return _ip()
    assert a.dtype == np.int64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ip)


HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libjumpmpm.so")

# Every symbol include/jump_mpm.h declares, with its ctypes signature.
SIGNATURES = {
    "mpm_abi_version": (C.c_int, []),
    "mpm_last_error": (C.c_char_p, []),
    "mpm_create": (C.c_int, [C.POINTER(GridDesc), C.POINTER(BodyDesc), C.c_int32,
                             C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "mpm_step": (C.c_int, [C.c_void_p, C.c_int64, _dp]),
    "mpm_step_energies": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, _dp, C.c_void_p]),
    "mpm_set_launch": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "mpm_probe_rates": (C.c_int, [_dp, _dp, _dp]),
    "mpm_probe_dw": (C.c_int, [C.c_int32, C.c_int64, _dp, _dp, _dp, _dp]),
    "mpm_get_launch": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "mpm_tune": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                           C.POINTER(C.c_int32), _dp, _dp]),
    "mpm_download": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(BodyView)]),
    "mpm_download_grid": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "mpm_energies": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "mpm_save": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_size_t)]),
    "mpm_load": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "mpm_last_step_ms": (C.c_int, [C.c_void_p, _dp]),
    "mpm_profile_stages": (C.c_int, [C.c_void_p, C.c_int64, _dp]),
    "mpm_destroy": (C.c_int, [C.c_void_p]),
    "mpm_energies_static": (C.c_int, [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]),
    "mpm_fwd_checkpointed": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32]),
    "mpm_bwd": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp]),
    "mpm_batch_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "mpm_batch_step": (C.c_int, [C.c_void_p, C.c_int64]),
    "mpm_batch_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "mpm_batch_download": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "mpm_batch_energies": (C.c_int, [C.c_void_p, _dp]),
    "mpm_batch_set_launch": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "mpm_batch_tune": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _dp]),
    "mpm_batch_jvp": (C.c_int, [C.c_void_p, C.c_int64, _dp, _dp]),
    "mpm_batch_set_strategy": (C.c_int, [C.c_void_p, C.c_int32]),
    "mpm_batch_strategy": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "mpm_batch_last_ms": (C.c_int, [C.c_void_p, _dp]),
    "mpm_batch_destroy": (C.c_int, [C.c_void_p]),
}


class InstanceDesc(C.Structure):
    _fields_ = [
        ("grid", GridDesc),
        ("bodies", C.POINTER(BodyDesc)),
        ("nbodies", C.c_int32),
        ("contact", C.c_int32),
        ("dt", C.c_double),
        ("tolerance", C.c_double),
        ("body_force", C.c_double * 3),
        ("friction", C.c_double),
    ]

STAGES = ("reset", "p2g", "grid", "g2p")

_lib = None
_lock = threading.Lock()


class MPMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


def load_library(path: str):
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def lib():
    """The CUDA library; raises if it has not been built (no CPU fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                    "g.build()\"` (the CUDA path has no CPU fallback)")
            L = load_library(LIB_PATH)
            if L.mpm_abi_version() != ABI_VERSION:
                raise RuntimeError(f"{LIB_PATH} has ABI version {L.mpm_abi_version()}, these bindings "
                                   f"{ABI_VERSION}: rebuild it")
            _lib = L
        return _lib


def check(code: int, L=None):
    if code != MPM_OK:
        L = L or lib()
        raise MPMError(code, L.mpm_last_error().decode())
