"""ctypes binding of ``liblettuce_gb300.so`` (include/lettuce_gb300.h).

The library is loaded from the package's ``_build`` folder. There is no
fallback: if it has not been built, or no CUDA device is present when a
kernel is launched, the call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

ABI_VERSION = 5
LINK_FORCE_BLOCK = 256  # LGB_LINK_FORCE_BLOCK
MAX_SUBSTEPS = 8
REDUCE_FIELDS = 5

# enums of include/lettuce_gb300.h
D1Q3, D2Q9, D3Q15, D3Q19, D3Q27 = 1, 2, 3, 4, 5
F64, F32, F16_SHIFTED, BF16_SHIFTED = 0, 1, 2, 3
NO_COLLISION, BGK, TRT, KBC, REGULARIZED, SMAGORINSKY, MRT = 0, 1, 2, 3, 4, 5, 6
MRT_EQ_GENERIC, MRT_EQ_DELLAR, MRT_EQ_LALLEMAND, MRT_EQ_HERMITE = 0, 1, 2, 3
FORCE_NONE, FORCE_GUO, FORCE_SHAN_CHEN = 0, 1, 2
SUB_COLLISION, SUB_BOUNCE_BACK, SUB_EQUILIBRIUM_PU, SUB_ANTI_BOUNCE_BACK, SUB_NONE = 0, 1, 2, 3, 4
SUB_EQUILIBRIUM_OUTLET_P, SUB_PARTIALLY_SATURATED = 5, 6
PULL, PUSH, LOCAL, AA_EVEN, AA_ODD, STREAM_ONLY, AA_UNPACK = 0, 1, 2, 3, 4, 5, 6
FLAG_INDEX_MASK, FLAG_LINKS, FLAG_PUSH_GUARD, FLAG_NO_STREAM = 0x1F, 0x20, 0x40, 0x80
OPT_ONE_CELL, OPT_PUSH_GUARD = 1, 2

EXPORTED = ["lgb_abi_version", "lgb_last_error", "lgb_step", "lgb_moments",
            "lgb_reduce_scratch_bytes", "lgb_reduce", "lgb_reduce_static", "lgb_convert",
            "lgb_batch_plan", "lgb_batched_step", "lgb_adjoint_step", "lgb_host_pointer",
            "lgb_equilibrium", "lgb_init_fneq", "lgb_enstrophy"]
REDUCE_STATIC_SCRATCH_BYTES = 48640


class Substep(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32),
                ("axis", ctypes.c_int32),
                ("sign", ctypes.c_int32),
                ("reserved", ctypes.c_int32),
                ("rho", ctypes.c_void_p),
                ("u", ctypes.c_void_p),
                ("rho_stride", ctypes.c_int64 * 3),
                ("u_stride", ctypes.c_int64 * 4),
                ("param", ctypes.c_double * 2)]


class StepDesc(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_int32),
                ("stencil", ctypes.c_int32),
                ("storage", ctypes.c_int32),
                ("collision", ctypes.c_int32),
                ("pattern", ctypes.c_int32),
                ("res", ctypes.c_int32 * 3),
                ("tau", ctypes.c_double),
                ("tau_minus", ctypes.c_double),
                ("f_in", ctypes.c_void_p),
                ("f_out", ctypes.c_void_p),
                ("flags", ctypes.c_void_p),
                ("no_stream_bits", ctypes.c_void_p),
                ("n_sub", ctypes.c_int32),
                ("collision_index", ctypes.c_int32),
                ("sub", Substep * MAX_SUBSTEPS),
                ("status", ctypes.c_void_p),
                ("options", ctypes.c_int32),
                ("force", ctypes.c_int32),
                ("force_tau", ctypes.c_double),
                ("accel", ctypes.c_double * 3),
                ("smagorinsky_constant", ctypes.c_double),
                ("mrt_equilibrium", ctypes.c_int32),
                ("reserved2", ctypes.c_int32),
                ("mrt_tables", ctypes.c_void_p),
                ("link_bits", ctypes.c_void_p),
                ("link_base", ctypes.c_void_p),
                ("link_pairs", ctypes.c_void_p),
                ("link_d", ctypes.c_void_p),
                ("link_val", ctypes.c_void_p),
                ("n_links", ctypes.c_int64),
                ("force_links", ctypes.c_void_p),
                ("n_force_links", ctypes.c_int64),
                ("force_out", ctypes.c_void_p),
                ("force_scratch", ctypes.c_void_p)]


class LibraryError(RuntimeError):
    pass


_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def load():
    """The loaded library; raises if it was not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise LibraryError(
                f"{path} is missing: the CUDA library of lettuce_gb300 is not "
                "built (run `python -m lettuce_gb300.build`). There is no "
                "fallback implementation.")
        L = ctypes.CDLL(path)
        P, I32, I64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
        L.lgb_abi_version.restype = ctypes.c_int
        L.lgb_last_error.restype = ctypes.c_char_p
        L.lgb_step.argtypes = [ctypes.POINTER(StepDesc), P]
        L.lgb_step.restype = ctypes.c_int
        L.lgb_moments.argtypes = [I32, I32, P, P, I32, P, P, P]
        L.lgb_moments.restype = ctypes.c_int
        L.lgb_reduce_scratch_bytes.restype = I64
        L.lgb_reduce.argtypes = [I32, I32, P, P, I32, P, P, P, P, P, P]
        L.lgb_reduce.restype = ctypes.c_int
        L.lgb_reduce_static.argtypes = [I32, I32, P, P, I32, P, P, P, P, P]
        L.lgb_reduce_static.restype = ctypes.c_int
        L.lgb_convert.argtypes = [I32, I32, P, I32, P, I64, P]
        L.lgb_adjoint_step.argtypes = [I32, I32, P, ctypes.c_double, P, P, P, P]
        L.lgb_adjoint_step.restype = ctypes.c_int
        L.lgb_convert.restype = ctypes.c_int
        L.lgb_host_pointer.argtypes = [P, ctypes.POINTER(ctypes.c_void_p)]
        L.lgb_host_pointer.restype = ctypes.c_int
        L.lgb_equilibrium.argtypes = [I32, I32, P, P, P, P, P, P, P, P, P]
        L.lgb_equilibrium.restype = ctypes.c_int
        L.lgb_init_fneq.argtypes = [I32, I32, P, P, P, ctypes.c_double, P, P]
        L.lgb_init_fneq.restype = ctypes.c_int
        L.lgb_enstrophy.argtypes = [I32, I32, P, P, P, P, P]
        L.lgb_enstrophy.restype = ctypes.c_int
        if L.lgb_abi_version() != ABI_VERSION:
            raise LibraryError(f"{path} has ABI version {L.lgb_abi_version()}, "
                               f"expected {ABI_VERSION}; rebuild it")
        _lib = L
        return L


def check(rc: int, what: str):
    if rc != 0:
        msg = load().lgb_last_error().decode(errors="replace")
        raise LibraryError(f"{what}: {msg}")


def i32x3(values):
    values = list(values) + [1] * (3 - len(values))
    return (ctypes.c_int32 * 3)(*values)
