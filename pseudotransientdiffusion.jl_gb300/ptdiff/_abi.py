"""ctypes binding of libptd.so (include/ptd.h).

The library must be built (``python pseudotransientdiffusion.jl_gb300/build.py``
or ``__graft_entry__.build()``); loading fails loudly when it is missing, there
is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG_DIR)
LIB_PATH = os.path.join(PKG_DIR, "libptd.so")
HEADER = os.path.join(ROOT, "include", "ptd.h")

PTD_OK, PTD_EINVAL, PTD_ENAN, PTD_ENOTCONV, PTD_ECUDA, PTD_ENOMEM, PTD_ESTATE, PTD_ETIMEOUT = range(8)
MODEL_LIN, MODEL_LINSTEP, MODEL_NONLIN = 0, 1, 2
PREC_FP64, PREC_FP32_DC, PREC_DF64, PREC_DFH, PREC_FP32_RB = 0, 1, 2, 3, 4
RESID_MIXED, RESID_CONSISTENT = 0, 1
NORM_RMS, NORM_MAX = 0, 1
FLAG_STRICT = 0x1
FLAG_AUTOTUNE = 0x2
FLAG_DC_NO_TBLOCK = 0x4
FLAG_RB_TBLOCK_3D = 0x8


class PtdParams(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("model", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("dt", C.c_double),
        ("nt", C.c_int32), ("itmax", C.c_int32), ("nchk", C.c_int32), ("precision", C.c_int32),
        ("tol", C.c_double), ("cfl", C.c_double), ("resc", C.c_double), ("D", C.c_double),
        ("resid_mode", C.c_int32), ("norm", C.c_int32),
        ("norm_len", C.c_double),
        ("flags", C.c_int32), ("dc_max_outer", C.c_int32),
        ("dc_inner_rtol", C.c_double),
        ("reserved", C.c_int32 * 8),
    ]


def check_field(a, n: int, name: str, out: bool = False):
    """A field handed to the library by address must hold exactly n float64
    values in x-fastest order: the library reads (or, out=True, writes) 8*n
    bytes at the address, so a wrong dtype or size would run past the buffer.
    Host arrays: float64, n elements, contiguous in Fortran order (a 1D array
    contiguous), writeable when out.  Tensors (anything with data_ptr(), on
    the host or the GPU): float64, n elements, contiguous.  Returns a
    unchanged; raises ValueError otherwise."""
    if hasattr(a, "data_ptr"):
        if str(a.dtype) != "torch.float64" or a.numel() != n or not a.is_contiguous():
            raise ValueError(f"{name}: expected a contiguous float64 tensor of {n} elements "
                             f"(got {a.dtype}, {a.numel()} elements)")
        return a
    if not hasattr(a, "dtype") or a.dtype != "float64" or a.size != n:
        raise ValueError(f"{name}: expected {n} float64 values (got {getattr(a, 'dtype', type(a).__name__)}, "
                         f"{getattr(a, 'size', '?')} values)")
    if not a.flags.f_contiguous or not a.flags.aligned:
        raise ValueError(f"{name}: expected contiguous x-fastest (Fortran-ordered) storage")
    if out and not a.flags.writeable:
        raise ValueError(f"{name}: the array is read-only")
    return a


class PtdError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        super().__init__(f"{where}: {strerror(status)} ({detail})")


_lib = None


def declared_functions():
    """Names of the entry points declared in include/ptd.h."""
    with open(HEADER) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"PTD_API\s+[\w\s\*]+?\b(ptd_\w+)\s*\(", text)))


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() "
                          "(pseudotransientdiffusion.jl_gb300/build.py) first")
    L = C.CDLL(LIB_PATH)
    dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_void_p
    pp = C.POINTER(PtdParams)
    sig = {
        "ptd_params_init": (C.c_int, [pp, C.c_int32, C.c_int32]),
        "ptd_create": (C.c_int, [C.POINTER(C.c_void_p), pp]),
        "ptd_solve": (C.c_int, [vp, vp, vp, ip, dp, C.c_int32, ip]),
        "ptd_set_state": (C.c_int, [vp, vp, vp]),
        "ptd_set_state2": (C.c_int, [vp, vp, vp, vp]),
        "ptd_measure_fp64_rate": (C.c_int, [dp]),
        "ptd_step": (C.c_int, [vp, C.c_int32, ip, dp, C.c_int32, ip]),
        "ptd_iterate": (C.c_int, [vp, C.c_int32]),
        "ptd_get_state": (C.c_int, [vp, vp]),
        "ptd_stream": (C.c_void_p, [vp]),
        "ptd_sync": (C.c_int, [vp]),
        "ptd_counters": (C.c_int, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
        "ptd_launch_config": (C.c_int, [vp, C.POINTER(C.c_int32)]),
        "ptd_set_launch_config": (C.c_int, [vp, C.POINTER(C.c_int32)]),
        "ptd_destroy": (None, [vp]),
        "ptd_strerror": (C.c_char_p, [C.c_int]),
        "ptd_last_error": (C.c_char_p, []),
        "ptd_abi_version": (C.c_int, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def strerror(status: int) -> str:
    return lib().ptd_strerror(status).decode()


def last_error() -> str:
    return lib().ptd_last_error().decode()


def check(status: int, where: str) -> int:
    if status != PTD_OK:
        raise PtdError(status, where, last_error())
    return status
