"""Batched solves: many independent 2D grids of uneven sizes in one launch
per PT iteration (libptd.so ``ptd_batch_*``).

``batch_instances(n, seed)`` generates the benchmark batch: square grids with
sides log-uniform in [128, 1024], step-function D = 1 below and 1e-4 above a
random horizontal interface at y in [0.3, 0.7] ly, H0 = 1 + A exp(-r^2)
around a random centre with amplitude A ~ U(0.5, 2).  The batch has no
reference counterpart; each instance is the reference's 2D step-diffusion
problem (scripts/diff_2D_linstep.jl) with its own D and H0.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from .scripts import LINSTEP, cell_centres


class PtdBatchParams(C.Structure):
    _fields_ = [
        ("ninst", C.c_int32), ("model", C.c_int32),
        ("lx", C.c_double), ("ly", C.c_double), ("dt", C.c_double),
        ("nt", C.c_int32), ("itmax", C.c_int32), ("nchk", C.c_int32), ("precision", C.c_int32),
        ("tol", C.c_double), ("cfl", C.c_double), ("resc", C.c_double), ("D", C.c_double),
        ("norm", C.c_int32), ("flags", C.c_int32),
        ("dc_max_outer", C.c_int32), ("pad0", C.c_int32),
        ("dc_inner_rtol", C.c_double),
        ("reserved", C.c_int32 * 8),
    ]


_bound = False


def _lib():
    global _bound
    L = _abi.lib()
    if not _bound:
        vp, ip = C.c_void_p, C.POINTER(C.c_int32)
        pp = C.POINTER(PtdBatchParams)
        L.ptd_batch_params_init.argtypes = [pp, C.c_int32, C.c_int32]
        L.ptd_batch_params_init.restype = C.c_int
        L.ptd_batch_create.argtypes = [C.POINTER(C.c_void_p), pp, ip, ip]
        L.ptd_batch_create.restype = C.c_int
        L.ptd_batch_solve.argtypes = [vp, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), ip,
                                      C.POINTER(C.c_double), ip]
        L.ptd_batch_solve.restype = C.c_int
        L.ptd_batch_tune.argtypes = [vp, ip, ip, C.POINTER(C.c_float)]
        L.ptd_batch_tune.restype = C.c_int
        L.ptd_batch_config.argtypes = [vp, ip, ip, ip]
        L.ptd_batch_config.restype = C.c_int
        L.ptd_batch_set_config.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32]
        L.ptd_batch_set_config.restype = C.c_int
        L.ptd_batch_counters.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.ptd_batch_counters.restype = C.c_int
        L.ptd_batch_destroy.argtypes = [vp]
        L.ptd_batch_destroy.restype = None
        _bound = True
    return L


def batch_params(ninst, model=LINSTEP, precision="fp32_dc", **kw) -> PtdBatchParams:
    p = PtdBatchParams()
    _abi.check(_lib().ptd_batch_params_init(C.byref(p), ninst, model), "ptd_batch_params_init")
    p.precision = ({"fp64": 0, "fp32_dc": 1, "df64": 2, "fp32_rb": 4}[precision] if isinstance(precision, str)
                   else precision)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class BatchSolver:
    def __init__(self, params: PtdBatchParams, nx, ny):
        self.params = params
        self.nx = np.ascontiguousarray(nx, dtype=np.int32)
        self.ny = np.ascontiguousarray(ny, dtype=np.int32)
        if not len(self.nx) == params.ninst == len(self.ny):
            raise ValueError(f"nx, ny: expected {params.ninst} sizes each (got {len(self.nx)}, {len(self.ny)})")
        self._h = C.c_void_p()
        _abi.check(_lib().ptd_batch_create(C.byref(self._h), C.byref(params),
                                           self.nx.ctypes.data_as(C.POINTER(C.c_int32)),
                                           self.ny.ctypes.data_as(C.POINTER(C.c_int32))), "ptd_batch_create")

    def close(self):
        if self._h:
            _lib().ptd_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tune(self):
        w, c, us = C.c_int32(0), C.c_int32(0), C.c_float(0)
        _abi.check(_lib().ptd_batch_tune(self._h, C.byref(w), C.byref(c), C.byref(us)), "ptd_batch_tune")
        return w.value, c.value, us.value

    def config(self):
        """(warps per CTA, rows per y chunk, inner iterations per launch)."""
        w, c, t = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        _abi.check(_lib().ptd_batch_config(self._h, C.byref(w), C.byref(c), C.byref(t)), "ptd_batch_config")
        return w.value, c.value, t.value

    def set_config(self, warps, chunk, iters_per_launch):
        """Set the launch shape (warps per CTA, rows per y chunk, FP32
        iterations per launch)."""
        _abi.check(_lib().ptd_batch_set_config(self._h, warps, chunk, iters_per_launch), "ptd_batch_set_config")

    def solve(self, Hs, Ds=None):
        """Solve in place on the list of fields Hs: Fortran-ordered host arrays,
        or contiguous float64 tensors (host or device; x fastest, i.e. the
        transpose of a C-ordered (ny, nx) tensor).  Returns (iters[ninst, nt],
        err_last[ninst])."""
        n = self.params.ninst
        cells = [int(a) * int(b) for a, b in zip(self.nx, self.ny)]
        if len(Hs) != n or (Ds is not None and len(Ds) != n):
            raise ValueError(f"expected {n} H arrays{' and D arrays' if Ds is not None else ''}")
        for i, H in enumerate(Hs):
            _abi.check_field(H, cells[i], f"H[{i}]", out=True)
        addr = lambda a: a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
        hp = (C.c_void_p * n)(*[addr(H) for H in Hs])
        dp = None
        if Ds is not None:
            Ds = [_abi.check_field(D if hasattr(D, "data_ptr") else np.asfortranarray(D, dtype=np.float64),
                                   cells[i], f"D[{i}]") for i, D in enumerate(Ds)]
            dp = (C.c_void_p * n)(*[addr(D) for D in Ds])
        iters = np.zeros(n * max(self.params.nt, 1), dtype=np.int32)
        err = np.zeros(n, dtype=np.float64)
        nd = C.c_int32(0)
        st = _lib().ptd_batch_solve(self._h, hp, dp, iters.ctypes.data_as(C.POINTER(C.c_int32)),
                                    err.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nd))
        _abi.check(st, "ptd_batch_solve")
        return iters.reshape(n, max(self.params.nt, 1)), err

    def counters(self):
        l, it = C.c_int64(0), C.c_int64(0)
        _abi.check(_lib().ptd_batch_counters(self._h, C.byref(l), C.byref(it)), "ptd_batch_counters")
        return l.value, it.value


def batch_instances(n=256, seed=0, nmin=128, nmax=1024, lx=10.0, ly=10.0):
    """(sizes, H0 list, D list) of the seeded benchmark batch."""
    rng = np.random.default_rng(seed)
    sides = np.rint(np.exp(rng.uniform(math.log(nmin), math.log(nmax), n))).astype(int)
    Hs, Ds = [], []
    for k in range(n):
        m = int(sides[k])
        xc, yc = cell_centres(lx, m), cell_centres(ly, m)
        ystar = rng.uniform(0.3, 0.7) * ly
        cx, cy = rng.uniform(0.25, 0.75) * lx, rng.uniform(0.25, 0.75) * ly
        amp = rng.uniform(0.5, 2.0)
        H = 1.0 + amp * np.exp(-(xc[:, None] - cx) ** 2 - (yc[None, :] - cy) ** 2)
        D = np.where(yc[None, :] < ystar, 1.0, 1e-4) * np.ones((m, 1))
        Hs.append(np.asfortranarray(H))
        Ds.append(np.asfortranarray(D))
    return sides, Hs, Ds
