"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; it checks the CUDA library and is never on the
product path.  ``build()`` compiles ``ptd_oracle.c`` with the Makefile beside
it (gcc, OpenMP, no FMA contraction).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libptd_oracle.so")
# the same source built for the host CPU (Makefile); only the timed CPU
# baseline of bench.py loads it
NATIVE_LIB_PATH = os.path.join(HERE, "libptd_oracle_native.so")


class OraParams(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("model", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("dt", C.c_double),
        ("nt", C.c_int32), ("itmax", C.c_int32), ("nout", C.c_int32),
        ("tol", C.c_double), ("cfl", C.c_double), ("resc", C.c_double), ("D", C.c_double),
        ("recip", C.c_int32), ("resid", C.c_int32), ("norm", C.c_int32), ("nthreads", C.c_int32),
        ("norm_len", C.c_double),
    ]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "ptd_oracle.c")
    stale = [p for p in (LIB_PATH, NATIVE_LIB_PATH)
             if not os.path.exists(p) or os.path.getmtime(p) < os.path.getmtime(src)]
    if force or stale:
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_libs = {}


def lib(native: bool = False):
    """The oracle library: the portable build (the checker), or with
    native=True the host-tuned build of the same source (CPU timing only)."""
    if native not in _libs:
        build()
        L = C.CDLL(NATIVE_LIB_PATH if native else LIB_PATH)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int32)
        L.ora_solve.argtypes = [C.POINTER(OraParams), dp, dp, ip, dp, C.c_int32, ip]
        L.ora_solve.restype = C.c_int
        L.ora_solve2.argtypes = [C.POINTER(OraParams), dp, dp, dp, ip, dp, C.c_int32, ip]
        L.ora_solve2.restype = C.c_int
        L.ora_iterate.argtypes = [C.POINTER(OraParams), dp, dp, dp, dp, dp, dp, C.c_int32]
        L.ora_iterate.restype = C.c_int
        L.ora_residual_norm.argtypes = [C.POINTER(OraParams), dp, dp, dp, dp]
        L.ora_residual_norm.restype = C.c_double
        L.ora_adjoint.argtypes = [C.POINTER(OraParams), dp, dp, dp, dp, dp, C.c_double]
        L.ora_adjoint.restype = C.c_int
        _libs[native] = L
    return _libs[native]


def _dptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def params(script, shape, *, nt=None, itmax=None, nout=None, resid=0, norm=0, nthreads=0,
           norm_len=0.0):
    s = script
    nx = shape[0]
    ny = shape[1] if len(shape) > 1 else 1
    nz = shape[2] if len(shape) > 2 else 1
    D = s.D if s.model == 0 else max(s.D, s.D2)
    return OraParams(s.ndim, s.model, nx, ny, nz, s.lx, s.ly, s.lz, s.dt,
                     s.nt if nt is None else nt,
                     s.itmax if itmax is None else itmax,
                     s.nout if nout is None else nout,
                     s.tol, s.cfl, s.resc, D, int(s.recip), resid, norm, nthreads, norm_len)


def solve(script, H0, D=None, *, nt=None, itmax=None, nout=None, resid=0, norm=0, nthreads=0,
          errcap=100000, norm_len=0.0, Hold0=None):
    """Run the reference algorithm on the CPU.  Returns (H, iters_per_step, errhist, status).
    Hold0: the first step's previous state (default H0; the reaction scripts use H0 = 0, Hold0 = Heq)."""
    H = np.array(H0, dtype=np.float64, order="F", copy=True)
    Ho = None if Hold0 is None else np.array(Hold0, dtype=np.float64, order="F", copy=True)
    p = params(script, H.shape, nt=nt, itmax=itmax, nout=nout, resid=resid, norm=norm,
               nthreads=nthreads, norm_len=norm_len)
    Dv = None if D is None else np.asfortranarray(D, dtype=np.float64)
    iters = np.zeros(max(p.nt, 1), dtype=np.int32)
    eh = np.zeros(errcap, dtype=np.float64)
    ne = C.c_int32(0)
    st = lib().ora_solve2(C.byref(p), _dptr(H), _dptr(Ho), _dptr(Dv),
                          iters.ctypes.data_as(C.POINTER(C.c_int32)), _dptr(eh), errcap, C.byref(ne))
    return H, iters[: p.nt].copy(), eh[: min(ne.value, errcap)].copy(), st


def iterate(script, H, Hold, q, niter, D=None, nthreads=0, native=False):
    """Fixed-iteration kernel loop (timed CPU baseline): updates H and q (3 arrays) in place.
    native=True runs the host-tuned build."""
    p = params(script, H.shape, nthreads=nthreads)
    Dv = None if D is None else np.asfortranarray(D, dtype=np.float64)
    st = lib(native).ora_iterate(C.byref(p), _dptr(H), _dptr(Hold), _dptr(Dv),
                           _dptr(q[0]), _dptr(q[1]), _dptr(q[2]), niter)
    if st:
        raise RuntimeError(f"ora_iterate failed ({st})")


def residual_norm(script, H, Hold, Hpre=None, D=None, norm=0):
    p = params(script, H.shape, norm=norm)
    Dv = None if D is None else np.asfortranarray(D, dtype=np.float64)
    return lib().ora_residual_norm(C.byref(p), _dptr(np.asfortranarray(H)),
                                   _dptr(np.asfortranarray(Hold)),
                                   _dptr(None if Hpre is None else np.asfortranarray(Hpre)), _dptr(Dv))


def forward_checkpoints(script, H0, m=None, *, nt=None, tol=None, itmax=None, nthreads=0):
    """H^0..H^nt of nt implicit steps, each solved from the previous state
    (fluxes restarted at every step).  Returns an array (nt+1, *H0.shape)."""
    s = script if tol is None else script.with_(tol=tol)
    nt = s.nt if nt is None else nt
    Hs = [np.array(H0, dtype=np.float64, order="F")]
    for _ in range(nt):
        H, _, _, st = solve(s, Hs[-1], m, nt=1, itmax=itmax, nthreads=nthreads)
        if st:
            raise RuntimeError(f"oracle forward failed ({st})")
        Hs.append(H)
    return np.stack(Hs)


def adjoint(script, Hs, Ht, m=None, rtol=1e-12, nthreads=0):
    """CPU FP64 reference adjoint: (grad_m, grad_H0) of 1/2 sum_inner (H^nt - Ht)^2."""
    shape = Hs.shape[1:]
    nt = Hs.shape[0] - 1
    p = params(script, shape, nt=nt, nthreads=nthreads)
    Hcat = np.concatenate([np.ravel(h, order="F") for h in Hs])
    gm = np.zeros(int(np.prod(shape)))
    gh = np.zeros(int(np.prod(shape)))
    mv = None if m is None else np.ravel(np.asarray(m, dtype=np.float64), order="F").copy()
    htv = np.ravel(np.asarray(Ht, dtype=np.float64), order="F").copy()
    st = lib().ora_adjoint(C.byref(p), _dptr(Hcat), _dptr(mv), _dptr(htv),
                           _dptr(gm) if m is not None else None, _dptr(gh), rtol)
    if st == 1:
        raise RuntimeError("ora_adjoint: bad arguments")
    return gm.reshape(shape, order="F"), gh.reshape(shape, order="F"), st
