"""Gradients of an L2 misfit through the implicit PT solve (libptd.so
``ptd_adj_*``), and their torch.autograd binding.

``AdjointSolver(params)`` wraps one ``ptd_adj`` context (3D, D = exp(m) H^3 or
D = H^3): ``forward(H0, m, Ht)`` runs ``params.nt`` implicit steps keeping one
checkpoint per step and returns L = 1/2 sum_inner (H^nt - Ht)^2;
``gradient()`` returns (dL/dm, dL/dH0).  ``DiffusionMisfit`` is the
torch.autograd.Function over the same calls (the Python counterpart of the
Julia ChainRulesCore rrule in the package extension julia/ext/PTDiffusionChainRulesCoreExt.jl).  No reference counterpart.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

_bound = False


def _lib():
    global _bound
    L = _abi.lib()
    if not _bound:
        vp, ip, dp = C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double)
        L.ptd_adj_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(_abi.PtdParams)]
        L.ptd_adj_create.restype = C.c_int
        L.ptd_adj_forward.argtypes = [vp, vp, vp, vp, dp, vp, ip]
        L.ptd_adj_forward.restype = C.c_int
        L.ptd_adj_gradient.argtypes = [vp, vp, vp, ip]
        L.ptd_adj_gradient.restype = C.c_int
        L.ptd_adj_residuals.argtypes = [vp, dp, dp]
        L.ptd_adj_residuals.restype = C.c_int
        L.ptd_adj_counters.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.ptd_adj_counters.restype = C.c_int
        L.ptd_adj_destroy.argtypes = [vp]
        L.ptd_adj_destroy.restype = None
        _bound = True
    return L


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


class AdjointSolver:
    def __init__(self, params: _abi.PtdParams):
        self.params = params
        self.shape = (params.nx, params.ny, params.nz)
        self._h = C.c_void_p()
        _abi.check(_lib().ptd_adj_create(C.byref(self._h), C.byref(params)), "ptd_adj_create")

    def close(self):
        if self._h:
            _lib().ptd_adj_destroy(self._h)
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

    def _n(self):
        return self.shape[0] * self.shape[1] * self.shape[2]

    def _f(self, a, name):
        if a is None:
            return None
        a = a.contiguous() if hasattr(a, "data_ptr") else np.asfortranarray(a, dtype=np.float64)
        return _abi.check_field(a, self._n(), name)

    def forward(self, H0, m, Ht, want_HN=False):
        H0, m, Ht = self._f(H0, "H0"), self._f(m, "m"), self._f(Ht, "Ht")
        loss = C.c_double(0.0)
        HN = np.zeros(self.shape, dtype=np.float64, order="F") if want_HN else None
        iters = np.zeros(max(self.params.nt, 1), dtype=np.int32)
        _abi.check(_lib().ptd_adj_forward(self._h, _ptr(H0), _ptr(m), _ptr(Ht), C.byref(loss), _ptr(HN),
                                          iters.ctypes.data_as(C.POINTER(C.c_int32))), "ptd_adj_forward")
        self.forward_iters = iters[: self.params.nt].copy()
        return (loss.value, HN) if want_HN else loss.value

    def gradient(self, want_m=True, want_H0=True, out_m=None, out_H0=None):
        """(dL/dm, dL/dH0) of the last forward().  out_m / out_H0: caller-owned
        outputs (numpy Fortran arrays or contiguous device tensors of nx*ny*nz
        float64), else new numpy arrays."""
        gm = out_m if out_m is not None else (np.zeros(self.shape, dtype=np.float64, order="F") if want_m else None)
        gh = out_H0 if out_H0 is not None else (np.zeros(self.shape, dtype=np.float64, order="F") if want_H0
                                                 else None)
        for g, name in ((gm, "out_m"), (gh, "out_H0")):
            if g is not None:
                _abi.check_field(g, self._n(), name, out=True)
        iters = np.zeros(max(self.params.nt, 1), dtype=np.int32)
        _abi.check(_lib().ptd_adj_gradient(self._h, _ptr(gm), _ptr(gh),
                                           iters.ctypes.data_as(C.POINTER(C.c_int32))), "ptd_adj_gradient")
        self.adjoint_iters = iters[: self.params.nt].copy()
        return gm, gh

    def residuals(self):
        """(final residual, target) of each step's adjoint solve in the last gradient()."""
        e = np.zeros(max(self.params.nt, 1))
        t = np.zeros(max(self.params.nt, 1))
        _abi.check(_lib().ptd_adj_residuals(self._h, e.ctypes.data_as(C.POINTER(C.c_double)),
                                            t.ctypes.data_as(C.POINTER(C.c_double))), "ptd_adj_residuals")
        return e[: self.params.nt], t[: self.params.nt]

    def counters(self):
        l, it = C.c_int64(0), C.c_int64(0)
        _abi.check(_lib().ptd_adj_counters(self._h, C.byref(l), C.byref(it)), "ptd_adj_counters")
        return l.value, it.value


def misfit_function():
    """torch.autograd.Function computing L(m, H0) = 1/2 ||H^nt(m, H0) - Ht||^2
    with the library's forward and adjoint (float64 tensors, x fastest,
    shape (nz, ny, nx) in torch's C order, which is the library's layout).
    The tensors go to the library as they are -- device tensors as device
    pointers, so a CUDA tensor is never copied through the host -- and the
    gradients are written into tensors on the inputs' device."""
    import torch

    class DiffusionMisfit(torch.autograd.Function):
        @staticmethod
        def forward(ctx, m, H0, Ht, solver):
            args = [t.detach().to(torch.float64).contiguous() for t in (H0, m, Ht)]
            loss = solver.forward(*args)
            ctx.solver = solver
            ctx.like = args[1]
            return torch.tensor(loss, dtype=torch.float64, device=m.device)

        @staticmethod
        def backward(ctx, gout):
            gm, gh = torch.empty_like(ctx.like), torch.empty_like(ctx.like)
            ctx.solver.gradient(out_m=gm, out_H0=gh)
            return gout * gm, gout * gh, None, None

    return DiffusionMisfit
