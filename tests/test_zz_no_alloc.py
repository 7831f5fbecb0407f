"""ptd_solve_2d_noalloc -- the entry point for callers that cannot allocate
GPU memory when they need a solve: it takes its scratch from a fixed device
array compiled into the library instead of cudaMalloc.  Checked through the
C ABI against the allocating entry point (ptd_solve) on two calls in a row,
so that the second call also shows that the contents the first call left in
the shared array do not leak into its result.  This file is collected last."""
import ctypes as C

import numpy as np
import pytest

import ptdiff
from ptdiff import _abi
from ptdiff import scripts as S

pytestmark = pytest.mark.gpu


def _lib():
    L = _abi.lib()
    L.ptd_solve_2d_noalloc.argtypes = [C.POINTER(_abi.PtdParams), C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.POINTER(C.c_int32)]
    L.ptd_solve_2d_noalloc.restype = C.c_int
    return L


def _noalloc_solve(s, shape, H0, D):
    torch = pytest.importorskip("torch")
    p = ptdiff.make_params(s, shape)
    Hd = torch.from_numpy(np.ravel(H0, order="F").copy()).cuda()
    Dd = None if D is None else torch.from_numpy(np.ravel(D, order="F").copy()).cuda()
    iters = (C.c_int32 * p.nt)()
    stream = torch.cuda.current_stream().cuda_stream
    st = _lib().ptd_solve_2d_noalloc(C.byref(p), C.c_void_p(Hd.data_ptr()),
                                     None if Dd is None else C.c_void_p(Dd.data_ptr()), C.c_void_p(stream), iters)
    torch.cuda.synchronize()
    return st, Hd.cpu().numpy().reshape(shape, order="F"), list(iters)


def _allocating_solve(s, shape, H0, D):
    H = np.array(H0, order="F", copy=True)
    with ptdiff.Solver(ptdiff.make_params(s, shape)) as sol:
        iters, _, st = sol.solve(H, D)
    return st, H, list(iters)


def test_noalloc_matches_allocating_solve_on_two_calls():
    cases = [("diff_2D_nonlin", (200, 150)), ("diff_2D_linstep", (97, 120))]
    for name, shape in cases:
        s = S.SCRIPTS[name]
        H0 = S.initial_condition(s, *shape)
        D = S.step_field(s, *shape) if s.model == S.LINSTEP else None
        st, H, it = _noalloc_solve(s, shape, H0, D)
        st_r, H_r, it_r = _allocating_solve(s, shape, H0, D)
        assert st == 0 and st_r == 0, _abi.last_error()
        assert it == it_r
        assert np.linalg.norm(H - H_r) <= 1e-12 * np.linalg.norm(H_r)


def test_noalloc_leaves_device_memory_unchanged_after_the_startup_call():
    """The start-up call (nt = 0) reserves the array and loads the kernels;
    the solves after it, first and second, change no device memory
    reservation (cudaMemGetInfo's free bytes stay equal)."""
    torch = pytest.importorskip("torch")
    s = S.SCRIPTS["diff_2D_nonlin"]
    shape = (300, 200)
    p = ptdiff.make_params(s, shape)
    p0 = ptdiff.make_params(s, shape, nt=0)
    H0 = S.initial_condition(s, *shape)
    Hd = torch.from_numpy(np.ravel(H0, order="F").copy()).cuda()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert _lib().ptd_solve_2d_noalloc(C.byref(p0), None, None, stream, None) == 0, _abi.last_error()
    free = [torch.cuda.mem_get_info()[0]]
    for _ in range(2):
        Hd.copy_(torch.from_numpy(np.ravel(H0, order="F").copy()))
        torch.cuda.synchronize()
        st = _lib().ptd_solve_2d_noalloc(C.byref(p), C.c_void_p(Hd.data_ptr()), None, stream, None)
        torch.cuda.synchronize()
        assert st == 0, _abi.last_error()
        free.append(torch.cuda.mem_get_info()[0])
    assert free[0] == free[1] == free[2], free


def test_noalloc_rejects_host_memory():
    s = S.SCRIPTS["diff_2D_linstep"]
    shape = (64, 64)
    p = ptdiff.make_params(s, shape)
    torch = pytest.importorskip("torch")
    Hd = torch.ones(64 * 64, dtype=torch.float64, device="cuda")
    Dh = np.ones(64 * 64)
    st = _lib().ptd_solve_2d_noalloc(C.byref(p), C.c_void_p(Hd.data_ptr()), Dh.ctypes.data_as(C.c_void_p),
                                     None, None)
    assert st == _abi.PTD_EINVAL and "D must be device memory" in _abi.last_error()
    Hh = np.ones(64 * 64)
    p = ptdiff.make_params(S.SCRIPTS["diff_2D_nonlin"], shape)
    st = _lib().ptd_solve_2d_noalloc(C.byref(p), Hh.ctypes.data_as(C.c_void_p), None, None, None)
    assert st == _abi.PTD_EINVAL and "H must be device memory" in _abi.last_error()


def test_noalloc_rejects_grids_above_the_limit():
    torch = pytest.importorskip("torch")
    s = S.SCRIPTS["diff_2D_nonlin"]
    p = ptdiff.make_params(s, (1024, 1024))
    Hd = torch.zeros(1024 * 1024, dtype=torch.float64, device="cuda")
    st = _lib().ptd_solve_2d_noalloc(C.byref(p), C.c_void_p(Hd.data_ptr()), None, None, None)
    assert st == _abi.PTD_EINVAL
    assert "PTD_NOALLOC_MAX_CELLS" in _abi.last_error()
