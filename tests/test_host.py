"""Host-side logic and the C ABI surface (no GPU needed).

* libptd.so loads and exports every entry point declared in include/ptd.h;
* the ctypes mirror of ptd_params has the C layout (checked against gcc);
* ptd_params_init restates the reference scripts' defaults;
* ptd_create validates its parameters before touching the GPU;
* the scripts table, grids and initial conditions follow the reference.
* the wrappers reject fields whose dtype, size or layout would make the
  library read or write past the buffer, before calling it.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from ptdiff import _abi
from ptdiff import scripts as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    declared = _abi.declared_functions()
    assert "ptd_solve" in declared and "ptd_create" in declared
    L = _abi.lib()
    for name in declared:
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _abi.LIB_PATH], capture_output=True, text=True)
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if " T " in ln}
    assert set(declared) <= exported
    # nothing but the C ABI is exported
    assert all(n.startswith("ptd_") for n in exported), sorted(exported)
    assert L.ptd_abi_version() == 1


def test_params_layout_matches_c(tmp_path):
    fields = [f for f, _ in _abi.PtdParams._fields_]
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT}/include/ptd.h"',
             'int main(void){', 'printf("%zu\\n", sizeof(ptd_params));']
    lines += [f'printf("%zu\\n", offsetof(ptd_params, {f}));' for f in fields]
    lines += ['return 0;}']
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                           check=True).stdout.split()]
    assert vals[0] == C.sizeof(_abi.PtdParams)
    for f, off in zip(fields, vals[1:]):
        assert getattr(_abi.PtdParams, f).offset == off, f


def test_batch_params_layout_matches_c(tmp_path):
    from ptdiff.batch import PtdBatchParams

    fields = [f for f, _ in PtdBatchParams._fields_]
    src = tmp_path / "blayout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT}/include/ptd.h"',
             'int main(void){', 'printf("%zu\\n", sizeof(ptd_batch_params));']
    lines += [f'printf("%zu\\n", offsetof(ptd_batch_params, {f}));' for f in fields]
    lines += ['return 0;}']
    src.write_text("\n".join(lines))
    exe = tmp_path / "blayout"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                           check=True).stdout.split()]
    assert vals[0] == C.sizeof(PtdBatchParams)
    for f, off in zip(fields, vals[1:]):
        assert getattr(PtdBatchParams, f).offset == off, f


def test_batch_create_rejects_invalid_params():
    from ptdiff import batch as B

    p = B.batch_params(2, precision="fp64")
    p.itmax = 95   # not a multiple of nchk
    h = C.c_void_p()
    n = (C.c_int32 * 2)(32, 40)
    assert B._lib().ptd_batch_create(C.byref(h), C.byref(p), n, n) == _abi.PTD_EINVAL
    assert "multiple of nchk" in _abi.last_error()
    p = B.batch_params(2, precision="fp64")
    n2 = (C.c_int32 * 2)(32, 2)
    assert B._lib().ptd_batch_create(C.byref(h), C.byref(p), n2, n2) == _abi.PTD_EINVAL
    p = B.batch_params(2, precision="fp64")
    p.precision = _abi.PREC_DFH   # single grids only
    assert B._lib().ptd_batch_create(C.byref(h), C.byref(p), n, n) == _abi.PTD_EINVAL
    # three instances of 2^39 cells each: every one valid, together above 2^40
    p = B.batch_params(3, precision="fp64")
    nx3, ny3 = (C.c_int32 * 3)(1 << 20, 1 << 20, 1 << 20), (C.c_int32 * 3)(1 << 19, 1 << 19, 1 << 19)
    assert B._lib().ptd_batch_create(C.byref(h), C.byref(p), nx3, ny3) == _abi.PTD_EINVAL
    assert "2^40 cells in all" in _abi.last_error()


@pytest.mark.parametrize("ndim,model", [(1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2), (3, 0), (3, 1), (3, 2)])
def test_params_init_matches_scripts(ndim, model):
    p = _abi.PtdParams()
    assert _abi.lib().ptd_params_init(C.byref(p), ndim, model) == 0
    name = {0: "lin", 1: "linstep", 2: "nonlin"}[model]
    s = S.SCRIPTS[f"diff_{ndim}D_{name}" + ("_multixpu" if ndim == 3 else "")]
    assert p.cfl == s.cfl and p.resc == s.resc
    assert p.tol == s.tol and p.itmax == s.itmax and p.nchk == s.nout
    assert p.dt == s.dt and p.nt == s.nt and p.lx == s.lx
    assert (p.nx, p.ny, p.nz)[:ndim] == (s.default_n,) * ndim


def _create(**kw):
    p = _abi.PtdParams()
    _abi.lib().ptd_params_init(C.byref(p), kw.pop("ndim", 2), kw.pop("model", 2))
    for k, v in kw.items():
        setattr(p, k, v)
    h = C.c_void_p()
    st = _abi.lib().ptd_create(C.byref(h), C.byref(p))
    return st, _abi.last_error()


@pytest.mark.parametrize("kw,msg", [
    (dict(nx=2), "needs >= 3 cells"),
    (dict(nz=4), "must be 1 for a 2D grid"),
    (dict(dt=0.0), "dt must be > 0"),
    (dict(nchk=0), "nchk must be >= 1"),
    (dict(itmax=-1), "itmax must be >= 0"),
    (dict(cfl=-1.0), "cfl must be > 0"),
    (dict(precision=7), "unknown precision"),
    (dict(resid_mode=3), "unknown resid_mode"),
    (dict(norm=5), "unknown norm"),
    (dict(flags=0x100), "unknown flags"),
    (dict(model=0, D=0.0), "D must be > 0"),
    (dict(ndim=4), "ndim must be"),
    (dict(nx=1 << 21, ny=1 << 20), "too large (limit 2^40 cells)"),
    (dict(ndim=3, nx=1 << 14, ny=1 << 13, nz=1 << 14), "too large (limit 2^40 cells)"),
    (dict(ndim=3, nx=1 << 30, ny=1 << 30, nz=1 << 30), "too large (limit 2^40 cells)"),   # 2^90: no wrap
])
def test_create_rejects_invalid_params(kw, msg):
    st, err = _create(**kw)
    assert st == _abi.PTD_EINVAL
    assert msg in err


def test_strerror_and_null_args():
    L = _abi.lib()
    assert _abi.strerror(0) == "ok"
    assert _abi.strerror(_abi.PTD_ENAN) == "residual is NaN"
    assert L.ptd_create(None, None) == _abi.PTD_EINVAL
    assert L.ptd_solve(None, None, None, None, None, 0, None) == _abi.PTD_EINVAL
    assert L.ptd_step(None, 1, None, None, 0, None) == _abi.PTD_EINVAL
    assert L.ptd_params_init(None, 2, 2) == _abi.PTD_EINVAL
    L.ptd_destroy(None)


def test_linrange_and_cell_centres():
    x = S.linrange(0.5, 9.5, 10)
    assert x[0] == 0.5 and x[-1] == 9.5
    assert np.allclose(np.diff(x), 1.0)
    xc = S.cell_centres(10.0, 64)
    assert xc[0] == 10.0 / 64 / 2 and np.allclose(np.diff(xc), 10.0 / 64)
    assert list(S.sample_indices(64)[:3]) == [0, 6, 12]


def test_step_fields():
    s1 = S.SCRIPTS["diff_1D_linstep"]
    D = S.step_field(s1, 64)
    assert (D[:30] == 1e-4).all() and (D[30:] == 1.0).all()  # ceil(64/2.2) = 30
    s2 = S.SCRIPTS["diff_2D_linstep"]
    D = S.step_field(s2, 64, 64)
    assert (D[:30, :] == 1e-4).all() and (D[:, :30] == 1e-4).all() and (D[30:, 30:] == 1.0).all()
    s3 = S.SCRIPTS["diff_3D_linstep_multixpu"]
    D = S.step_field(s3, 32, 32, 32)
    # x_g = (ix-1)*dx < lx/2.2 -> first 15 planes (14*0.3125 = 4.375 < 4.545)
    assert (D[:15] == 1e-4).all() and (D[15:, 15:, :] == 1.0).all()


def test_benchmark_initial_condition():
    s = S.CONFIGS["2d_nonlin_4096"]
    H = S.initial_condition(s, 32, 32)
    assert H[0, 5] == 1.0 and H[-1, 5] == 1.0 and H[5, 0] == 1.0 and H[5, -1] == 1.0
    assert np.isclose(H[15, 15], 1.0 + np.exp(-2 * (10 / 64) ** 2))
    assert s.nout == 100 and s.nt == 5
    assert S.CONFIGS["3d_nonlin_512"].nt == 3


def test_adjoint_create_rejects_unsupported_precisions():
    from ptdiff import adjoint as A
    from ptdiff.solvers import make_params

    for prec in ("dfh", "fp32_dc"):
        p = make_params(S.SCRIPTS["diff_3D_nonlin_multixpu"], (16, 16, 16), precision=prec)
        h = C.c_void_p()
        assert A._lib().ptd_adj_create(C.byref(h), C.byref(p)) == _abi.PTD_EINVAL
        assert "the adjoint runs in" in _abi.last_error()


@pytest.mark.parametrize("kw,msg", [({"resid_mode": 1}, "mixed residual")])
def test_rebased_fp32_rejections(kw, msg):
    from ptdiff.solvers import make_params

    p = make_params(S.SCRIPTS["diff_2D_lin"], (32, 32), precision="fp32_rb")
    for k, v in kw.items():
        setattr(p, k, v)
    h = C.c_void_p()
    assert _abi.lib().ptd_create(C.byref(h), C.byref(p)) == _abi.PTD_EINVAL
    assert msg in _abi.last_error()


def test_field_check_rejects_what_would_run_past_the_buffer():
    """Fields go to the library by address (8*n bytes read or written), so
    the wrappers reject a wrong dtype, size or layout before the call."""
    n = 6 * 5
    good = np.zeros((6, 5), order="F")
    assert _abi.check_field(good, n, "H", out=True) is good
    assert _abi.check_field(np.zeros(n), n, "H") is not None             # 1D contiguous
    bad = [np.zeros((6, 5), dtype=np.float32, order="F"),                # 4-byte values
           np.zeros((6, 4), order="F"),                                  # too few values
           np.zeros((6, 5), order="C"),                                  # y fastest
           np.zeros(2 * n)[::2],                                         # strided view
           [0.0] * n]                                                    # not an array
    for a in bad:
        with pytest.raises(ValueError):
            _abi.check_field(a, n, "H")
    ro = np.zeros((6, 5), order="F")
    ro.flags.writeable = False
    assert _abi.check_field(ro, n, "D") is ro                           # read-only input is fine
    with pytest.raises(ValueError, match="read-only"):
        _abi.check_field(ro, n, "H", out=True)
    torch = pytest.importorskip("torch")
    assert _abi.check_field(torch.zeros(n, dtype=torch.float64), n, "H") is not None
    for t in (torch.zeros(n, dtype=torch.float32), torch.zeros(n + 1, dtype=torch.float64),
              torch.zeros(5, 6, dtype=torch.float64).t()):
        with pytest.raises(ValueError):
            _abi.check_field(t, n, "H")


def test_batch_solve_checks_counts_and_sizes_before_the_call():
    from ptdiff import batch as B

    b = object.__new__(B.BatchSolver)   # no ptd_batch_create: the checks run first
    b.params = B.PtdBatchParams()
    b.params.ninst = 2
    b.nx = np.array([4, 5], dtype=np.int32)
    b.ny = np.array([4, 6], dtype=np.int32)
    b._h = C.c_void_p()
    H = [np.zeros((4, 4), order="F"), np.zeros((5, 6), order="F")]
    with pytest.raises(ValueError, match="expected 2 H arrays"):
        b.solve(H[:1])
    with pytest.raises(ValueError, match=r"H\[1\]"):
        b.solve([H[0], np.zeros((5, 5), order="F")])
    with pytest.raises(ValueError, match=r"D\[0\]"):
        b.solve(H, [np.zeros((3, 4)), np.zeros((5, 6))])
    with pytest.raises(ValueError):
        B.BatchSolver(B.batch_params(2, model=1), [4, 5], [4])
