"""Parity of the CUDA library (through the C ABI) with the CPU oracle and the
reference's golden data, for the three FP64-accuracy forms of the PT
iteration: native FP64, double-float (DF64, FP32 pipe) and double-float
arithmetic on an FP64 H (DFH).  Bar: PT iteration counts equal, relative L2
error of H <= 1e-10."""
import numpy as np
import pytest

import ptdiff
from golden_cases import (COUNT_SCRIPTS, GOLDEN_CASES, golden_array, load_counts, load_reftests,
                          multirank_norm_len, reference_isapprox, sample, start_fields)
from oracle import oracle as O
from ptdiff import _abi
from ptdiff import scripts as S

pytestmark = pytest.mark.gpu

REF = load_reftests()
COUNTS = load_counts()
RTOL_FP64 = 1e-10


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def gpu_solve(s, shape, D=None, H0=None, **kw):
    H, Hold = start_fields(s, shape)
    if H0 is not None:
        H = np.array(H0, order="F", copy=True)
    p = ptdiff.make_params(s, shape, **kw)
    with ptdiff.Solver(p) as sol:
        iters, eh, st = sol.solve(H, D, raise_on_nan=False, Hold=Hold)
    return H, iters, eh, st


def oracle_kw(kw):
    out = {}
    for k in ("nt", "itmax", "norm_len"):
        if k in kw:
            out[k] = kw[k]
    if "nchk" in kw:
        out["nout"] = kw["nchk"]
    if kw.get("resid") == "consistent":
        out["resid"] = 1
    if kw.get("norm") == "max":
        out["norm"] = 1
    return out


def compare(s, shape, **kw):
    D = S.step_field(s, *shape) if s.model == S.LINSTEP else None
    H0, Hold0 = start_fields(s, shape)
    H, iters, eh, st = gpu_solve(s, shape, D, **kw)
    Hr, iters_r, eh_r, st_r = O.solve(s, H0, D, Hold0=Hold0, **oracle_kw(kw))
    assert st == 0 and st_r == 0
    assert list(iters) == list(iters_r)
    assert rel_l2(H, Hr) <= RTOL_FP64
    assert len(eh) == len(eh_r)
    if len(eh):
        # the iteration parameters are evaluated in FP32 on the GPU: the err
        # history agrees to ~1e-6 relative, the converged H to ~1e-14
        assert np.allclose(eh, eh_r, rtol=1e-4, atol=1e-12)
    return H, iters


PRECS = ["fp64", "df64", "dfh"]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", sorted(GOLDEN_CASES))
def test_golden_cases(name, prec):
    n = GOLDEN_CASES[name]
    s = S.SCRIPTS[name]
    H, _ = compare(s, (n,) * s.ndim, precision=prec)
    got = sample(H, n, s.ndim)
    ref = golden_array(REF[name])
    assert reference_isapprox(got, ref)
    assert rel_l2(got, ref) <= RTOL_FP64


# DF64 holds H with a 48-bit significand: one unit in the last place of H moves
# the residual by ~2^-48 |H| (1/dt + sum_d 4 sigma_d K), which reaches tol on
# fine 1D/2D grids (1D nx >= 2048, 2D >= 1024^2); the DF64 cases stay below.
LIMITS = {"fp64": {1: 2048, 2: 256, 3: 126}, "df64": {1: 1024, 2: 256, 3: 126},
          "dfh": {1: 2048, 2: 256, 3: 126}}


def _count_cases():
    out = []
    for prec in PRECS:
        for key, rows in COUNTS.items():
            s = S.SCRIPTS[COUNT_SCRIPTS[key]]
            for row in rows:
                if row[0] <= LIMITS[prec][s.ndim]:
                    out.append((key, tuple(row), prec))
    return out


@pytest.mark.parametrize("key,row,prec", _count_cases())
def test_published_iteration_counts(key, row, prec):
    s = S.SCRIPTS[COUNT_SCRIPTS[key]]
    shape = row[: s.ndim]
    D = S.step_field(s, *shape) if s.model == S.LINSTEP else None
    nl = multirank_norm_len(shape[0]) if s.ndim == 3 else 0.0
    _, iters, _, st = gpu_solve(s, shape, D, norm_len=nl, precision=prec)
    assert st == 0
    assert int(iters.sum()) == row[s.ndim]


@pytest.mark.parametrize("name,shape", [
    ("diff_2D_nonlin", (37, 95)), ("diff_2D_lin", (3, 3)), ("diff_2D_linstep", (66, 33)),
    ("diff_2D_nonlin", (200, 7)), ("diff_3D_nonlin_multixpu", (35, 17, 9)),
    ("diff_3D_linstep_multixpu", (3, 4, 5)), ("diff_3D_lin_multixpu", (63, 33, 20)),
    ("diff_1D_nonlin", (3,)), ("diff_1D_linstep", (1000,)),
])
@pytest.mark.parametrize("prec", PRECS)
def test_ragged_and_tiny_grids(name, shape, prec):
    compare(S.SCRIPTS[name], shape, precision=prec)


@pytest.mark.parametrize("kw", [
    dict(nchk=7), dict(nchk=1), dict(itmax=95), dict(itmax=50, nchk=200), dict(itmax=0),
    dict(norm="max"), dict(resid="consistent"), dict(nt=0), dict(nchk=13, itmax=100),
])
@pytest.mark.parametrize("name,shape", [("diff_2D_nonlin", (48, 40)), ("diff_3D_linstep_multixpu", (20, 18, 16)),
                                        ("diff_1D_lin", (64,))])
@pytest.mark.parametrize("prec", PRECS)
def test_driver_options(name, shape, kw, prec):
    compare(S.SCRIPTS[name], shape, precision=prec, **kw)


@pytest.mark.parametrize("prec", PRECS)
def test_perf_scripts_fixed_iterations(prec):
    for name, shape in [("diff_2D_nonlin_perf", (96, 64)), ("diff_3D_nonlin_perf", (40, 40, 40))]:
        _, iters = compare(S.SCRIPTS[name], shape, precision=prec)
        assert list(iters) == [S.SCRIPTS[name].itmax] * S.SCRIPTS[name].nt


@pytest.mark.parametrize("prec", PRECS)
def test_nan_input_reports_enan(prec):
    s = S.SCRIPTS["diff_2D_nonlin"]
    H0 = S.initial_condition(s, 40, 40)
    H0[20, 20] = np.nan
    _, _, _, st = gpu_solve(s, (40, 40), H0=H0, precision=prec)
    assert st == _abi.PTD_ENAN
    _, _, _, st_r = O.solve(s, H0)
    assert st_r == 2


def test_strict_mode_reports_not_converged():
    s = S.SCRIPTS["diff_2D_lin"]
    _, iters, _, st = gpu_solve(s, (64, 64), itmax=30, strict=True)
    assert st == _abi.PTD_ENOTCONV
    assert list(iters) == [30] * 5


@pytest.mark.parametrize("prec", PRECS + ["fp32_dc"])
def test_device_pointers(prec):
    torch = pytest.importorskip("torch")
    s = S.SCRIPTS["diff_2D_linstep"]
    shape = (70, 50)
    H0 = S.initial_condition(s, *shape)
    D = S.step_field(s, *shape)
    Hd = torch.from_numpy(np.ravel(H0, order="F").copy()).cuda()
    Dd = torch.from_numpy(np.ravel(D, order="F").copy()).cuda()
    p = ptdiff.make_params(s, shape, precision=prec)
    with ptdiff.Solver(p) as sol:
        iters, _, st = sol.solve(Hd, Dd)
    Hr, iters_r, _, _ = O.solve(s, H0, D)
    assert st == 0
    if prec == "fp32_dc":
        assert rel_l2(Hd.cpu().numpy(), np.ravel(Hr, order="F")) <= 5e-8
    else:
        assert list(iters) == list(iters_r)
        assert rel_l2(Hd.cpu().numpy(), np.ravel(Hr, order="F")) <= RTOL_FP64


def test_resident_state_api_matches_solve():
    s = S.SCRIPTS["diff_3D_nonlin_multixpu"]
    shape = (24, 24, 24)
    H0 = S.initial_condition(s, *shape)
    p = ptdiff.make_params(s, shape)
    with ptdiff.Solver(p) as sol:
        sol.set_state(H0)
        its = [int(sol.step(1)[0][0]) for _ in range(s.nt)]
        H = sol.get_state().reshape(shape, order="F")
        launches, iters_done = sol.counters()
    Hr, iters_r, _, _ = O.solve(s, H0)
    assert its == list(iters_r)
    assert rel_l2(H, Hr) <= RTOL_FP64
    assert iters_done >= sum(its) and launches > iters_done


@pytest.mark.parametrize("prec", PRECS)
def test_iterate_matches_oracle_iterations(prec):
    s = S.SCRIPTS["diff_2D_nonlin_perf"]
    shape = (130, 70)
    H0 = S.initial_condition(s, *shape)
    p = ptdiff.make_params(s, shape, precision=prec)
    with ptdiff.Solver(p) as sol:
        sol.set_state(H0)
        sol.iterate(77)
        H = sol.get_state().reshape(shape, order="F")
    Hr = np.array(H0, order="F")
    q = [np.zeros_like(Hr) for _ in range(3)]
    O.iterate(s, Hr, H0.copy(order="F"), q, 77)
    assert rel_l2(H, Hr) <= 1e-12


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name,shape", [("diff_2D_nonlin", (130, 97)), ("diff_3D_linstep_multixpu", (40, 36, 50))])
def test_autotuned_launch_shape_gives_the_same_solution(name, shape, prec):
    s = S.SCRIPTS[name]
    D = S.step_field(s, *shape) if s.model == S.LINSTEP else None
    H0 = S.initial_condition(s, *shape)
    H = np.array(H0, order="F", copy=True)
    with ptdiff.Solver(ptdiff.make_params(s, shape, precision=prec, autotune=True)) as sol:
        cfg = sol.launch_config()
        iters, _, st = sol.solve(H, D)
    assert cfg["warps2d"] in (2, 4, 8) and cfg["chunk2d"] in (16, 32, 64, 128)
    assert cfg["rows3d"] in (8, 16) and cfg["chunk3d"] in (16, 32, 64, 128, 256, 512)
    Hr, iters_r, _, _ = O.solve(s, H0, D)
    assert st == 0 and list(iters) == list(iters_r)
    assert rel_l2(H, Hr) <= RTOL_FP64


# DFH keeps H in FP64: it reaches tol on the fine grids where DF64's 48-bit H
# cannot, with FP64's iteration counts (and the published ones within 1 %).
# (Not 1D lin/linstep at nx >= 8192: there FP64's own residual floor is within
# 32x of tol, and the 48-bit flux arithmetic's floor is 32x higher.)
@pytest.mark.parametrize("key,n", [("1D_nonlin", 4096), ("1D_lin", 4096), ("2D_nonlin", 1024),
                                   ("2D_linstep", 1024), ("2D_nonlin", 4096), ("3D_nonlin", 254)])
def test_dfh_matches_fp64_on_fine_grids(key, n):
    s = S.SCRIPTS[COUNT_SCRIPTS[key]]
    shape = (n,) * s.ndim
    D = S.step_field(s, *shape) if s.model == S.LINSTEP else None
    nl = multirank_norm_len(n) if s.ndim == 3 else 0.0
    H64, it64, _, st64 = gpu_solve(s, shape, D, norm_len=nl, precision="fp64")
    Hh, ith, _, sth = gpu_solve(s, shape, D, norm_len=nl, precision="dfh")
    assert st64 == 0 and sth == 0
    assert list(ith) == list(it64)
    assert rel_l2(Hh, H64) <= RTOL_FP64
    published = {tuple(r[: s.ndim]): r[s.ndim] for r in COUNTS[key]}[shape]
    assert abs(int(ith.sum()) - published) <= 0.01 * published


def test_run_script_writes_the_reference_outputs(tmp_path):
    sio = pytest.importorskip("scipy.io")
    res = ptdiff.run_script("diff_2D_nonlin", 64, 64, save=True, save_viz=True,
                            output_dir=str(tmp_path / "output"), viz_dir=str(tmp_path / "out_visu"))
    assert (tmp_path / "output" / "out_diff_2D_nonlin.txt").read_text() == "64 64 170 5\n"
    m = sio.loadmat(str(tmp_path / "out_visu" / "diff_2D_nonlin.mat"))
    assert np.array_equal(m["H_2D"], res.H) and m["xc_2D"].shape == (64, 1)
    perf = ptdiff.run_script("diff_3D_nonlin_perf", 32, save=True, output_dir=str(tmp_path / "output"))
    row = (tmp_path / "output" / "out_diff_3D_nonlin_perf.txt").read_text().split()
    assert row[:5] == ["1", "32", "32", "32", str(perf.ittot)]
    assert float(row[6]) == 10 * 32 ** 3 * 8 / 1e9 and float(row[8]) > 0


@pytest.mark.parametrize("prec", ["fp64", "dfh", "fp32_rb"])
@pytest.mark.parametrize("name,shape,cfg", [
    ("diff_2D_nonlin", (130, 97), {"warps2d": 1, "chunk2d": 1}), ("diff_2D_nonlin", (130, 97), {"warps2d": 8, "chunk2d": 200}),
    ("diff_2D_linstep", (66, 33), {"warps2d": 2, "chunk2d": 7}),
    ("diff_3D_nonlin_multixpu", (40, 36, 50), {"rows3d": 8, "chunk3d": 1}),
    ("diff_3D_linstep_multixpu", (40, 36, 50), {"rows3d": 16, "chunk3d": 13})])
def test_set_launch_config_keeps_the_solution(name, shape, cfg, prec):
    s = S.SCRIPTS[name]
    if prec == "fp32_rb" and cfg.get("rows3d") == 8:
        cfg = dict(cfg, rows3d=16)
    D = S.step_field(s, *shape) if s.model == S.LINSTEP else None
    H0 = S.initial_condition(s, *shape)
    H = np.array(H0, order="F", copy=True)
    with ptdiff.Solver(ptdiff.make_params(s, shape, precision=prec)) as sol:
        sol.set_launch_config(**cfg)
        got = sol.launch_config()
        iters, _, st = sol.solve(H, D)
    assert all(got[k] == v for k, v in cfg.items())
    Hr, iters_r, _, _ = O.solve(s, H0, D)
    assert st == 0
    if prec == "fp32_rb":
        rms = float(np.sqrt(np.mean(np.square(Hr))))
        assert rel_l2(H, Hr) <= 2 * s.dt * s.tol / rms
    else:
        assert list(iters) == list(iters_r)
        assert rel_l2(H, Hr) <= RTOL_FP64


@pytest.mark.parametrize("name,shape", [("diff_2D_nonlin", (96, 96)), ("diff_3D_nonlin_multixpu", (34, 34, 34))])
def test_resc_search_never_worse_than_the_script(name, shape):
    from ptdiff import dispersion as DP

    s = S.SCRIPTS[name]
    best, counts = DP.tune_resc(s, shape)
    assert best in counts and s.resc in counts
    assert counts[best] <= counts[s.resc]
