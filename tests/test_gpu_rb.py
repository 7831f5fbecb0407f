"""FP32 PT iterations on the change since an FP64 base, rebased in FP64
(precision FP32_RB).  Every step must end with both the reference's check
residual and the FP64 residual of the returned H at tol, so the bar against
the FP64 oracle is the bound 2*dt*tol/rms(H) that any two solutions
converged to tol obey; the PT iteration counts stay close to FP64's (the
form keeps the iteration's fluxes across rebases)."""
import numpy as np
import pytest

import ptdiff
from oracle import oracle as O
from golden_cases import start_fields
from ptdiff import _abi
from ptdiff import scripts as S

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def run(s, shape, H0=None, **kw):
    H, Hold = start_fields(s, shape)
    if H0 is not None:
        H = np.array(H0, order="F", copy=True)
    D = S.step_field(s, *shape) if s.model == S.LINSTEP else None
    p = ptdiff.make_params(s, shape, precision="fp32_rb", **kw)
    with ptdiff.Solver(p) as sol:
        iters, eh, st = sol.solve(H, D, raise_on_nan=False, Hold=Hold)
    return H, D, iters, eh, st


@pytest.mark.parametrize("name,shape", [
    ("diff_1D_lin", (128,)), ("diff_1D_linstep", (200,)), ("diff_1D_nonlin", (97,)), ("diff_1D_react", (64,)),
    ("diff_2D_lin", (64, 64)), ("diff_2D_linstep", (66, 33)), ("diff_2D_nonlin", (64, 64)),
    ("diff_2D_react", (64, 64)),
    ("diff_2D_nonlin", (3, 3)), ("diff_2D_nonlin", (37, 95)),
    ("diff_3D_lin_multixpu", (24, 24, 24)), ("diff_3D_linstep_multixpu", (3, 4, 5)),
    ("diff_3D_nonlin_multixpu", (32, 30, 34)), ("diff_3D_linstep_multixpu", (40, 36, 50))])
def test_rebased_fp32_matches_oracle(name, shape):
    s = S.SCRIPTS[name]
    H, D, iters, eh, st = run(s, shape)
    H0, Hold0 = start_fields(s, shape)
    Hr, it_r, _, st_r = O.solve(s, H0, D, Hold0=Hold0)
    assert st == 0 and st_r == 0
    rms = float(np.sqrt(np.mean(np.square(Hr))))
    assert rel_l2(H, Hr) <= 2 * s.dt * s.tol / rms
    # close to the FP64 counts: a few extra check blocks at most per step
    assert np.all(iters <= it_r + 6 * s.nout + 20), (list(iters), list(it_r))
    assert len(eh) > 0 and eh[-1] <= s.tol


@pytest.mark.parametrize("name,shape", [("diff_2D_nonlin_perf", (64, 64)), ("diff_3D_nonlin_perf", (32, 32, 32))])
def test_rebased_fp32_fixed_iterations(name, shape):
    """Perf scripts (nchk > itmax): exactly itmax PT iterations per step, no
    checks; FP32 changes on an FP64 base track the FP64 iterates closely."""
    s = S.SCRIPTS[name]
    H, D, iters, eh, st = run(s, shape)
    Hr, it_r, _, _ = O.solve(s, S.initial_condition(s, *shape), D)
    assert list(iters) == list(it_r) == [s.itmax] * s.nt
    assert len(eh) == 0
    assert rel_l2(H, Hr) <= 1e-6


@pytest.mark.parametrize("name,shape", [("2d_nonlin_4096", (512, 512)), ("3d_nonlin_512", (64, 64, 64))])
def test_rebased_fp32_benchmark_problems(name, shape):
    """The benchmark problems (H0 = 1 + exp(-r^2), Dirichlet H = 1) at reduced
    size: against the GPU FP64 solve."""
    s = ptdiff.scripts.CONFIGS[name]
    H, _, iters, _, st = run(s, shape, nt=2)
    H64 = S.initial_condition(s, *shape)
    with ptdiff.Solver(ptdiff.make_params(s, shape, nt=2)) as sol:
        it64, _, st64 = sol.solve(H64)
    assert st == 0 and st64 == 0
    rms = float(np.sqrt(np.mean(np.square(H64))))
    assert rel_l2(H, H64) <= 2 * s.dt * s.tol / rms
    assert np.all(np.abs(iters.astype(int) - it64.astype(int)) <= 3 * s.nout), (list(iters), list(it64))


def test_rebased_fp32_nan_and_strict():
    s = S.SCRIPTS["diff_2D_nonlin"]
    H0 = S.initial_condition(s, 40, 40)
    H0[20, 20] = np.nan
    _, _, _, _, st = run(s, (40, 40), H0=H0)
    assert st == _abi.PTD_ENAN
    _, _, iters, _, st = run(S.SCRIPTS["diff_2D_lin"], (64, 64), itmax=30, strict=True)
    assert st == _abi.PTD_ENOTCONV
    assert list(iters) == [30] * 5


def test_rebased_fp32_device_pointers_and_iterate():
    torch = pytest.importorskip("torch")
    s = S.SCRIPTS["diff_3D_nonlin_multixpu"]
    shape = (33, 28, 30)
    H0 = S.initial_condition(s, *shape)
    Hd = torch.from_numpy(np.ravel(H0, order="F").copy()).cuda()
    p = ptdiff.make_params(s, shape, precision="fp32_rb")
    with ptdiff.Solver(p) as sol:
        iters, _, st = sol.solve(Hd)
        sol.set_state(H0)
        sol.iterate(25)   # fixed iterations (perf protocol), folded into the FP64 state
        Hi = sol.get_state()
    Hr, _, _, _ = O.solve(s, H0)
    assert st == 0
    rms = float(np.sqrt(np.mean(np.square(Hr))))
    assert rel_l2(Hd.cpu().numpy(), np.ravel(Hr, order="F")) <= 2 * s.dt * s.tol / rms
    H25 = np.array(H0, order="F")
    q = [np.zeros_like(H25) for _ in range(3)]
    O.iterate(s, H25, H0.copy(order="F"), q, 25)
    assert rel_l2(Hi, np.ravel(H25, order="F") if Hi.ndim == 1 else H25) <= 1e-5


@pytest.mark.parametrize("name,shape,kw,okw", [
    ("diff_2D_nonlin", (50, 61), {"norm": "max"}, {"norm": 1}),
    ("diff_2D_linstep", (66, 33), {"nchk": 7}, {"nout": 7}),
    ("diff_3D_nonlin_multixpu", (30, 31, 29), {"nchk": 3}, {"nout": 3}),
    ("diff_2D_lin", (64, 64), {"nchk": 10, "itmax": 95}, {"nout": 10, "itmax": 95}),
    ("diff_2D_nonlin", (64, 64), {"nchk": 1}, {"nout": 1})])
def test_rebased_fp32_driver_options(name, shape, kw, okw):
    s = S.SCRIPTS[name]
    H, D, iters, eh, st = run(s, shape, **kw)
    Hr, it_r, _, st_r = O.solve(s, S.initial_condition(s, *shape), D, **okw)
    assert st == 0 and st_r == 0
    rms = float(np.sqrt(np.mean(np.square(Hr))))
    assert rel_l2(H, Hr) <= 2 * s.dt * s.tol / rms
    nchk = kw.get("nchk", s.nout)
    assert np.all(iters <= it_r + 6 * nchk + 20) and np.all(iters % nchk == 0), (list(iters), list(it_r))


@pytest.mark.parametrize("shape", [(40, 44), (24, 26, 22)])
def test_rebased_fp32_expm_model_matches_fp64(shape):
    """D = exp(m) H^3 (the adjoint's model) with a seeded log-coefficient field."""
    base = S.SCRIPTS["diff_2D_nonlin" if len(shape) == 2 else "diff_3D_nonlin_multixpu"]
    s = base.with_(name="expm", model=S.NONLIN_EXPM, shift=1.0, dirichlet=1.0, ic="linrange", ttot=0.4)
    m = np.asfortranarray(S.log_coefficient_field(shape, lengths=(10.0,) * len(shape), seed=3))
    out = {}
    for prec in ("fp64", "fp32_rb"):
        H = S.initial_condition(s, *shape)
        with ptdiff.Solver(ptdiff.make_params(s, shape, precision=prec)) as sol:
            iters, _, st = sol.solve(H, m)
        assert st == 0
        out[prec] = (H, iters)
    (H64, it64), (H32, it32) = out["fp64"], out["fp32_rb"]
    rms = float(np.sqrt(np.mean(np.square(H64))))
    assert rel_l2(H32, H64) <= 2 * s.dt * s.tol / rms
    assert np.all(np.abs(it32.astype(int) - it64.astype(int)) <= 3 * s.nout)


# 2D FP32 iterations run two per launch (temporal blocking) when the check
# cadence is even; each iteration's arithmetic is the one-per-launch
# kernel's, so the two agree to the order of the residual reduction.
@pytest.mark.parametrize("name,shape,kw", [
    ("diff_2D_lin", (64, 64), {}), ("diff_2D_linstep", (66, 33), {}), ("diff_2D_nonlin", (97, 130), {}),
    ("diff_2D_nonlin", (3, 3), {}), ("diff_2D_linstep", (200, 7), {}), ("diff_2D_lin", (31, 250), {}),
    ("diff_2D_react", (64, 64), {}), ("diff_2D_nonlin", (58, 60), {"nchk": 2}),
    ("diff_2D_nonlin", (64, 64), {"nchk": 10, "itmax": 95}), ("diff_2D_nonlin_perf", (64, 64), {"itmax": 33}),
    # LIN and NONLIN run two columns per lane (60 per warp): several tiles, a last
    # face at the 62nd column of a tile (nx = 60 t + 62), widths around the pitch
    ("diff_2D_nonlin", (122, 40), {}), ("diff_2D_lin", (182, 61), {}), ("diff_2D_nonlin", (256, 96), {}),
    ("diff_2D_nonlin", (121, 33), {}), ("diff_2D_lin", (63, 70), {})])
def test_rebased_fp32_temporal_blocking_matches_one_iteration_per_launch(name, shape, kw):
    s = S.SCRIPTS[name]
    H2, _, it2, _, st2 = run(s, shape, **kw)
    H1, _, it1, _, st1 = run(s, shape, dc_tblock=False, **kw)
    assert st1 == 0 and st2 == 0
    assert list(it1) == list(it2)
    assert rel_l2(H2, H1) <= 1e-12


# 3D LIN and NONLIN likewise with PTD_FLAG_RB_TBLOCK_3D (z temporal blocking, rb3d_tb2_kernel): grids
# of one z chunk and of several (the march of each chunk starts two planes
# below it), ragged x/y tiles, odd check cadences (one iteration per
# launch), itmax not a multiple of nchk, the fixed-iteration protocol.
@pytest.mark.parametrize("name,shape,kw", [
    ("diff_3D_lin_multixpu", (34, 30, 28), {}), ("diff_3D_nonlin_multixpu", (40, 33, 45), {}),
    ("diff_3D_nonlin_multixpu", (3, 3, 3), {}), ("diff_3D_nonlin_multixpu", (70, 17, 21), {"nchk": 2}),
    ("diff_3D_nonlin_multixpu", (30, 31, 64), {"nchk": 10, "itmax": 95}),
    ("diff_3D_nonlin_multixpu", (29, 45, 36), {"nchk": 5}),
    ("diff_3D_nonlin_perf", (32, 32, 32), {"itmax": 33}), ("diff_3D_lin_multixpu", (60, 4, 100), {})])
def test_rebased_fp32_3d_temporal_blocking_matches_one_iteration_per_launch(name, shape, kw):
    s = S.SCRIPTS[name]
    H2, _, it2, _, st2 = run(s, shape, rb_tblock_3d=True, **kw)
    H1, _, it1, _, st1 = run(s, shape, **kw)
    assert st1 == 0 and st2 == 0
    assert list(it1) == list(it2)
    assert rel_l2(H2, H1) <= 1e-12


def test_rebased_fp32_3d_temporal_blocking_fixed_iterations():
    """Fixed iterations (the perf protocol): the two-iteration launches give
    the iterates of one-iteration launches, odd counts included."""
    s = S.SCRIPTS["diff_3D_nonlin_multixpu"]
    shape = (48, 40, 52)
    out = []
    for tblock in (True, False):
        with ptdiff.Solver(ptdiff.make_params(s, shape, precision="fp32_rb", rb_tblock_3d=tblock)) as sol:
            H = S.initial_condition(s, *shape)
            sol.set_state(H)
            sol.iterate(37)
            out.append(sol.get_state())
    assert rel_l2(out[0], out[1]) <= 1e-13


def test_rebased_fp32_temporal_blocking_expm_and_iterate():
    """D = exp(m) H^3 with temporal blocking, and odd fixed-iteration counts
    (a single-iteration launch finishes them)."""
    base = S.SCRIPTS["diff_2D_nonlin"]
    s = base.with_(name="expm", model=S.NONLIN_EXPM, shift=1.0, dirichlet=1.0, ic="linrange", ttot=0.4)
    shape = (61, 47)
    m = np.asfortranarray(S.log_coefficient_field(shape, lengths=(10.0, 10.0), seed=5))
    out = []
    for tblock in (True, False):
        H = S.initial_condition(s, *shape)
        with ptdiff.Solver(ptdiff.make_params(s, shape, precision="fp32_rb", dc_tblock=tblock)) as sol:
            iters, _, st = sol.solve(H, m)
            assert st == 0
            H2 = S.initial_condition(s, *shape)
            sol.set_state(H2, m)
            sol.iterate(37)
            Hi = sol.get_state()
        out.append((H, iters, Hi))
    (Ha, ia, Hia), (Hb, ib, Hib) = out
    assert list(ia) == list(ib)
    assert rel_l2(Ha, Hb) <= 1e-12
    assert rel_l2(Hia, Hib) <= 1e-12


@pytest.mark.parametrize("prec,name,shape", [
    ("fp64", "2d_nonlin_4096", (384, 384)), ("dfh", "2d_nonlin_4096", (384, 384)),
    ("fp64", "3d_nonlin_512", (64, 64, 64)), ("df64", "3d_nonlin_512", (64, 64, 64)),
    ("fp32_rb", "2d_nonlin_4096", (384, 384)), ("fp32_rb", "3d_nonlin_512", (64, 64, 64)),
    ("fp32_rb", "1d_lin_512", (512,)),
    ("fp32_dc", "2d_nonlin_4096", (384, 384)), ("fp32_dc", "3d_nonlin_512", (64, 64, 64)),
    ("fp32_dc", "1d_lin_512", (512,))])
def test_check_residual_is_deterministic(prec, name, shape):
    """The check residual is summed from per-warp / per-block slots in a fixed
    order: two solves of the same problem give the same error history bit for
    bit (and so the same stopping iterations)."""
    s = S.CONFIGS[name]
    out = []
    for _ in range(2):
        H = S.initial_condition(s, *shape)
        with ptdiff.Solver(ptdiff.make_params(s, shape, nt=2, precision=prec)) as sol:
            iters, eh, st = sol.solve(H)
        assert st == 0
        out.append((list(iters), np.asarray(eh).copy(), H))
    (i1, e1, h1), (i2, e2, h2) = out
    assert i1 == i2
    assert np.array_equal(e1, e2)
    assert np.array_equal(np.ravel(h1), np.ravel(h2))


@pytest.mark.parametrize("name,shape,nchk", [("2d_nonlin_4096", (256, 256), 100), ("3d_nonlin_512", (48, 48, 48), 10),
                                             ("2d_nonlin_4096", (200, 180), 7)])
def test_rebased_step_launches_no_kernel_past_its_stop(name, shape, nchk):
    """A step is one graph launch: one check block per pass of its loop, the
    FP64 rebase in an IF node opened at the end of a phase.  Its launches are
    its PT launches (iterations / iterations per launch) plus a few
    bookkeeping kernels per check block and per rebase, and at most one idle
    check block (odd launch counts)."""
    s = S.CONFIGS[name]
    H = S.initial_condition(s, *shape)
    with ptdiff.Solver(ptdiff.make_params(s, shape, nt=2, nchk=nchk, precision="fp32_rb")) as sol:
        l0, _ = sol.counters()
        iters, _, st = sol.solve(H)
        l1, _ = sol.counters()
    assert st == 0
    tb = 2 if len(shape) == 2 and nchk % 2 == 0 else 1
    bound = sum(it // tb + 6 * (it // nchk + 2) + nchk for it in (int(v) for v in iters))
    assert 0 < l1 - l0 <= bound, (l1 - l0, list(iters))
