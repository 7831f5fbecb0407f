"""Batched solves (ptd_batch_*): every instance must match the one-grid
oracle run of its own problem -- equal PT iteration counts and relative L2
error <= 1e-10 for FP64/DF64; the converged-to-tol bound for FP32_DC and
FP32_RB (whose counts also stay within 1 % plus two check blocks of the
oracle's, and equal those of the one-grid FP32_RB solver)."""
import numpy as np
import pytest

import ptdiff
from oracle import oracle as O
from ptdiff import scripts as S

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def oracle_instance(model, H0, D, **kw):
    base = S.SCRIPTS["diff_2D_linstep" if model == S.LINSTEP else "diff_2D_nonlin"
                     if model == S.NONLIN else "diff_2D_lin"]
    s = base.with_(**kw)
    return O.solve(s, H0, D)


@pytest.mark.parametrize("prec", ["fp64", "df64", "fp32_dc", "fp32_rb"])
@pytest.mark.parametrize("model", [S.LINSTEP, S.NONLIN])
def test_batch_matches_oracle(prec, model):
    sizes, Hs, Ds = ptdiff.batch_instances(7, seed=3, nmin=12, nmax=90)
    Hs0 = [H.copy(order="F") for H in Hs]
    if model != S.LINSTEP:
        Ds = None
    nt = 2
    p = ptdiff.batch_params(len(sizes), model=model, precision=prec, nt=nt,
                            resc=(1 / 1.2 if model == S.NONLIN else 1.0))
    with ptdiff.BatchSolver(p, sizes, sizes) as b:
        iters, err = b.solve(Hs, Ds)
        launches, its = b.counters()
    assert launches > 0 and its > 0
    for k in range(len(sizes)):
        Hr, it_r, _, st = oracle_instance(model, Hs0[k], None if Ds is None else Ds[k], ttot=0.2 * nt,
                                          resc=p.resc)
        assert st == 0
        if prec == "fp32_rb":
            for a, b_ in zip(iters[k], it_r):
                assert abs(int(a) - int(b_)) <= 0.01 * b_ + 2 * p.nchk, (iters[k], it_r)
        if prec in ("fp32_dc", "fp32_rb"):
            rms = float(np.sqrt(np.mean(np.square(Hr))))
            Ht, _, _, _ = oracle_instance(model, Hs0[k], None if Ds is None else Ds[k], ttot=0.2 * nt,
                                          resc=p.resc, tol=1e-11)
            assert rel_l2(Hs[k], Ht) <= 2 * 0.2 * 1e-8 / rms
            assert err[k] <= 1e-8
        else:
            assert list(iters[k]) == list(it_r)
            assert rel_l2(Hs[k], Hr) <= 1e-10


@pytest.mark.parametrize("prec", ["fp64", "fp32_dc"])
def test_batch_autotuner(prec):
    sizes, Hs, Ds = ptdiff.batch_instances(5, seed=4, nmin=40, nmax=200)
    Hs0 = [H.copy(order="F") for H in Hs]
    p = ptdiff.batch_params(len(sizes), model=S.LINSTEP, precision=prec, nt=1)
    with ptdiff.BatchSolver(p, sizes, sizes) as b:
        w, c, us = b.tune()
        assert w in (2, 4, 8) and c in (16, 32, 64, 128) and us > 0
        assert b.config()[:2] == (w, c) and b.config()[2] in ((1, 2) if prec == "fp32_dc" else (1,))
        iters, err = b.solve(Hs, Ds)
    for k in range(len(sizes)):
        Hr, it_r, _, _ = oracle_instance(S.LINSTEP, Hs0[k], Ds[k], ttot=0.2)
        if prec == "fp64":
            assert list(iters[k]) == list(it_r)
            assert rel_l2(Hs[k], Hr) <= 1e-10
        else:
            assert err[k] <= 1e-8


@pytest.mark.parametrize("model", [S.LIN, S.LINSTEP, S.NONLIN])
def test_batch_temporal_blocking_matches_one_iteration_per_launch(model):
    """FP32_DC: two inner iterations per launch give the per-launch kernel's
    iterations (same arithmetic per iteration) on uneven instances."""
    from ptdiff import _abi

    sizes, Hs, Ds = ptdiff.batch_instances(6, seed=5, nmin=3, nmax=140)
    if model != S.LINSTEP:
        Ds = None
    out = []
    for flags in (0, _abi.FLAG_DC_NO_TBLOCK):
        H = [h.copy(order="F") for h in Hs]
        p = ptdiff.batch_params(len(sizes), model=model, precision="fp32_dc", nt=2, flags=flags,
                                resc=(1 / 1.2 if model == S.NONLIN else 1.0))
        with ptdiff.BatchSolver(p, sizes, sizes) as b:
            assert b.config()[2] == (1 if flags else 2)
            iters, err = b.solve(H, Ds)
        out.append((H, iters))
    (H2, it2), (H1, it1) = out
    assert np.array_equal(it1, it2)
    for k in range(len(sizes)):
        assert rel_l2(H2[k], H1[k]) <= 1e-12


@pytest.mark.parametrize("model", [S.LIN, S.LINSTEP, S.NONLIN])
@pytest.mark.parametrize("flags", [0, "no_tblock"])
def test_batch_rebased_matches_one_grid_solver(model, flags):
    """FP32_RB: each instance of the batch takes the PT iterations of the
    one-grid FP32_RB solver on its own problem (the same FP32 iterations,
    rebases and stopping rule) and returns its H; one- and two-iteration
    launches alike, on uneven instances down to 3 x 3."""
    from ptdiff import _abi

    fl = 0 if flags == 0 else _abi.FLAG_DC_NO_TBLOCK
    sizes, Hs, Ds = ptdiff.batch_instances(6, seed=6, nmin=3, nmax=130)
    if model != S.LINSTEP:
        Ds = None
    resc = 1 / 1.2 if model == S.NONLIN else 1.0
    H = [h.copy(order="F") for h in Hs]
    p = ptdiff.batch_params(len(sizes), model=model, precision="fp32_rb", nt=2, flags=fl, resc=resc)
    with ptdiff.BatchSolver(p, sizes, sizes) as b:
        assert b.config()[2] == (1 if fl else 2)
        iters, err = b.solve(H, Ds)
    base = S.SCRIPTS["diff_2D_linstep" if model == S.LINSTEP else "diff_2D_nonlin"
                     if model == S.NONLIN else "diff_2D_lin"]
    for k in range(len(sizes)):
        s = base.with_(ttot=0.4, resc=resc)
        shape = (int(sizes[k]), int(sizes[k]))
        H1 = Hs[k].copy(order="F")
        with ptdiff.Solver(ptdiff.make_params(s, shape, precision="fp32_rb", dc_tblock=not fl)) as sol:
            it1, _, st = sol.solve(H1, None if Ds is None else Ds[k])
        assert st == 0
        assert list(iters[k]) == list(it1), (k, list(iters[k]), list(it1))
        assert rel_l2(H[k], H1) <= 1e-12
        assert err[k] <= 1e-8


def test_batch_device_tensors_match_host_arrays():
    """H and D handed over as device tensors (the fields stay on the GPU) give
    the host arrays' result."""
    import torch

    sizes, Hs, Ds = ptdiff.batch_instances(4, seed=8, nmin=20, nmax=70)
    p = ptdiff.batch_params(len(sizes), model=S.LINSTEP, precision="fp32_rb", nt=1)
    Hh = [h.copy(order="F") for h in Hs]
    Hd = [torch.from_numpy(np.ravel(h, order="F").copy()).cuda() for h in Hs]
    Dd = [torch.from_numpy(np.ravel(d, order="F").copy()).cuda() for d in Ds]
    with ptdiff.BatchSolver(p, sizes, sizes) as b:
        it_h, _ = b.solve(Hh, Ds)
        it_d, _ = b.solve(Hd, Dd)
    assert np.array_equal(it_h, it_d)
    for k in range(len(sizes)):
        assert np.array_equal(np.ravel(Hh[k], order="F"), Hd[k].cpu().numpy())


@pytest.mark.parametrize("prec", ["fp32_rb", "fp64", "df64", "fp32_dc"])
def test_batch_is_deterministic(prec):
    """Every form of the batch sums its check residuals (and the FP64 residuals
    of the rebased and defect-correction forms) from per-warp / per-chunk
    slots in a fixed order, so two solves give the same iterations, residuals
    and H bit for bit."""
    sizes, Hs, Ds = ptdiff.batch_instances(5, seed=9, nmin=30, nmax=150)
    p = ptdiff.batch_params(len(sizes), model=S.LINSTEP, precision=prec, nt=2)
    out = []
    with ptdiff.BatchSolver(p, sizes, sizes) as b:
        for _ in range(2):
            H = [h.copy(order="F") for h in Hs]
            iters, err = b.solve(H, Ds)
            out.append((iters, err, H))
    (i1, e1, h1), (i2, e2, h2) = out
    assert np.array_equal(i1, i2)
    assert np.array_equal(e1, e2)
    for a, c in zip(h1, h2):
        assert np.array_equal(a, c)


def test_batch_set_config():
    """A launch shape set by hand is the one in use, and the solve it gives
    agrees with the tuned one to the converged-to-tol bound."""
    sizes, Hs, Ds = ptdiff.batch_instances(4, seed=10, nmin=20, nmax=100)
    p = ptdiff.batch_params(len(sizes), model=S.LINSTEP, precision="fp32_rb", nt=1)
    with ptdiff.BatchSolver(p, sizes, sizes) as b:
        Ha = [h.copy(order="F") for h in Hs]
        b.solve(Ha, Ds)
        b.set_config(4, 24, 1)
        assert b.config() == (4, 24, 1)
        Hb = [h.copy(order="F") for h in Hs]
        b.solve(Hb, Ds)
        with pytest.raises(ptdiff._abi.PtdError):
            b.set_config(3, 24, 1)
    for a, c in zip(Ha, Hb):
        rms = float(np.sqrt(np.mean(np.square(a))))
        assert rel_l2(c, a) <= 2 * 0.2 * 1e-8 / rms


@pytest.mark.parametrize("prec,nchk", [("fp64", 10), ("fp64", 7), ("fp32_dc", 10)])
def test_batch_launches_end_with_the_solve(prec, nchk):
    """A batch step is one graph launch whose loop the device ends once every
    instance has stopped: the PT launches are the largest instance's
    iterations plus at most one idle check block, with a few bookkeeping
    kernels per check block.  (The rebased batch runs phases of ~200
    iterations common to all instances, ended by the FP64 rebase of every
    running instance; its launches for an instance whose phase is over return
    after one load.)"""
    sizes, Hs, Ds = ptdiff.batch_instances(4, seed=12, nmin=24, nmax=96)
    p = ptdiff.batch_params(len(sizes), model=S.LINSTEP, precision=prec, nt=1, nchk=nchk, itmax=10000 * nchk)
    with ptdiff.BatchSolver(p, sizes, sizes) as b:
        l0, _ = b.counters()
        iters, _ = b.solve([h.copy(order="F") for h in Hs], Ds)
        l1, _ = b.counters()
    if prec == "fp32_dc":   # inner iterations of several inner solves: a loose bound
        assert 0 < l1 - l0 <= 3 * int(np.max(iters)) + 200
    else:
        m = int(np.max(iters))
        assert 0 < l1 - l0 <= m + 6 * (m // nchk + 2) + 2 * nchk + 20, (l1 - l0, m)
