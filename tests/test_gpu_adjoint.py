"""Adjoint gradients (ptd_adj_*): against the CPU FP64 reference adjoint of
the oracle (itself pinned by finite differences, tests/test_oracle.py) and
against central finite differences of the library's own forward solve, in
random directions.  Bar: 1e-6 relative."""
import numpy as np
import pytest

import ptdiff
from oracle import oracle as O
from ptdiff import scripts as S

pytestmark = pytest.mark.gpu


def problem(shape=(14, 13, 12), model=S.NONLIN_EXPM, nt=3):
    base = S.SCRIPTS["diff_3D_nonlin_multixpu"]
    s = base.with_(name="adj", model=model, shift=1.0, dirichlet=1.0, ttot=0.1 * nt, dt=0.1, tol=1e-12,
                   itmax=200000, ic="linrange")
    H0 = S.initial_condition(s, *shape)
    m = S.log_coefficient_field(shape, seed=1) if model == S.NONLIN_EXPM else None
    mt = (m if m is not None else 0.0) + 0.3 * S.log_coefficient_field(shape, seed=2)
    Ht = O.forward_checkpoints(s.with_(model=S.NONLIN_EXPM), H0, mt)[-1]
    return s, H0, m, Ht


def make(s, shape, prec):
    p = ptdiff.make_params(s, shape, precision=prec, nchk=10)
    return ptdiff.AdjointSolver(p)


@pytest.mark.parametrize("prec", ["fp64", "df64", "fp32_rb"])
@pytest.mark.parametrize("model", [S.NONLIN_EXPM, S.NONLIN])
def test_adjoint_matches_reference_adjoint(prec, model):
    shape = (14, 13, 12)
    s, H0, m, Ht = problem(shape, model)
    with make(s, shape, prec) as A:
        loss, HN = A.forward(H0, m, Ht, want_HN=True)
        gm, gh = A.gradient()
    Hs = O.forward_checkpoints(s, H0, m)
    assert np.linalg.norm(HN - Hs[-1]) <= 1e-10 * np.linalg.norm(Hs[-1])
    d = (Hs[-1] - Ht)[1:-1, 1:-1, 1:-1]
    assert abs(loss - 0.5 * np.sum(d * d)) <= 1e-9 * loss
    gm_r, gh_r, st = O.adjoint(s, Hs, Ht, m)
    assert st == 0
    if model == S.NONLIN_EXPM:
        assert np.linalg.norm(gm - gm_r) <= 1e-6 * np.linalg.norm(gm_r)
    assert np.linalg.norm(gh - gh_r) <= 1e-6 * np.linalg.norm(gh_r)


@pytest.mark.parametrize("prec", ["fp64", "df64", "fp32_rb"])
def test_adjoint_matches_finite_differences(prec):
    shape = (14, 13, 12)
    s, H0, m, Ht = problem(shape)
    rng = np.random.default_rng(11)
    with make(s, shape, prec) as A:
        A.forward(H0, m, Ht)
        gm, gh = A.gradient()
        def fd(f, eps=1e-4):
            # central differences at eps and eps/2, Richardson-combined (O(eps^4))
            d1 = (f(eps) - f(-eps)) / (2 * eps)
            d2 = (f(eps / 2) - f(-eps / 2)) / eps
            return (4 * d2 - d1) / 3

        for _ in range(3):
            dm = rng.standard_normal(shape)
            g = fd(lambda e: A.forward(H0, m + e * dm, Ht))
            assert abs(g - np.sum(gm * dm)) <= 1e-6 * abs(g)
            dh = rng.standard_normal(shape)
            g = fd(lambda e: A.forward(H0 + e * dh, m, Ht))
            assert abs(g - np.sum(gh * dh)) <= 1e-6 * abs(g)


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    shape = (14, 13, 12)
    s, H0, m, Ht = problem(shape)
    with make(s, shape, "df64") as A:
        F = ptdiff.misfit_function()
        tt = lambda a: torch.from_numpy(np.ascontiguousarray(a.transpose(2, 1, 0))).cuda()
        mt = tt(m).requires_grad_(True)
        h0 = tt(H0).requires_grad_(True)
        L = F.apply(mt, h0, tt(Ht), A)
        L.backward()
        gm, gh = A.gradient()
    assert np.allclose(mt.grad.cpu().numpy().transpose(2, 1, 0), gm)
    assert np.allclose(h0.grad.cpu().numpy().transpose(2, 1, 0), gh)


@pytest.mark.parametrize("prec", ["fp64", "fp32_rb"])
def test_adjoint_odd_check_cadence_matches_reference_adjoint(prec):
    """An odd check cadence: every pass of a solve graph's loop holds two check
    blocks, so that each pass starts on the same buffer parity."""
    shape = (14, 13, 12)
    s, H0, m, Ht = problem(shape)
    with ptdiff.AdjointSolver(ptdiff.make_params(s, shape, precision=prec, nchk=7)) as A:
        A.forward(H0, m, Ht)
        gm, gh = A.gradient()
    Hs = O.forward_checkpoints(s, H0, m)
    gm_r, gh_r, st = O.adjoint(s, Hs, Ht, m)
    assert st == 0
    assert np.linalg.norm(gm - gm_r) <= 1e-6 * np.linalg.norm(gm_r)
    assert np.linalg.norm(gh - gh_r) <= 1e-6 * np.linalg.norm(gh_r)


@pytest.mark.parametrize("prec", ["fp64", "df64", "fp32_rb"])
def test_adjoint_is_deterministic(prec):
    """Every norm of the adjoint (check residuals, right-hand sides, rebase
    residuals, the loss) is summed from per-CTA slots in a fixed order: two
    gradient evaluations agree bit for bit."""
    shape = (14, 13, 12)
    s, H0, m, Ht = problem(shape)
    out = []
    for _ in range(2):
        with make(s, shape, prec) as A:
            loss = A.forward(H0, m, Ht)
            gm, gh = A.gradient()
            out.append((loss, gm, gh, list(A.adjoint_iters)))
    (l1, m1, h1, i1), (l2, m2, h2, i2) = out
    assert l1 == l2 and i1 == i2
    assert np.array_equal(m1, m2) and np.array_equal(h1, h2)


@pytest.mark.parametrize("prec,nchk", [("fp64", 10), ("fp32_rb", 10), ("fp64", 7), ("fp32_rb", 7)])
def test_adjoint_solves_launch_no_block_past_their_stop(prec, nchk):
    """Each adjoint solve is one graph launch whose loop the device ends: the
    PT launches of a gradient are its iterations plus at most one idle check
    block per solve (odd cadences), with a few bookkeeping kernels per check
    block and per step."""
    shape = (14, 13, 12)
    s, H0, m, Ht = problem(shape)
    with ptdiff.AdjointSolver(ptdiff.make_params(s, shape, precision=prec, nchk=nchk)) as A:
        A.forward(H0, m, Ht)
        l0, _ = A.counters()
        A.gradient()
        l1, _ = A.counters()
        its = [int(v) for v in A.adjoint_iters]
    per_step = [it + (it // nchk + 1) * 5 + nchk + 10 for it in its]
    assert 0 < l1 - l0 <= sum(per_step), (l1 - l0, its)
