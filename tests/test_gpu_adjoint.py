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
