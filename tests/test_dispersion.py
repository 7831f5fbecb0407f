"""The PT iteration parameters from the reference's dispersion analysis
(dispersion_analysis/dispersion_analysis_transient_diffusion1D.m): the
closed-form Re_opt is the critically damped value, maximises the decay rate
of the slowest mode, and is the Re of the solver scripts."""
import math

import numpy as np
import pytest

from ptdiff import dispersion as DP
from ptdiff import scripts as S


@pytest.mark.parametrize("da", [0.0, 1.0, 25.0, 500.0, 1e4])
def test_re_opt_is_critically_damped_and_fastest(da):
    re = DP.re_opt(da)
    lam = DP.dispersion_roots(re, da)
    assert np.allclose(lam[0], lam[1], rtol=1e-6, atol=1e-6)            # double root
    assert abs((re + da / re) ** 2 - 4 * (math.pi ** 2 + da)) <= 1e-9 * re ** 2
    grid = np.linspace(0.5 * re, 2.0 * re, 301)
    rates = [DP.decay_rate(r, da, kmax=8) for r in grid]
    assert abs(grid[int(np.argmax(rates))] - re) <= 0.01 * re           # the maximum of the spectral abscissa


def test_stationary_limit_is_two_pi():
    assert DP.re_opt(0.0) == pytest.approx(2 * math.pi)


@pytest.mark.parametrize("name", ["diff_1D_lin", "diff_2D_lin", "diff_3D_lin_multixpu"])
def test_scripts_use_re_opt(name):
    s = S.SCRIPTS[name]
    L = max(s.lx, s.ly, s.lz) if s.ndim > 1 else s.lx
    da = DP.damkohler(L, s.D, s.dt)
    assert DP.re_opt(da) == pytest.approx(math.pi + math.sqrt(math.pi ** 2 + L * L / s.D / s.dt))
