"""Iteration parameters of the accelerated PT method from its dispersion
analysis, and an empirical search of the residual-scaling factor.

The reference derives its Reynolds number symbolically
(dispersion_analysis/dispersion_analysis_transient_diffusion1D.m:1-27,
..._stationary_diffusion1D.m): with the PT equations
    rho dH/dtau + dq/dx + rho_ph H/dt = 0,    theta_r dq/dtau + q + D dH/dx = 0,
the wave speed V_p = sqrt(D/(rho theta_r)), Re = rho V_p L/D and
Da = L^2 rho_ph/(D dt), a Fourier mode H ~ exp(-lambda V_p tau/L) sin(pi k x/L)
satisfies
    lambda^2 - (Re + Da/Re) lambda + (pi^2 k^2 + Da) = 0.
The slowest mode (k = 1) decays fastest when the discriminant vanishes
(critical damping): Re_opt = pi + sqrt(pi^2 + Da), the value every solver
script uses (e.g. scripts/diff_2D_lin.jl:51).  This module restates that
relation numerically and adds `tune_resc`, the empirical counterpart for the
nonlinear models (whose scripts scale Re by Resc = 1/1.2): it times a few
candidate factors on a coarse grid through the GPU library and keeps the one
with the fewest PT iterations.
"""
from __future__ import annotations

import math

import numpy as np


def re_opt(da: float) -> float:
    """Critically damped Reynolds number of the slowest mode (k = 1)."""
    return math.pi + math.sqrt(math.pi ** 2 + da)


def damkohler(L: float, D: float, dt: float, rho_ph: float = 1.0) -> float:
    """Da = L^2 rho_ph / (D dt) of the transient problem (0: stationary)."""
    return L * L * rho_ph / (D * dt) if dt > 0 else 0.0


def dispersion_roots(re: float, da: float, k: int = 1) -> np.ndarray:
    """Roots lambda of lambda^2 - (Re + Da/Re) lambda + (pi^2 k^2 + Da) = 0."""
    return np.roots([1.0, -(re + da / re), math.pi ** 2 * k * k + da])


def decay_rate(re: float, da: float, kmax: int = 64) -> float:
    """Spectral abscissa: the smallest real part of the roots over the modes
    k = 1..kmax, the asymptotic convergence rate of the PT iteration per unit
    of scaled pseudo-time (larger is faster)."""
    return min(float(np.min(dispersion_roots(re, da, k).real)) for k in range(1, kmax + 1))


def tune_resc(script, shape, candidates=(0.5, 0.6, 0.7, 0.8, 1.0 / 1.2, 0.9, 1.0, 1.1), precision="fp64",
              nt: int = 1, **params):
    """Empirical search of the Re scaling factor (the scripts' Resc) for a
    script on a (coarse) grid: one solve per candidate through the GPU
    library, keeping the candidate with the fewest PT iterations (ties: the
    one closest to the script's own value).  Returns (best, {resc: iters})."""
    from .solvers import Solver, make_params
    from .scripts import LINSTEP, initial_condition, step_field

    counts = {}
    for r in candidates:
        H = initial_condition(script, *shape)
        D = step_field(script, *shape) if script.model == LINSTEP else None
        p = make_params(script, shape, nt=nt, precision=precision, **params)
        p.resc = float(r)
        with Solver(p) as sol:
            iters, _, st = sol.solve(H, D, raise_on_nan=False)
        if st == 0:
            counts[float(r)] = int(np.sum(iters))
    if not counts:
        raise RuntimeError("tune_resc: no candidate converged")
    best = min(counts, key=lambda r: (counts[r], abs(r - script.resc)))
    return best, counts
