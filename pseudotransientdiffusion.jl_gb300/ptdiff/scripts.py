"""The reference's solver scripts as data: parameters, grids, initial conditions.

Each entry of :data:`SCRIPTS` restates the hard-coded physics and numerics of
one reference driver function (``diffusion_1D_()`` / ``diffusion_2D_()`` /
``diffusion_3D_()``), so that :mod:`ptdiff.solvers` can run it through the
CUDA library with the same inputs the script would use:

============================  ==================================================
name                          reference (file:line of the driver's set-up block)
============================  ==================================================
diff_1D_lin                   scripts/diff_1D_lin.jl:33-61
diff_1D_linstep               scripts/diff_1D_linstep.jl:44-75
diff_1D_nonlin                scripts/diff_1D_nonlin.jl:40-63
diff_2D_lin                   scripts/diff_2D_lin.jl:36-65
diff_2D_linstep               scripts/diff_2D_linstep.jl:53-88
diff_2D_nonlin                scripts/diff_2D_nonlin.jl:46-74
diff_2D_nonlin_perf           scripts/diff_2D_nonlin_perf.jl:56-86
diff_3D_lin_multixpu          scripts/diff_3D/diff_3D_lin_multixpu.jl:44-87
diff_3D_linstep_multixpu      scripts/diff_3D/diff_3D_linstep_multixpu.jl:67-119
diff_3D_nonlin_multixpu       scripts/diff_3D/diff_3D_nonlin_multixpu.jl:57-99
diff_3D_nonlin_multixpu_perf  scripts/diff_3D/diff_3D_nonlin_multixpu_perf.jl:66-110
diff_3D_nonlin_perf           scripts/diff_3D/diff_3D_nonlin_perf.jl:61-93
============================  ==================================================

Grid sizes come from the NX/NY/NZ environment variables in the reference
(e.g. ``scripts/diff_2D_nonlin.jl:6-7``); here they are arguments.  The 3D
``*_multixpu`` scripts run on one rank (no MPI halo), where ImplicitGlobalGrid's
global coordinate is ``x_g(ix) = (ix-1)*dx`` and ``nx_g() = nx``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

LIN, LINSTEP, NONLIN, NONLIN_EXPM = 0, 1, 2, 3
MODEL_NAMES = {"lin": LIN, "linstep": LINSTEP, "nonlin": NONLIN, "nonlin_expm": NONLIN_EXPM}


@dataclass(frozen=True)
class Script:
    """Physics and numerics of one reference driver."""

    name: str
    ndim: int
    model: int
    lx: float = 10.0
    ly: float = 10.0
    lz: float = 10.0
    ttot: float = 1.0
    dt: float = 0.2
    tol: float = 1e-8
    itmax: int = 100000
    nout: int = 10
    cfl: float = 0.99
    resc: float = 1.0
    D: float = 1.0            # linear: D; step: D1 (the value outside the step)
    D2: float = 1e-4          # step: the value inside the step
    recip: bool = False       # reciprocal arithmetic of the *_perf scripts
    ic: str = "linrange"      # "linrange" (xc = LinRange) or "xg" (ImplicitGlobalGrid x_g)
    shift: float = 0.0        # H0 = shift + exp(-r^2) (the reference uses 0)
    dirichlet: float | None = None  # boundary cells set to this value (None: keep H0 there)
    react: bool = False       # reaction form: H starts at 0, Hold = Heq = H0, dt = theta_kin
    default_n: int = 512
    extra: dict = field(default_factory=dict)

    @property
    def nt(self) -> int:
        # nt = Int(ceil(ttot/dt))  (e.g. scripts/diff_2D_nonlin.jl:74)
        return int(math.ceil(self.ttot / self.dt))

    def with_(self, **kw) -> "Script":
        return replace(self, **kw)


_S2 = 1.0 / math.sqrt(2.0)
_S3 = 1.0 / math.sqrt(3.0)

SCRIPTS = {
    s.name: s
    for s in [
        Script("diff_1D_lin", 1, LIN, cfl=0.99, D=1.0),
        Script("diff_1D_linstep", 1, LINSTEP, cfl=0.99, D=1.0, D2=1e-4),
        Script("diff_1D_nonlin", 1, NONLIN, cfl=1.0),
        Script("diff_2D_lin", 2, LIN, cfl=_S2, D=1.0),
        Script("diff_2D_linstep", 2, LINSTEP, cfl=_S2, D=1.0, D2=1e-4),
        Script("diff_2D_nonlin", 2, NONLIN, cfl=_S2, resc=1.0 / 1.2),
        Script("diff_2D_nonlin_perf", 2, NONLIN, cfl=_S2, resc=1.0 / 1.2, ttot=0.4,
               itmax=100, nout=2000, recip=True),
        Script("diff_3D_lin_multixpu", 3, LIN, cfl=_S3, D=1.0, ic="xg", default_n=64),
        Script("diff_3D_linstep_multixpu", 3, LINSTEP, cfl=_S3, D=1.0, D2=1e-4, ic="xg",
               default_n=64),
        Script("diff_3D_nonlin_multixpu", 3, NONLIN, cfl=_S3, resc=1.0 / 1.2, ic="xg",
               default_n=64),
        Script("diff_3D_nonlin_multixpu_perf", 3, NONLIN, cfl=_S3, resc=1.0 / 1.2, ttot=0.4,
               itmax=1000, nout=2000, recip=True, ic="xg", default_n=64),
        Script("diff_3D_nonlin_perf", 3, NONLIN, cfl=_S3, resc=1.0 / 1.2, ttot=0.4,
               itmax=1000, nout=2000, recip=True, ic="linrange", default_n=64),
        # steady diffusion-reaction (scripts/diff_1D_react.jl:31-57, diff_2D_react.jl:33-60):
        # theta_kin = 0.1 plays dt, Heq = H0 plays Hold, H starts at 0, one PT loop
        Script("diff_1D_react", 1, LIN, lx=20.0, cfl=0.99, D=1.0, dt=0.1, ttot=0.1, react=True),
        Script("diff_2D_react", 2, LIN, cfl=_S2, D=1.0, dt=0.1, ttot=0.1, react=True),
    ]
}


def linrange(a: float, b: float, n: int) -> np.ndarray:
    """Julia's ``LinRange(a, b, n)`` element by element: ``(1-t)*a + t*b`` with
    ``t = j/(n-1)`` (Base ``lerpi``)."""
    if n == 1:
        return np.array([a], dtype=np.float64)
    j = np.arange(n, dtype=np.float64)
    t = j / float(n - 1)
    return (1.0 - t) * a + t * b


def cell_centres(length: float, n: int) -> np.ndarray:
    """``xc = LinRange(dx/2, lx - dx/2, nx)`` with ``dx = lx/nx`` (e.g. diff_2D_nonlin.jl:63)."""
    dx = length / n
    return linrange(dx / 2, length - dx / 2, n)


def _centred_sq(length: float, n: int, ic: str) -> np.ndarray:
    """(x - l/2)^2 at the cell centres, in the arithmetic of the script's IC line."""
    dx = length / n
    if ic == "xg":
        # (x_g(ix,dx,H0) - 0.5*lx + dx/2)^2, x_g = (ix-1)*dx  (diff_3D_nonlin_multixpu.jl:86)
        xg = np.arange(n, dtype=np.float64) * dx
        v = (xg - 0.5 * length) + dx / 2
        return v * v
    if ic == "linrange3":
        # (xc[ix] - 0.5*lx)^2 with scalar indexing (diff_3D/diff_3D_nonlin_perf.jl:89)
        v = cell_centres(length, n) - 0.5 * length
        return v * v
    # Broadcast over a LinRange: (xc .- lx/2) is itself a LinRange (diff_2D_nonlin.jl:71)
    v = linrange(dx / 2 - length / 2, (length - dx / 2) - length / 2, n)
    return v * v


def initial_condition(s: Script, nx: int, ny: int = 1, nz: int = 1) -> np.ndarray:
    """H0 of the script, indexed ``H[ix, iy, iz]`` and stored Fortran-ordered
    (x fastest), like the reference's Julia arrays."""
    ic = s.ic
    if s.ndim == 3 and ic == "linrange":
        ic = "linrange3"
    ax = _centred_sq(s.lx, nx, ic)
    if s.ndim == 1:
        H = np.exp(-ax)
    elif s.ndim == 2:
        ay = _centred_sq(s.ly, ny, ic)
        H = np.exp(-ax[:, None] - ay[None, :])
    else:
        ay = _centred_sq(s.ly, ny, ic)
        az = _centred_sq(s.lz, nz, ic)
        H = np.exp((-ax[:, None, None] - ay[None, :, None]) - az[None, None, :])
    H = np.asfortranarray(H)
    if s.shift != 0.0:
        H = H + s.shift
    H = np.asfortranarray(H)
    if s.dirichlet is not None:
        for d in range(s.ndim):
            lo = [slice(None)] * s.ndim
            lo[d] = 0
            H[tuple(lo)] = s.dirichlet
            lo[d] = -1
            H[tuple(lo)] = s.dirichlet
    return H


def step_field(s: Script, nx: int, ny: int = 1, nz: int = 1) -> np.ndarray:
    """The step model's cell diffusivity D (x fastest)."""
    shape = (nx,) if s.ndim == 1 else (nx, ny) if s.ndim == 2 else (nx, ny, nz)
    D = np.full(shape, s.D, dtype=np.float64, order="F")
    if s.ndim == 1:
        # D[1:Int(ceil(nx/2.2))] .= D2  (diff_1D_linstep.jl:69-70)
        D[: int(math.ceil(nx / 2.2))] = s.D2
    elif s.ndim == 2:
        # diff_2D_linstep.jl:82-83
        D[: int(math.ceil(nx / 2.2)), :] = s.D2
        D[:, : int(math.ceil(ny / 2.2))] = s.D2
    else:
        # coordinate rule x_g < lx/2.2 or y_g < ly/2.2 (diff_3D/diff_3D_linstep_multixpu.jl:99-104)
        dx, dy = s.lx / nx, s.ly / ny
        xg = np.arange(nx, dtype=np.float64) * dx
        yg = np.arange(ny, dtype=np.float64) * dy
        D[xg < s.lx / 2.2, :, :] = s.D2
        D[:, yg < s.ly / 2.2, :] = s.D2
    return D


def grid_shape(s: Script, nx: int, ny: int | None = None, nz: int | None = None):
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    if s.ndim == 1:
        return (nx,)
    if s.ndim == 2:
        return (nx, ny)
    return (nx, ny, nz)


def sample_indices(n: int, k: int = 12) -> np.ndarray:
    """``Int.(ceil.(LinRange(1, n, 12)))`` of the reference tests (test/test_2D.jl:19-20),
    returned 0-based."""
    return np.ceil(linrange(1.0, float(n), k)).astype(np.int64) - 1


def iteration_parameters(s: Script, shape) -> dict:
    """The scalar iteration parameters of the script (reference a1 block,
    e.g. scripts/diff_2D_lin.jl:49-53): dx, Vpdtau, L, Re, theta, dtau."""
    lengths = (s.lx, s.ly, s.lz)[: s.ndim]
    h = [lengths[d] / shape[d] for d in range(s.ndim)]
    vpdt = s.cfl * min(h)
    L = max(lengths)
    out = {"h": h, "vpdt": vpdt, "L": L}
    if s.model != NONLIN:
        Dre = s.D if s.model == LIN else max(s.D, s.D2)
        re = math.pi + math.sqrt(math.pi * math.pi + ((L * L / Dre) / s.dt))
        out.update(re=re, theta=(L / vpdt) / re)
        if s.model == LIN:
            out["dtau"] = ((vpdt * L) / s.D) / re
    return out


# The benchmark workloads: the reference scripts with H0 = 1 + exp(-r^2) and
# H = 1 held on the boundary cells (no reference counterpart for the
# nonlinear ones; the linear 1D case is an exact shift of diff_1D_lin).
CONFIGS = {
    "1d_lin_512": SCRIPTS["diff_1D_lin"].with_(name="1d_lin_512", shift=1.0, dirichlet=1.0,
                                               default_n=512),
    "2d_nonlin_4096": SCRIPTS["diff_2D_nonlin"].with_(name="2d_nonlin_4096", shift=1.0, dirichlet=1.0,
                                                      nout=100, default_n=4096),
    "3d_nonlin_512": SCRIPTS["diff_3D_nonlin_multixpu"].with_(name="3d_nonlin_512", shift=1.0,
                                                              dirichlet=1.0, ttot=0.6, ic="linrange",
                                                              default_n=512),
}


def log_coefficient_field(shape, lengths=(10.0, 10.0, 10.0), corr=1.0, std=0.3, seed=0):
    """Smooth Gaussian random field m (cell centres, x fastest): white noise
    filtered in Fourier space by a Gaussian kernel of correlation length
    `corr`, rescaled to standard deviation `std`; seeded."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal(shape)
    k2 = np.zeros(shape)
    for d, n in enumerate(shape):
        h = lengths[d] / n
        k = 2 * np.pi * np.fft.fftfreq(n, d=h)
        sh = [1] * len(shape)
        sh[d] = n
        k2 = k2 + (k ** 2).reshape(sh)
    f = np.real(np.fft.ifftn(np.fft.fftn(z) * np.exp(-0.25 * corr * corr * k2)))
    f = (f - f.mean()) / f.std() * std
    return np.asfortranarray(f)
