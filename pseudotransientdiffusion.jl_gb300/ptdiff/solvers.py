"""Host-side mirror of the reference's solver drivers on top of libptd.so.

``run_script(name, nx, ...)`` does what ``diffusion_{1,2,3}D_()`` of the named
reference script does (e.g. scripts/diff_2D_nonlin.jl:46-106): it derives the
grid, builds H0 (and the step field D) with the script's arithmetic, solves
``nt`` physical steps with the accelerated PT iteration -- on the GPU, through
the C ABI -- and returns the cell centres and H (the script's
``USE_RETURN=true`` return value, scripts/diff_2D_nonlin.jl:105) together with
the iteration counts it prints (:92) and the residual history.

:class:`Solver` is the thin object wrapper of one ``ptd_ctx``.
"""
from __future__ import annotations

import ctypes as C
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .scripts import LINSTEP, SCRIPTS, Script, cell_centres, grid_shape, initial_condition, step_field

PRECISIONS = {"fp64": _abi.PREC_FP64, "fp32_dc": _abi.PREC_FP32_DC, "df64": _abi.PREC_DF64,
              "dfh": _abi.PREC_DFH, "fp32_rb": _abi.PREC_FP32_RB}


def make_params(script: Script, shape, *, nt=None, itmax=None, nchk=None, tol=None,
                precision="fp64", resid="mixed", norm="rms", norm_len=0.0, strict=False,
                autotune=False, dc_max_outer=0, dc_inner_rtol=0.0, dc_tblock=True,
                rb_tblock_3d=False) -> _abi.PtdParams:
    """ptd_params for a script at a grid shape (x fastest).  dc_tblock=False:
    one FP32 iteration per launch in 2D (FP32_DC, FP32_RB) instead of two;
    rb_tblock_3d=True: two FP32_RB iterations per launch in 3D."""
    p = _abi.PtdParams()
    _abi.check(_abi.lib().ptd_params_init(C.byref(p), script.ndim, script.model), "ptd_params_init")
    p.nx = shape[0]
    p.ny = shape[1] if script.ndim > 1 else 1
    p.nz = shape[2] if script.ndim > 2 else 1
    p.lx, p.ly, p.lz = script.lx, script.ly, script.lz
    p.dt = script.dt
    p.nt = script.nt if nt is None else nt
    p.itmax = script.itmax if itmax is None else itmax
    p.nchk = script.nout if nchk is None else nchk
    p.tol = script.tol if tol is None else tol
    p.cfl = script.cfl
    p.resc = script.resc
    p.D = script.D if script.model != LINSTEP else max(script.D, script.D2)
    p.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    p.resid_mode = {"mixed": _abi.RESID_MIXED, "consistent": _abi.RESID_CONSISTENT}[resid]
    p.norm = {"rms": _abi.NORM_RMS, "max": _abi.NORM_MAX}[norm]
    p.norm_len = norm_len
    p.flags = ((_abi.FLAG_STRICT if strict else 0) | (_abi.FLAG_AUTOTUNE if autotune else 0)
               | (0 if dc_tblock else _abi.FLAG_DC_NO_TBLOCK) | (_abi.FLAG_RB_TBLOCK_3D if rb_tblock_3d else 0))
    p.dc_max_outer = dc_max_outer
    p.dc_inner_rtol = dc_inner_rtol
    return p


def _ptr(a):
    """Address of a host numpy array or of a device tensor (anything with data_ptr())."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


class Solver:
    """One ptd_ctx: device buffers for one grid and parameter set."""

    def __init__(self, params: _abi.PtdParams):
        self.params = params
        self._h = C.c_void_p()
        _abi.check(_abi.lib().ptd_create(C.byref(self._h), C.byref(params)), "ptd_create")

    def close(self):
        if self._h:
            _abi.lib().ptd_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _check_array(self, a, name, out=False):
        return _abi.check_field(a, self.params.nx * self.params.ny * self.params.nz, name, out)

    def solve(self, H, D=None, err_cap: int = 100000, raise_on_nan: bool = True, Hold=None):
        """Solve nt steps in place on H (numpy Fortran array or device tensor).
        Hold: the first step's previous state (default H).
        Returns (iters_per_step, errhist, status)."""
        H = self._check_array(H, "H", out=True)
        if D is not None:
            D = self._check_array(D, "D")
        if Hold is not None:
            Hold = self._check_array(Hold, "Hold")
            _abi.check(_abi.lib().ptd_set_state2(self._h, _ptr(H), _ptr(Hold), _ptr(D)), "ptd_set_state2")
            return self._step_and_get(H, err_cap, raise_on_nan)
        nt = max(self.params.nt, 1)
        iters = np.zeros(nt, dtype=np.int32)
        eh = np.zeros(max(err_cap, 1), dtype=np.float64)
        ne = C.c_int32(0)
        st = _abi.lib().ptd_solve(self._h, _ptr(H), _ptr(D), iters.ctypes.data_as(C.POINTER(C.c_int32)),
                                  eh.ctypes.data_as(C.POINTER(C.c_double)), err_cap, C.byref(ne))
        if st not in (_abi.PTD_OK, _abi.PTD_ENAN, _abi.PTD_ENOTCONV) or (st == _abi.PTD_ENAN and raise_on_nan):
            _abi.check(st, "ptd_solve")
        return iters[: self.params.nt].copy(), eh[: min(ne.value, err_cap)].copy(), st

    def _step_and_get(self, H, err_cap, raise_on_nan):
        nt = max(self.params.nt, 1)
        iters = np.zeros(nt, dtype=np.int32)
        eh = np.zeros(max(err_cap, 1), dtype=np.float64)
        ne = C.c_int32(0)
        st = _abi.lib().ptd_step(self._h, self.params.nt, iters.ctypes.data_as(C.POINTER(C.c_int32)),
                                 eh.ctypes.data_as(C.POINTER(C.c_double)), err_cap, C.byref(ne))
        if st not in (_abi.PTD_OK, _abi.PTD_ENAN, _abi.PTD_ENOTCONV) or (st == _abi.PTD_ENAN and raise_on_nan):
            _abi.check(st, "ptd_step")
        _abi.check(_abi.lib().ptd_get_state(self._h, _ptr(H)), "ptd_get_state")
        return iters[: self.params.nt].copy(), eh[: min(ne.value, err_cap)].copy(), st

    def set_state(self, H, D=None):
        H = self._check_array(H, "H")
        if D is not None:
            D = self._check_array(D, "D")
        _abi.check(_abi.lib().ptd_set_state(self._h, _ptr(H), _ptr(D)), "ptd_set_state")

    def step(self, nsteps: int, err_cap: int = 100000):
        iters = np.zeros(max(nsteps, 1), dtype=np.int32)
        eh = np.zeros(max(err_cap, 1), dtype=np.float64)
        ne = C.c_int32(0)
        st = _abi.lib().ptd_step(self._h, nsteps, iters.ctypes.data_as(C.POINTER(C.c_int32)),
                                 eh.ctypes.data_as(C.POINTER(C.c_double)), err_cap, C.byref(ne))
        _abi.check(st, "ptd_step")
        return iters[:nsteps].copy(), eh[: min(ne.value, err_cap)].copy()

    def iterate(self, niter: int):
        _abi.check(_abi.lib().ptd_iterate(self._h, niter), "ptd_iterate")

    def get_state(self, out=None):
        if out is None:
            shape = (self.params.nx, self.params.ny, self.params.nz)
            out = np.zeros(shape, dtype=np.float64, order="F")
        self._check_array(out, "out", out=True)
        _abi.check(_abi.lib().ptd_get_state(self._h, _ptr(out)), "ptd_get_state")
        return out

    def sync(self):
        _abi.check(_abi.lib().ptd_sync(self._h), "ptd_sync")

    @property
    def stream(self) -> int:
        return _abi.lib().ptd_stream(self._h) or 0

    def counters(self):
        l, it = C.c_int64(0), C.c_int64(0)
        _abi.check(_abi.lib().ptd_counters(self._h, C.byref(l), C.byref(it)), "ptd_counters")
        return l.value, it.value

    def launch_config(self):
        cfg = (C.c_int32 * 4)()
        _abi.check(_abi.lib().ptd_launch_config(self._h, cfg), "ptd_launch_config")
        return {"warps2d": cfg[0], "chunk2d": cfg[1], "rows3d": cfg[2], "chunk3d": cfg[3]}

    def set_launch_config(self, warps2d=None, chunk2d=None, rows3d=None, chunk3d=None):
        cur = self.launch_config()
        new = [warps2d or cur["warps2d"], chunk2d or cur["chunk2d"], rows3d or cur["rows3d"],
               chunk3d or cur["chunk3d"]]
        _abi.check(_abi.lib().ptd_set_launch_config(self._h, (C.c_int32 * 4)(*new)), "ptd_set_launch_config")


@dataclass
class Result:
    """What a reference driver returns and prints."""

    coords: tuple            # (xc,) / (xc, yc) / (xc, yc, zc)
    H: np.ndarray            # final H, shape (nx[, ny[, nz]]), x fastest
    iters: np.ndarray        # PT iterations per physical step
    errhist: np.ndarray      # err of every residual check
    status: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def ittot(self) -> int:
        return int(np.sum(self.iters))

    def as_return(self):
        """The script's USE_RETURN tuple: (xc, H), (xc, yc, H) or (xc, yc, zc, H)."""
        return (*self.coords, self.H)


def _env_int(name, default):
    v = os.environ.get(name)
    return int(v) if v else default


def _env_flag(name):
    return os.environ.get(name, "false").strip().lower() in ("1", "true", "yes")


def output_stem(s: Script) -> str:
    """Name the driver gives its output files: the 3D multi-rank solvers write
    out_diff_3D_<model>.txt / diff_3D_<model>.mat
    (scripts/diff_3D/diff_3D_nonlin_multixpu.jl:131,137), every other script
    its own name."""
    return s.name[: -len("_multixpu")] if s.name.endswith("_multixpu") else s.name


def run_script(name: str, nx: int | None = None, ny: int | None = None, nz: int | None = None, *,
               script: Script | None = None, precision="fp64", verbose=False, save=None, save_viz=None,
               output_dir="output", viz_dir="out_visu", **overrides) -> Result:
    """Run the named reference driver on the GPU.  Grid sizes default to the
    script's NX/NY/NZ environment variables (then to its built-in default);
    ``save`` / ``save_viz`` default to DO_SAVE / DO_SAVE_VIZ, like the scripts
    (scripts/diff_2D_nonlin.jl:8-10,95-104): an iteration-count row appended
    to ``<output_dir>/out_<stem>.txt`` and a ``<viz_dir>/<stem>.mat`` snapshot.
    The *_perf scripts time the physical steps after the first, as the
    reference does (scripts/diff_2D_nonlin_perf.jl:91,105-110), and write
    their timing row instead."""
    from . import output as out

    s = script if script is not None else SCRIPTS[name]
    nx = nx if nx is not None else _env_int("NX", s.default_n)
    ny = ny if ny is not None else _env_int("NY", nx)
    nz = nz if nz is not None else _env_int("NZ", nx)
    save = _env_flag("DO_SAVE") if save is None else save
    save_viz = _env_flag("DO_SAVE_VIZ") if save_viz is None else save_viz
    shape = grid_shape(s, nx, ny, nz)
    H = initial_condition(s, *shape)
    D = step_field(s, *shape) if s.model == LINSTEP else None
    params = make_params(s, shape, precision=precision, **overrides)
    perf = s.name.endswith("_perf")
    extra = {}
    with Solver(params) as sol:
        if s.react:
            Heq = H
            H = np.zeros_like(Heq, order="F")
            iters, eh, st = sol.solve(H, D, Hold=Heq)
        elif perf and params.nt > 1:
            sol.set_state(H, D)
            i0, e0 = sol.step(1)
            sol.sync()
            t0 = time.perf_counter()
            i1, e1 = sol.step(params.nt - 1)
            sol.sync()
            t_toc = time.perf_counter() - t0
            H = sol.get_state().reshape(shape, order="F")
            iters, eh, st = np.concatenate([i0, i1]), np.concatenate([e0, e1]), 0
            niter = int(np.sum(i1))
            a_eff = (2 * (s.ndim + 1) + 2) * int(np.prod(shape)) * 8 / 1e9
            t_it = t_toc / max(niter, 1)
            extra = {"t_toc": t_toc, "A_eff": a_eff, "t_it": t_it, "T_eff": a_eff / t_it, "niter": niter}
        else:
            iters, eh, st = sol.solve(H, D)
    lengths = (s.lx, s.ly, s.lz)
    coords = tuple(cell_centres(lengths[d], shape[d]) for d in range(s.ndim))
    res = Result(coords, H, iters, eh, st, extra)
    if verbose and s.react:   # scripts/diff_1D_react.jl:70, diff_2D_react.jl:74
        dims = ", ".join(f"{c} = {n}" for c, n in zip(("nx", "ny"), shape))
        print(f"{dims}, iterations tot = {res.ittot} ")
    elif verbose:
        if extra:
            teff3 = float("%.3g" % extra["T_eff"])   # round(T_eff, sigdigits=3)
            print(f"PERF: Time = {extra['t_toc']:1.3f} sec, T_eff = {teff3:1.2f} GB/s (niter = {extra['niter']})")
        print(f"Total time = {s.ttot:1.2f}, time steps = {len(iters)}, nx = {nx}, iterations tot = {res.ittot} ")
    stem = output_stem(s)
    if save and not s.react:   # the reaction scripts write no files
        if extra:
            row = out.perf_row(shape, res.ittot, extra["t_toc"], extra["A_eff"], extra["t_it"], extra["T_eff"])
        else:
            row = out.counts_row(shape, res.ittot, len(iters))
        out.append_row(os.path.join(output_dir, f"out_{stem}.txt"), row)
    if save_viz and not s.react:
        out.write_mat(os.path.join(viz_dir, f"{stem}.mat"), H, lengths)
    return res
