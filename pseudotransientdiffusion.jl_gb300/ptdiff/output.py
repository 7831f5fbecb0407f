"""The reference's output formats, so that its post-processing reads our runs.

* iteration-count rows appended to ``output/out_diff_<case>.txt``:
  ``nx [ny [nz]] ittot nt`` (scripts/diff_1D_lin.jl:87, diff_2D_nonlin.jl:98,
  diff_3D/diff_3D_nonlin_multixpu.jl:132);
* performance rows of the perf scripts: 2D ``nx ny ittot t_toc A_eff t_it
  T_eff`` (scripts/diff_2D_nonlin_perf.jl:117) and 3D ``nprocs nx ny nz ittot
  t_toc A_eff t_it T_eff`` (diff_3D/diff_3D_nonlin_perf.jl:128,
  diff_3D_nonlin_multixpu_perf.jl:150), A_eff in GB, t in s, T_eff in GB/s;
* MATLAB v5 snapshots ``out_visu/<script>.mat`` holding ``H_<n>D`` and the
  cell centres ``xc_<n>D`` (``yc``, ``zc``), zlib-compressed
  (scripts/diff_2D_nonlin.jl:103, consumed by visu/*.m).

Floats are written the way Julia prints them (shortest round-trip digits,
``1.5e-5`` rather than ``1.5e-05``), so rows are byte-identical to the
reference's for the same numbers.
"""
from __future__ import annotations

import math
import os

import numpy as np

from .scripts import cell_centres


def julia_float(x: float) -> str:
    """`string(x::Float64)` of Julia: shortest round-trip digits, scientific
    notation below 1e-4 and from 1e16, exponent without padding."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Inf" if x > 0 else "-Inf"
    s = repr(x)
    if "e" in s:
        mant, exp = s.split("e")
        if "." not in mant:
            mant += ".0"
        return f"{mant}e{int(exp)}"
    return s


def _field(v) -> str:
    return str(v) if isinstance(v, (int, np.integer)) else julia_float(v)


def counts_row(shape, ittot: int, nt: int) -> str:
    """One row of output/out_diff_<case>.txt."""
    return " ".join(str(int(n)) for n in shape) + f" {int(ittot)} {int(nt)}"


def perf_row(shape, ittot: int, t_toc: float, a_eff_gb: float, t_it: float, t_eff: float,
             nprocs: int = 1) -> str:
    """One row of the perf scripts' output (2D: no nprocs column)."""
    head = [] if len(shape) == 2 else [int(nprocs)]
    vals = head + [int(n) for n in shape] + [int(ittot), t_toc, a_eff_gb, t_it, t_eff]
    return " ".join(_field(v) for v in vals)


def parse_row(line: str):
    """Numbers of a row: ints where the text is an integer, floats elsewhere."""
    out = []
    for tok in line.split():
        try:
            out.append(int(tok))
        except ValueError:
            out.append(float(tok))
    return out


def append_row(path: str, row: str) -> None:
    """Append a row, creating the directory as the scripts do (mkdir if absent)."""
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "a") as fh:
        fh.write(row + "\n")


def snapshot_dict(H, lengths) -> dict:
    """The .mat variables of a driver: H_<n>D and the cell centres."""
    H = np.asarray(H, dtype=np.float64)
    nd = H.ndim
    out = {f"H_{nd}D": H}
    for d, name in zip(range(nd), ("xc", "yc", "zc")):
        out[f"{name}_{nd}D"] = cell_centres(lengths[d], H.shape[d]).reshape(-1, 1)
    return out


def write_mat(path: str, H, lengths) -> None:
    """MATLAB v5 snapshot of H (Fortran-ordered numpy array) and its cell
    centres, compressed, column vectors for the coordinates (MAT.jl writes a
    Julia Vector as n x 1)."""
    from scipy.io import savemat

    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    savemat(path, snapshot_dict(H, lengths), do_compression=True, oned_as="column")
