"""The reference's output formats (ptdiff.output): iteration-count rows,
perf rows and MATLAB snapshots.  Rows are checked byte-for-byte against the
reference's own output files (tests/golden/output_rows.json)."""
import json
import os

import numpy as np
import pytest

from ptdiff import output as OUT
from ptdiff import scripts as S

HERE = os.path.dirname(os.path.abspath(__file__))
ROWS = json.load(open(os.path.join(HERE, "golden", "output_rows.json")))


def _dims(name):
    return {"1D": 1, "2D": 2, "3D": 3}[name.split("_")[2]]


@pytest.mark.parametrize("name", sorted(ROWS))
def test_rows_round_trip_byte_exact(name):
    nd = _dims(name)
    for line in ROWS[name]:
        v = OUT.parse_row(line)
        if len(v) == nd + 2:                 # nx [ny [nz]] ittot nt
            got = OUT.counts_row(v[:nd], v[nd], v[nd + 1])
        elif nd == 2:                        # nx ny ittot t_toc A_eff t_it T_eff
            got = OUT.perf_row(v[:2], v[2], *v[3:7])
        else:                                # nprocs nx ny nz ittot t_toc A_eff t_it T_eff
            got = OUT.perf_row(v[1:4], v[4], *v[5:9], nprocs=v[0])
        assert got == line


@pytest.mark.parametrize("x,s", [(6.5536e-5, "6.5536e-5"), (10.73741824, "10.73741824"), (2.0, "2.0"),
                                 (1e16, "1.0e16"), (0.0001, "0.0001"), (float("nan"), "NaN"),
                                 (-3.5e-7, "-3.5e-7"), (float("inf"), "Inf")])
def test_julia_float_printing(x, s):
    assert OUT.julia_float(x) == s


def test_append_row_creates_directory(tmp_path):
    path = tmp_path / "output" / "out_diff_2D_nonlin.txt"
    OUT.append_row(str(path), OUT.counts_row((64, 64), 170, 5))
    OUT.append_row(str(path), OUT.counts_row((128, 128), 300, 5))
    assert path.read_text() == "64 64 170 5\n128 128 300 5\n"


@pytest.mark.parametrize("shape", [(7,), (6, 5), (4, 3, 5)])
def test_mat_snapshot(tmp_path, shape):
    sio = pytest.importorskip("scipy.io")
    H = np.asfortranarray(np.random.default_rng(0).standard_normal(shape))
    path = tmp_path / "out_visu" / "snap.mat"
    OUT.write_mat(str(path), H, (10.0, 10.0, 10.0))
    m = sio.loadmat(str(path))
    nd = len(shape)
    assert np.array_equal(m[f"H_{nd}D"].reshape(shape), H)
    for d, name in enumerate(("xc", "yc", "zc")[:nd]):
        xc = m[f"{name}_{nd}D"]
        assert xc.shape == (shape[d], 1)   # MAT.jl writes a Julia Vector as a column
        assert np.array_equal(xc[:, 0], S.cell_centres(10.0, shape[d]))
