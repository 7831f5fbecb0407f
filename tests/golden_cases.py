"""Shared definitions of the reference's golden test cases (test/test_1D.jl,
test/test_2D.jl, test/test_3D_{1..5}.jl): script name -> grid size."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# NX of each reference test (test/test_1D.jl:9, test/test_2D.jl:9-10, test/shared.jl:9-11)
GOLDEN_CASES = {
    "diff_1D_lin": 64,
    "diff_1D_linstep": 64,
    "diff_1D_nonlin": 64,
    "diff_1D_react": 64,
    "diff_2D_lin": 64,
    "diff_2D_linstep": 64,
    "diff_2D_nonlin": 64,
    "diff_2D_nonlin_perf": 64,
    "diff_2D_react": 64,
    "diff_3D_lin_multixpu": 32,
    "diff_3D_linstep_multixpu": 32,
    "diff_3D_nonlin_multixpu": 32,
    "diff_3D_nonlin_multixpu_perf": 32,
    "diff_3D_nonlin_perf": 32,
}

# output/out_diff_<key>.txt -> script
COUNT_SCRIPTS = {
    "1D_lin": "diff_1D_lin", "1D_linstep": "diff_1D_linstep", "1D_nonlin": "diff_1D_nonlin",
    "2D_lin": "diff_2D_lin", "2D_linstep": "diff_2D_linstep", "2D_nonlin": "diff_2D_nonlin",
    "3D_lin": "diff_3D_lin_multixpu", "3D_linstep": "diff_3D_linstep_multixpu",
    "3D_nonlin": "diff_3D_nonlin_multixpu",
}


def start_fields(s, shape):
    """(H, Hold) the script starts from: H0 twice, or for the reaction scripts
    H = 0 and Hold = Heq = H0 (scripts/diff_1D_react.jl:45-47)."""
    from ptdiff.scripts import initial_condition

    H0 = initial_condition(s, *shape)
    if s.react:
        return np.zeros_like(H0, order="F"), H0
    return H0, None


def load_reftests():
    with open(os.path.join(HERE, "golden", "reftests.json")) as fh:
        return json.load(fh)


def load_counts():
    with open(os.path.join(HERE, "golden", "iteration_counts.json")) as fh:
        return json.load(fh)


def golden_array(entry):
    return np.array(entry["H"], dtype=np.float64).reshape(entry["size"], order="F")


def sample(H, n, ndim):
    from ptdiff.scripts import sample_indices

    idx = sample_indices(n)
    return H[np.ix_(*([idx] * ndim))]


def multirank_norm_len(n_global: int, ndim: int = 3, dims: int = 2) -> float:
    """len_ResH_g of the 3D multi-rank scripts (diff_3D_nonlin_multixpu.jl:89) for
    a global grid n_global produced by `dims` ranks per dimension
    (nx_g = dims*(nx-2)+2, scripts/diff_3D/runme.sh:41)."""
    nloc = (n_global - 2) // dims + 2
    return float(((nloc - 2 - 2) * dims + 2) ** ndim)


def reference_isapprox(a, b, rtol=1.4901161193847656e-8):
    """Julia isapprox on arrays (norm-wise, the reference tests' comparison)."""
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))
