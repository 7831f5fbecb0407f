"""ptdiff -- Python host side of the GB300 accelerated pseudo-transient
diffusion library (libptd.so, C ABI in include/ptd.h).

``run_script`` mirrors the reference's solver drivers; ``Solver`` wraps one
library context.  All PT iterations run in the CUDA library: importing this
package does not import any CPU implementation of the solver.
"""
from . import _abi, dispersion, output, scripts
from ._abi import PtdError, PtdParams
from .scripts import SCRIPTS, Script, initial_condition, step_field
from .solvers import Result, Solver, make_params, run_script
from .batch import BatchSolver, batch_instances, batch_params
from .adjoint import AdjointSolver, misfit_function

__all__ = ["_abi", "dispersion", "output", "scripts", "PtdError", "PtdParams", "SCRIPTS", "Script", "initial_condition",
           "step_field", "Result", "Solver", "make_params", "run_script", "BatchSolver", "batch_instances",
           "batch_params", "AdjointSolver", "misfit_function"]
