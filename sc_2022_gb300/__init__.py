"""GB300-native matrix-free SBP-SAT Poisson solver (libsbpmg) with the
reference's entry points: matrix_free_A_full_GPU, CG_full_GPU,
CG_Matrix_Free_GPU_v2, matrix_free_MGCG, matrix_free_Two_level_multigrid,
matrix_free_richardson, matrix_free_restriction_2d_GPU,
matrix_free_prolongation_2d_GPU.
"""
from . import _lib
from ._lib import SbpError
from .adjoint import HMisfit, PoissonSolve, mgcg_rrule
from .high_order import (CG_high_order_GPU, CG_p4_GPU, HighOrderSolver, MGCG_high_order_GPU,
                         matrix_free_A_high_order_GPU, matrix_free_A_p4_GPU)
from .matrix_free import (CG_Matrix_Free_GPU_v2, CG_full_GPU, initial_guess_interpolation_CG_GPU,
                          initial_guess_interpolation_three_level_CG_GPU, jacobi,
                          matrix_free_A_full_GPU,
                          matrix_free_A_full_GPU_f32, matrix_free_MGCG,
                          matrix_free_prolongation_2d_GPU, matrix_free_restriction_2d_GPU,
                          matrix_free_richardson, matrix_free_Two_level_multigrid)
from .variable import (MGCG_variable_GPU, VariableCoefficientSolver, assemble_variable_host,
                       coarsen_coefficients_host, galerkin_coarse_host,
                       matrix_free_A_variable_GPU)
from .solver import (BatchSolver, Options, SolveResult, Solver, default_options,
                     reference_two_level_options)

__all__ = [
    "CG_Matrix_Free_GPU_v2", "CG_full_GPU", "jacobi", "matrix_free_A_full_GPU",
    "matrix_free_A_full_GPU_f32", "matrix_free_MGCG", "matrix_free_prolongation_2d_GPU",
    "matrix_free_restriction_2d_GPU", "matrix_free_richardson",
    "matrix_free_Two_level_multigrid", "Options", "SolveResult", "Solver", "default_options",
    "reference_two_level_options", "SbpError", "load_library", "HMisfit", "PoissonSolve",
    "mgcg_rrule", "BatchSolver", "initial_guess_interpolation_CG_GPU",
    "initial_guess_interpolation_three_level_CG_GPU", "CG_p4_GPU", "matrix_free_A_p4_GPU",
    "CG_high_order_GPU", "HighOrderSolver", "MGCG_high_order_GPU", "matrix_free_A_high_order_GPU",
    "MGCG_variable_GPU", "VariableCoefficientSolver", "assemble_variable_host",
    "coarsen_coefficients_host", "galerkin_coarse_host", "matrix_free_A_variable_GPU",
]


def load_library():
    """Load libsbpmg.so; raises ImportError if it has not been built."""
    return _lib.load()
