"""Fourth-order (p = 4) SBP-SAT operator on the GPU.

The reference builds the p = 4 operator only as an assembled CPU matrix
(``Operators_2d(...; p = 4)`` / ``Assembling_matrix(level; p = 4)`` in
``level_2_multigrid_new.jl:48-188`` with the ``p == 4`` branches of
``diagonal_sbp.jl``); its GPU kernels are second order.  Here the same
operator is matrix-free: the interior stencil (-1/12, 4/3, -5/2, 4/3, -1/12)
along both directions, 4 x 6 boundary closures and the same SAT penalties as
the second-order operator, applied in FP64 by one sm_103a kernel.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib as L
from .solver import SolveResult, _stream_ptr, check_grid, ptr

SQRT_EPS = math.sqrt(2.220446049250313e-16)
MIN_N = 9


def _check_p4(idata: torch.Tensor, odata: torch.Tensor) -> int:
    n = check_grid(idata, name="idata")
    check_grid(odata, name="odata")
    if odata.numel() != idata.numel():
        raise ValueError("idata and odata must have the same size")
    if n < MIN_N:
        raise ValueError(f"the p = 4 operator needs n >= {MIN_N}, got {n}")
    return n


def matrix_free_A_p4_GPU(idata: torch.Tensor, odata: torch.Tensor, sign: int = -1) -> None:
    """odata = sign * A_p4 * idata, A_p4 the SPD p = 4 operator.  The default
    sign = -1 matches matrix_free_A_full_GPU (the reference's GPU kernels
    return -A u)."""
    n = _check_p4(idata, odata)
    L.check(L.load().sbp_apply_p4_f64(ptr(idata), ptr(odata), n, sign, _stream_ptr()),
            "sbp_apply_p4_f64")


def CG_p4_GPU(b: torch.Tensor, x: torch.Tensor, sign: int = 1, abstol: float = 0.0,
              reltol: float = 0.0, maxiter: int | None = None,
              raise_on_fail: bool = False) -> SolveResult:
    """Plain CG on (sign * A_p4) x = b from the caller's x (mutated).  Stops at
    ||r|| < abstol if abstol > 0, else ||r|| < reltol * ||r0|| (abstol =
    sqrt(eps) when both are zero, as the reference's CG)."""
    n = _check_p4(b, x)
    if abstol <= 0.0 and reltol <= 0.0:
        abstol = SQRT_EPS
    maxiter = n * n if maxiter is None else maxiter
    res = L.sbp_result()
    cap = min(maxiter, 100000) + 1
    buf = (C.c_double * cap)()
    st = L.load().sbp_cg_p4_solve(ptr(b), ptr(x), n, sign, abstol, reltol, maxiter,
                                  C.byref(res), buf, cap, _stream_ptr())
    if st < 0 and (raise_on_fail or st not in (L.SBP_ERR_MAXITER, L.SBP_ERR_BREAKDOWN)):
        L.check(st, "sbp_cg_p4_solve")
    cnt = min(cap, res.iters + 1)
    return SolveResult(res.iters, st, list(buf[:cnt]), res.initial_norm, res.final_norm,
                       res.threshold)
