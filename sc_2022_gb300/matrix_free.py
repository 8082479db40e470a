"""The reference's GPU entry points, same names and argument meaning, backed
by libsbpmg's sm_103a kernels.

Each function names the Julia function it replaces (path:line inside
AlexandreChern/SC_2022).  Arrays are torch CUDA float64 tensors holding the
column-major n x n grid (see :mod:`sc_2022_gb300.solver`).  Like the
reference, outputs are caller-owned tensors mutated in place, and the
solvers return the reference's tuples.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib as L
from .solver import (Options, Solver, _stream_ptr, check_grid, default_options, ptr,
                     reference_two_level_options)

SQRT_EPS = math.sqrt(2.220446049250313e-16)

_solver_cache: dict = {}


# Largest grid of the direct (fast-diagonalisation) coarse solve.
COARSE_MAX_N = 1025

def _cached_solver(n: int, options: Options | None) -> Solver:
    key = (n, None if options is None else tuple(vars(options).items()),
           torch.cuda.current_device())
    s = _solver_cache.get(key)
    if s is None:
        s = Solver(n, options)
        _solver_cache[key] = s
    return s


def matrix_free_A_full_GPU(idata: torch.Tensor, odata: torch.Tensor) -> None:
    """odata = -A * idata (``split_matrix_free.jl:444-486``): one fused
    sm_103a stencil pass instead of the reference's 6 launches, 4
    allocations and 4 broadcast merges."""
    n = check_grid(idata, name="idata")
    check_grid(odata, name="odata")
    if odata.numel() != idata.numel():
        raise ValueError("idata and odata must have the same size")
    L.check(L.load().sbp_apply_f64(ptr(idata), ptr(odata), n, -1, _stream_ptr()),
            "sbp_apply_f64")


def matrix_free_A_full_GPU_f32(idata: torch.Tensor, odata: torch.Tensor) -> None:
    """FP32 variant of :func:`matrix_free_A_full_GPU` (no reference
    counterpart; used by the mixed-precision V-cycle)."""
    n = check_grid(idata, torch.float32, name="idata")
    check_grid(odata, torch.float32, name="odata")
    L.check(L.load().sbp_apply_f32(ptr(idata), ptr(odata), n, -1, _stream_ptr()),
            "sbp_apply_f32")


def CG_full_GPU(b_reshaped_GPU: torch.Tensor, x_GPU: torch.Tensor, abstol: float = SQRT_EPS,
                maxiter: int | None = None):
    """Matrix-free CG (``split_matrix_free.jl:647-686``).  Iterates with
    matrix_free_A_full_GPU, i.e. solves (-A) x = b, from the caller's x
    (mutated).  Returns (num_iter_steps, abstol, norms[end])."""
    n = check_grid(b_reshaped_GPU, name="b")
    s = _cached_solver(n, None)
    res = s.cg(b_reshaped_GPU, x_GPU, sign=-1, abstol=abstol,
               maxiter=n * n if maxiter is None else maxiter)
    # the reference's norms holds sqrt(rs) up to the last non-converged step
    last = res.norms[-2] if (res.converged and len(res.norms) >= 2) else res.norms[-1]
    return res.iters, abstol, last


def CG_Matrix_Free_GPU_v2(x_GPU, Ap_GPU, b_reshaped_GPU, Nx, Ny, abstol: float = SQRT_EPS):
    """``split_matrix_free.jl:688-714``: like CG_full_GPU with a caller
    workspace Ap_GPU (its final contents are unspecified).  Returns
    (iters, abstol, sqrt(norms[end])) -- the reference takes the square root
    of an entry that already is a norm, and this keeps that return value."""
    n = check_grid(b_reshaped_GPU, name="b")
    if Nx != n or Ny != n:
        raise ValueError("only square grids (Nx == Ny == n) are supported, as in the reference")
    matrix_free_A_full_GPU(x_GPU, Ap_GPU)
    s = _cached_solver(n, None)
    res = s.cg(b_reshaped_GPU, x_GPU, sign=-1, abstol=abstol, maxiter=n * n)
    last = res.norms[-2] if (res.converged and len(res.norms) >= 2) else res.norms[-1]
    return res.iters, abstol, math.sqrt(last)


def _mg_options(n: int, nu: int, A_2h) -> Options:
    if isinstance(A_2h, Options):
        return A_2h
    if (n + 1) // 2 <= COARSE_MAX_N:
        o = reference_two_level_options(n)
    else:
        # The reference's exact coarse LU at (n+1)/2 is replaced by the
        # multi-level V-cycle beyond the largest direct coarse grid.
        o = default_options()
    o.nu_pre = o.nu_post = nu
    return o


def matrix_free_MGCG(b_GPU: torch.Tensor, x_GPU: torch.Tensor, A_2h=None,
                     maxiter: int | None = None, abstol: float = SQRT_EPS,
                     NUM_V_CYCLES: int = 1, nu: int = 3, use_galerkin=True, direct_sol=0,
                     H_tilde=0, SBPp: int = 2):
    """MG-preconditioned CG (``preconditioned_CG/matrix_free_mg_cg.jl:281-324``)
    on A x = b from the caller's x (mutated).  Returns (iters, norms, x).

    ``A_2h`` is the reference's coarse LU factor; here it may be a
    :class:`Solver` (reused), an :class:`Options`, or None: the reference's
    two-level Richardson preconditioner with an exact coarse solve when
    (n+1)/2 <= 1025 (N <= 2049), else the default V-cycle.  NUM_V_CYCLES, use_galerkin,
    direct_sol and H_tilde are accepted for signature compatibility; the
    reference ignores them as well (SBPp must be 2).
    """
    if SBPp != 2:
        raise ValueError("only the 2nd-order SBP operator (SBPp=2) is implemented")
    n = check_grid(b_GPU, name="b")
    solver = A_2h if isinstance(A_2h, Solver) else _cached_solver(n, _mg_options(n, nu, A_2h))
    res = solver.mgcg(b_GPU, x_GPU, abstol=abstol, maxiter=n * n if maxiter is None else maxiter)
    return res.iters, res.norms, x_GPU


def matrix_free_Two_level_multigrid(b_GPU: torch.Tensor, A_2h=None, nu: int = 3,
                                    NUM_V_CYCLES: int = 1, SBPp: int = 2):
    """One V-cycle from zero (``matrix_free_mg_cg.jl:143-176``).  Returns
    (v, norm(A v - b))."""
    if NUM_V_CYCLES != 1:
        raise ValueError("only NUM_V_CYCLES=1 is supported (the reference's MGCG uses 1)")
    n = check_grid(b_GPU, name="b")
    solver = A_2h if isinstance(A_2h, Solver) else _cached_solver(n, _mg_options(n, nu, A_2h))
    v = torch.empty_like(b_GPU)
    solver.vcycle(b_GPU, v)
    nrm = C.c_double()
    L.check(L.load().sbp_residual_norm_f64(ptr(v), ptr(b_GPU), n, 1, C.byref(nrm),
                                           _stream_ptr()), "sbp_residual_norm_f64")
    return v, nrm.value


def matrix_free_richardson(idata_GPU: torch.Tensor, odata_GPU: torch.Tensor, b_GPU: torch.Tensor,
                           maxiter: int = 3, omega: float = 0.15) -> None:
    """``matrix_free_mg_cg.jl:134-140``: maxiter sweeps
    v <- v + omega (b - A v); both idata and odata hold the result."""
    n = check_grid(idata_GPU, name="idata")
    check_grid(odata_GPU, name="odata")
    check_grid(b_GPU, name="b")
    L.check(L.load().sbp_richardson_f64(ptr(idata_GPU), ptr(odata_GPU), ptr(b_GPU), n, maxiter,
                                        omega, _stream_ptr()), "sbp_richardson_f64")


def jacobi(idata_GPU: torch.Tensor, odata_GPU: torch.Tensor, b_GPU: torch.Tensor,
           maxiter: int = 3, omega: float = 2.0 / 3.0) -> None:
    """Weighted Jacobi (``jacobi_brittany!``, level_2_multigrid_new.jl:335-344),
    matrix-free on the GPU; both idata and odata hold the result."""
    n = check_grid(idata_GPU, name="idata")
    L.check(L.load().sbp_jacobi_f64(ptr(idata_GPU), ptr(odata_GPU), ptr(b_GPU), n, maxiter,
                                    omega, _stream_ptr()), "sbp_jacobi_f64")


def matrix_free_restriction_2d_GPU(idata: torch.Tensor, odata: torch.Tensor,
                                   kind: int = L.SBP_RESTRICT_NORMAL) -> None:
    """Full-weighting restriction (``matrix_free_mg_cg.jl:98-131``) without
    the reference's zero-padded copy: odata ((n+1)/2 squared) = R idata."""
    n = check_grid(idata, name="idata")
    nc = check_grid(odata, name="odata")
    if nc != (n + 1) // 2:
        raise ValueError("odata must be ((n+1)/2)^2")
    L.check(L.load().sbp_restrict_f64(ptr(idata), ptr(odata), n, kind, _stream_ptr()),
            "sbp_restrict_f64")


def matrix_free_prolongation_2d_GPU(idata: torch.Tensor, odata: torch.Tensor,
                                    accumulate: bool = False) -> None:
    """Bilinear prolongation (``matrix_free_mg_cg.jl:41-77``), every fine
    point written once: odata ((2n-1)^2) = P idata (n^2)."""
    nc = check_grid(idata, name="idata")
    nf = check_grid(odata, name="odata")
    if nf != 2 * nc - 1:
        raise ValueError("odata must be (2n-1)^2")
    L.check(L.load().sbp_prolong_f64(ptr(idata), ptr(odata), nc, int(accumulate),
                                     _stream_ptr()), "sbp_prolong_f64")


# ---------------------------------------------------------------------------
# Nested iteration (initial guess from the coarse problem)
# ---------------------------------------------------------------------------
def _coarse_exact(b_2h: torch.Tensor) -> torch.Tensor:
    """x = A^-1 b on the grid of b: the fast-diagonalisation direct solve of a
    one-level handle (coarse grids up to 1025^2), else MGCG to 1e-14."""
    n = check_grid(b_2h, name="b_2h")
    x = torch.zeros_like(b_2h)
    if n <= COARSE_MAX_N:
        o = default_options()
        o.coarse_n = n
        _cached_solver(n, o).vcycle(b_2h, x)
    else:
        _cached_solver(n, default_options()).mgcg(b_2h, x, reltol=1e-14, raise_on_fail=True)
    return x


def _prolong(xc: torch.Tensor, n: int) -> torch.Tensor:
    nc = check_grid(xc, name="coarse")
    if 2 * nc - 1 != n:
        raise ValueError(f"coarse grid {nc} does not prolong to {n}")
    out = torch.empty(n * n, dtype=torch.float64, device=xc.device)
    L.check(L.load().sbp_prolong_f64(ptr(xc), ptr(out), nc, 0, _stream_ptr()), "sbp_prolong_f64")
    return out


def _cg_from(b: torch.Tensor, x: torch.Tensor, abstol: float, maxiter: int | None):
    """IterativeSolvers-style cg!: stop at max(sqrt(eps) |b - A x0|, abstol)."""
    n = check_grid(b, name="b")
    r0 = C.c_double()
    L.check(L.load().sbp_residual_norm_f64(ptr(x), ptr(b), n, 1, C.byref(r0), _stream_ptr()),
            "sbp_residual_norm_f64")
    tol = max(SQRT_EPS * r0.value, abstol)
    res = _cached_solver(n, None).cg(b, x, sign=1, abstol=tol,
                                      maxiter=n * n if maxiter is None else maxiter)
    return res


def initial_guess_interpolation_CG_GPU(b_GPU: torch.Tensor, b_2h: torch.Tensor, x=None,
                                       Nx_2h=None, abstol: float = SQRT_EPS,
                                       maxiter: int | None = None):
    """``matrix_free_mg_cg.jl:379-384``: exact solve of the coarse problem
    A_2h x_2h = b_2h (its own right-hand side), bilinear prolongation of x_2h
    as the initial guess, CG on A x = b.  Returns (x, iters, resnorms).  ``x``
    and ``Nx_2h`` are accepted for signature compatibility (the reference
    ignores x as well; the coarse size is b_2h's)."""
    n = check_grid(b_GPU, name="b")
    xs = _prolong(_coarse_exact(b_2h.reshape(-1)), n)
    res = _cg_from(b_GPU.reshape(-1), xs, abstol, maxiter)
    return xs, res.iters, list(res.norms)


def initial_guess_interpolation_three_level_CG_GPU(b_GPU: torch.Tensor, b_2h_GPU: torch.Tensor,
                                                   b_4h: torch.Tensor, x=None, Nx_2h=None,
                                                   Nx_4h=None, abstol: float = SQRT_EPS,
                                                   maxiter: int | None = None):
    """``matrix_free_mg_cg.jl:386-396``: exact solve on 4h, prolong, CG on 2h
    with b_2h, prolong, CG on h.  Returns (x, iters_2h, iters_h, resnorm_2h,
    resnorm_h)."""
    n = check_grid(b_GPU, name="b")
    n2 = check_grid(b_2h_GPU, name="b_2h")
    x2 = _prolong(_coarse_exact(b_4h.reshape(-1)), n2)
    r2 = _cg_from(b_2h_GPU.reshape(-1), x2, abstol, maxiter)
    xs = _prolong(x2, n)
    r1 = _cg_from(b_GPU.reshape(-1), xs, abstol, maxiter)
    return xs, r2.iters, r1.iters, list(r2.norms), list(r1.norms)
