"""Higher-order (p = 4, 6) SBP-SAT operators and solvers on the GPU.

The reference builds the p = 4 and p = 6 operators only as assembled CPU
matrices (``Operators_2d(...; p)`` / ``Assembling_matrix(level; p)`` in
``level_2_multigrid_new.jl:48-188`` with the ``p == 4`` and ``p == 6``
branches of ``diagonal_sbp.jl``).  It preconditions them with a CPU
multigrid (``precond_matrix(A, b; SBPp)``, ``initial_guess_cg.jl:458-510``);
its GPU kernels are second order.

Here the same operators are matrix-free FP64 sm_103a kernels:
- the interior D2 stencil along both directions;
- bm x bn boundary closures (4 x 6 for p = 4, 6 x 9 for p = 6);
- the SAT penalties of the second-order operator.
They come with CG and a multigrid-preconditioned CG whose V-cycle
re-discretises the order-p operator on every level.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib as L
from .solver import Options, SolveResult, _stream_ptr, check_grid, default_options, ptr

SQRT_EPS = math.sqrt(2.220446049250313e-16)
MIN_N = {4: 8, 6: 12}


def _check_pair(a: torch.Tensor, b: torch.Tensor, p: int, names=("idata", "odata")) -> int:
    if p not in MIN_N:
        raise ValueError(f"SBP order p must be 4 or 6, got {p}")
    n = check_grid(a, name=names[0])
    check_grid(b, name=names[1])
    if b.numel() != a.numel():
        raise ValueError(f"{names[0]} and {names[1]} must have the same size")
    if n < MIN_N[p]:
        raise ValueError(f"the p = {p} operator needs n >= {MIN_N[p]}, got {n}")
    return n


def matrix_free_A_high_order_GPU(idata: torch.Tensor, odata: torch.Tensor, p: int = 4,
                                 sign: int = -1) -> None:
    """odata = sign * A_p * idata, A_p the SPD order-p operator.  The default
    sign = -1 matches matrix_free_A_full_GPU (the reference's GPU kernels
    return -A u)."""
    n = _check_pair(idata, odata, p)
    L.check(L.load().sbp_apply_ho_f64(ptr(idata), ptr(odata), n, p, sign, _stream_ptr()),
            "sbp_apply_ho_f64")


def matrix_free_A_p4_GPU(idata: torch.Tensor, odata: torch.Tensor, sign: int = -1) -> None:
    """:func:`matrix_free_A_high_order_GPU` with p = 4."""
    matrix_free_A_high_order_GPU(idata, odata, 4, sign)


class HighOrderSolver:
    """Order-p (4 or 6) solver handle for n x n grids: plain CG on any
    n >= the operator's minimum, multigrid-preconditioned CG when n coarsens
    to ``options.coarse_n`` (or n <= coarse_n: one direct level).
    ``options=None`` uses :func:`default_options` (Jacobi 2/3, 3 + 3 sweeps,
    Galerkin-scaled restriction, direct solve at 65^2), FP64."""

    def __init__(self, n: int, p: int = 4, options: Options | None = None):
        if p not in MIN_N:
            raise ValueError(f"SBP order p must be 4 or 6, got {p}")
        self.n, self.p = n, p
        self.options = options if options is not None else default_options()
        self._lib = L.load()
        h = C.c_void_p()
        oc = self.options.to_c()
        L.check(self._lib.sbp_ho_solver_create(C.byref(h), n, p, C.byref(oc)),
                "sbp_ho_solver_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sbp_ho_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def levels(self) -> int:
        return L.check(self._lib.sbp_ho_solver_levels(self._h), "sbp_ho_solver_levels")

    @property
    def device_bytes(self) -> int:
        return int(self._lib.sbp_ho_solver_device_bytes(self._h))

    def _pair(self, b, x):
        n = _check_pair(b, x, self.p, ("b", "x"))
        if n != self.n:
            raise ValueError(f"grid size mismatch: solver n={self.n}, b has n={n}")
        return n

    def _run(self, call, name, maxiter, raise_on_fail):
        res = L.sbp_result()
        cap = min(maxiter, 100000) + 1
        buf = (C.c_double * cap)()
        st = call(C.byref(res), buf, cap)
        if st < 0 and (raise_on_fail or st not in (L.SBP_ERR_MAXITER, L.SBP_ERR_BREAKDOWN)):
            L.check(st, name)
        cnt = min(cap, res.iters + 1)
        return SolveResult(res.iters, st, list(buf[:cnt]), res.initial_norm, res.final_norm,
                           res.threshold)

    def mgcg(self, b: torch.Tensor, x: torch.Tensor, abstol: float = 0.0, reltol: float = 0.0,
             maxiter: int | None = None, stream=None, raise_on_fail=False) -> SolveResult:
        """MGCG on A_p x = b from the caller's x (overwritten).  Stops at
        ||r|| < abstol if abstol > 0, else ||r|| < reltol * ||r0||."""
        n = self._pair(b, x)
        maxiter = n * n if maxiter is None else maxiter
        sp = _stream_ptr(stream)
        return self._run(lambda res, buf, cap: self._lib.sbp_ho_mgcg_solve(
            self._h, ptr(b), ptr(x), abstol, reltol, maxiter, res, buf, cap, sp),
            "sbp_ho_mgcg_solve", maxiter, raise_on_fail)

    def cg(self, b: torch.Tensor, x: torch.Tensor, sign: int = 1, abstol: float = 0.0,
           reltol: float = 0.0, maxiter: int | None = None, stream=None,
           raise_on_fail=False) -> SolveResult:
        """Plain CG on (sign * A_p) x = b from the caller's x."""
        n = self._pair(b, x)
        maxiter = n * n if maxiter is None else maxiter
        sp = _stream_ptr(stream)
        return self._run(lambda res, buf, cap: self._lib.sbp_ho_cg_solve(
            self._h, ptr(b), ptr(x), sign, abstol, reltol, maxiter, res, buf, cap, sp),
            "sbp_ho_cg_solve", maxiter, raise_on_fail)

    def vcycle(self, b: torch.Tensor, v: torch.Tensor, stream=None) -> None:
        """v = one order-p V-cycle from zero for the right-hand side b."""
        self._pair(b, v)
        L.check(self._lib.sbp_ho_vcycle_apply(self._h, ptr(b), ptr(v), _stream_ptr(stream)),
                "sbp_ho_vcycle_apply")


_cache: dict = {}


def _solver(n: int, p: int, options: Options | None) -> HighOrderSolver:
    key = (n, p, None if options is None else tuple(vars(options).items()),
           torch.cuda.current_device())
    s = _cache.get(key)
    if s is None:
        s = HighOrderSolver(n, p, options)
        _cache[key] = s
    return s


def CG_high_order_GPU(b: torch.Tensor, x: torch.Tensor, p: int = 4, sign: int = 1,
                      abstol: float = 0.0, reltol: float = 0.0, maxiter: int | None = None,
                      raise_on_fail: bool = False) -> SolveResult:
    """Plain CG on (sign * A_p) x = b from the caller's x (mutated): CG_CPU
    (``level_2_multigrid_new.jl:258-291``) on the order-p operator.  Stops at
    ||r|| < abstol if abstol > 0, else ||r|| < reltol * ||r0|| (abstol =
    sqrt(eps) when both are zero, as the reference's CG)."""
    n = _check_pair(b, x, p, ("b", "x"))
    if abstol <= 0.0 and reltol <= 0.0:
        abstol = SQRT_EPS
    return _solver(n, p, None).cg(b, x, sign=sign, abstol=abstol, reltol=reltol,
                                  maxiter=maxiter, raise_on_fail=raise_on_fail)


def CG_p4_GPU(b: torch.Tensor, x: torch.Tensor, sign: int = 1, abstol: float = 0.0,
              reltol: float = 0.0, maxiter: int | None = None,
              raise_on_fail: bool = False) -> SolveResult:
    """:func:`CG_high_order_GPU` with p = 4."""
    return CG_high_order_GPU(b, x, 4, sign, abstol, reltol, maxiter, raise_on_fail)


def MGCG_high_order_GPU(b: torch.Tensor, x: torch.Tensor, p: int = 4, abstol: float = 0.0,
                        reltol: float = 0.0, maxiter: int | None = None,
                        options: Options | None = None,
                        raise_on_fail: bool = False) -> SolveResult:
    """Multigrid-preconditioned CG on A_p x = b (the GPU counterpart of the
    reference's CPU ``precond_matrix(A, b; SBPp = p)`` preconditioned CG)."""
    n = _check_pair(b, x, p, ("b", "x"))
    if abstol <= 0.0 and reltol <= 0.0:
        abstol = SQRT_EPS
    return _solver(n, p, options).mgcg(b, x, abstol=abstol, reltol=reltol, maxiter=maxiter,
                                       raise_on_fail=raise_on_fail)
