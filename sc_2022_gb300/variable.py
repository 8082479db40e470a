"""Variable-coefficient second-order SBP-SAT operator, div(c grad u), on the
GPU.

The reference builds the 1D variable-coefficient operator
``variable_diagonal_sbp_D2(2, N, B)`` (``diagonal_sbp.jl:470-495, 709-740``)
and assembles it in 2D on the CPU in ``get_operators``
(``legacy_functions.jl:100-174``), where it runs it with B = 1.  Here the
operator with any nodal field c > 0 is matrix-free on the GPU:
- every grid line carries the 1D operator of its own coefficients;
- the SATs are those of ``Assembling_matrix``, with the boundary flux and
  the Dirichlet penalty scaled by c at the boundary point.
It comes with CG and a multigrid-preconditioned CG whose coarse levels
re-discretise the operator with harmonic-mean coarse coefficients.  c = 1 gives the
constant-coefficient operator exactly.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L
from .solver import Options, SolveResult, _stream_ptr, check_grid, default_options, ptr

SQRT_EPS = math.sqrt(2.220446049250313e-16)
MAX_COARSE = 33


def matrix_free_A_variable_GPU(idata: torch.Tensor, coef: torch.Tensor, odata: torch.Tensor,
                               sign: int = -1) -> None:
    """odata = sign * A_c * idata for nodal coefficients coef (all n x n
    float64 device grids).  The default sign = -1 matches
    matrix_free_A_full_GPU."""
    n = check_grid(idata, name="idata")
    check_grid(coef, name="coef")
    check_grid(odata, name="odata")
    if not (coef.numel() == odata.numel() == idata.numel()):
        raise ValueError("idata, coef and odata must have the same size")
    L.check(L.load().sbp_apply_vc_f64(ptr(idata), ptr(coef), ptr(odata), n, sign,
                                      _stream_ptr()), "sbp_apply_vc_f64")


def assemble_variable_host(n: int, coef) -> tuple:
    """The variable-coefficient A as CSR arrays (row_ptr, col, val) built on
    the host by the library from the same per-point stencil its GPU solver
    uses (no GPU needed)."""
    c = np.ascontiguousarray(np.asarray(coef, dtype=np.float64).ravel())
    if c.size != n * n:
        raise ValueError("coef must hold n * n values")
    lib = L.load()
    cap = 9 * n * n
    row_ptr = np.zeros(n * n + 1, dtype=np.int64)
    col = np.zeros(cap, dtype=np.int32)
    val = np.zeros(cap, dtype=np.float64)
    nnz = C.c_longlong()
    L.check(lib.sbp_vc_assemble_host(n, c.ctypes.data_as(C.POINTER(C.c_double)),
                                     row_ptr.ctypes.data_as(C.POINTER(C.c_longlong)),
                                     col.ctypes.data_as(C.POINTER(C.c_int)),
                                     val.ctypes.data_as(C.POINTER(C.c_double)), cap,
                                     C.byref(nnz)), "sbp_vc_assemble_host")
    return row_ptr, col[:nnz.value].copy(), val[:nnz.value].copy()


def coarsen_coefficients_host(coef) -> np.ndarray:
    """The coarse coefficients ((n+1)/2 x (n+1)/2) the solver's next level
    uses below the n x n field ``coef`` (n odd): the full-weighting harmonic
    mean, computed on the host with the device kernel's arithmetic."""
    c = np.ascontiguousarray(np.asarray(coef, dtype=np.float64))
    n = int(round(np.sqrt(c.size)))
    if n * n != c.size or n % 2 == 0:
        raise ValueError("coef must be an n x n field with n odd")
    nc = (n + 1) // 2
    out = np.empty(nc * nc, dtype=np.float64)
    L.check(L.load().sbp_vc_coarsen_host(nc, c.ctypes.data_as(C.POINTER(C.c_double)),
                                         out.ctypes.data_as(C.POINTER(C.c_double))),
            "sbp_vc_coarsen_host")
    return out.reshape(nc, nc)


def galerkin_coarse_host(coef, levels: int = 1) -> list:
    """Galerkin coarse operators P' A P of the variable-coefficient operator
    with the n x n nodal field ``coef`` (n odd), ``levels`` levels down, built
    on the host by the library.  Returns one dict per coarse level with the
    9-point stencil arrays 'D', 'E', 'N', 'NE', 'NW' (each m x m, indexed
    [j, i]): D the diagonal of A_c, the others the couplings of -A_c to
    (i+1, j), (i, j+1), (i+1, j+1) and (i-1, j+1)."""
    c = np.ascontiguousarray(np.asarray(coef, dtype=np.float64))
    n = int(round(np.sqrt(c.size)))
    if n * n != c.size or n % 2 == 0 or n < 3:
        raise ValueError("coef must be an n x n field with n odd and n >= 3")
    lib = L.load()
    dp = C.POINTER(C.c_double)
    out = []
    for lev in range(levels):
        if n < 3 or n % 2 == 0:
            raise ValueError(f"level {lev}: {n} points cannot be coarsened")
        m = (n + 1) // 2
        arrs = {k: np.zeros(m * m) for k in ("D", "E", "N", "NE", "NW")}
        ptrs = [arrs[k].ctypes.data_as(dp) for k in ("D", "E", "N", "NE", "NW")]
        if lev == 0:
            L.check(lib.sbp_vc_galerkin_coarse_host(n, c.ctypes.data_as(dp), *ptrs),
                    "sbp_vc_galerkin_coarse_host")
        else:
            prev = out[-1]
            fine = [np.ascontiguousarray(prev[k]).ravel() for k in ("D", "E", "N", "NE", "NW")]
            L.check(lib.sbp_galerkin9_coarse_host(n, *[f.ctypes.data_as(dp) for f in fine],
                                                  *ptrs), "sbp_galerkin9_coarse_host")
        out.append({k: v.reshape(m, m) for k, v in arrs.items()})
        n = m
    return out


class VariableCoefficientSolver:
    """Solver handle for div(c grad u) with the coefficient field ``coef``
    (an n x n float64 device grid, copied at creation).  Plain CG on any
    n >= 3; multigrid-preconditioned CG when n = 2^k + 1 (coarsening to
    min(options.coarse_n, 33)) or n <= 33.  ``options=None`` uses
    :func:`default_options`."""

    def __init__(self, n: int, coef: torch.Tensor, options: Options | None = None):
        m = check_grid(coef, name="coef")
        if m != n:
            raise ValueError(f"coef is a {m} x {m} grid, expected n = {n}")
        self.n = n
        self.options = options if options is not None else default_options()
        self._lib = L.load()
        h = C.c_void_p()
        oc = self.options.to_c()
        L.check(self._lib.sbp_vc_solver_create(C.byref(h), n, ptr(coef), C.byref(oc)),
                "sbp_vc_solver_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sbp_vc_solver_destroy(self._h)
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
        return L.check(self._lib.sbp_vc_solver_levels(self._h), "sbp_vc_solver_levels")

    @property
    def device_bytes(self) -> int:
        return int(self._lib.sbp_vc_solver_device_bytes(self._h))

    def _pair(self, b, x):
        n = check_grid(b, name="b")
        check_grid(x, name="x")
        if n != self.n or x.numel() != b.numel():
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
        """MGCG on A_c x = b from the caller's x (overwritten)."""
        n = self._pair(b, x)
        maxiter = n * n if maxiter is None else maxiter
        sp = _stream_ptr(stream)
        return self._run(lambda res, buf, cap: self._lib.sbp_vc_mgcg_solve(
            self._h, ptr(b), ptr(x), abstol, reltol, maxiter, res, buf, cap, sp),
            "sbp_vc_mgcg_solve", maxiter, raise_on_fail)

    def cg(self, b: torch.Tensor, x: torch.Tensor, sign: int = 1, abstol: float = 0.0,
           reltol: float = 0.0, maxiter: int | None = None, stream=None,
           raise_on_fail=False) -> SolveResult:
        """Plain CG on (sign * A_c) x = b from the caller's x."""
        n = self._pair(b, x)
        maxiter = n * n if maxiter is None else maxiter
        sp = _stream_ptr(stream)
        return self._run(lambda res, buf, cap: self._lib.sbp_vc_cg_solve(
            self._h, ptr(b), ptr(x), sign, abstol, reltol, maxiter, res, buf, cap, sp),
            "sbp_vc_cg_solve", maxiter, raise_on_fail)

    def vcycle(self, b: torch.Tensor, v: torch.Tensor, stream=None) -> None:
        """v = one V-cycle from zero for the right-hand side b."""
        self._pair(b, v)
        L.check(self._lib.sbp_vc_vcycle_apply(self._h, ptr(b), ptr(v), _stream_ptr(stream)),
                "sbp_vc_vcycle_apply")


def MGCG_variable_GPU(b: torch.Tensor, x: torch.Tensor, coef: torch.Tensor, abstol: float = 0.0,
                      reltol: float = 0.0, maxiter: int | None = None,
                      options: Options | None = None) -> SolveResult:
    """One-shot multigrid-preconditioned CG on A_c x = b (builds a handle;
    keep a :class:`VariableCoefficientSolver` to solve repeatedly)."""
    n = check_grid(b, name="b")
    if abstol <= 0.0 and reltol <= 0.0:
        abstol = SQRT_EPS
    with VariableCoefficientSolver(n, coef, options) as s:
        return s.mgcg(b, x, abstol=abstol, reltol=reltol, maxiter=maxiter)
