"""Solver handles and options over the libsbpmg C ABI.

Device arrays are torch CUDA tensors used as plain device buffers: float64
(or float32 for the FP32 apply), contiguous, n*n elements.  A tensor of
shape (n, n) indexed ``t[j, i]`` has exactly the memory layout of the
reference's column-major ``CuArray{Float64,2}`` of size (n, n) indexed
``a[i, j]``; flat tensors of n*n elements are accepted as well.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import torch

from . import _lib as L


def _stream_ptr(stream=None):
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


def grid_n(t: torch.Tensor) -> int:
    """Points per side of a square grid tensor."""
    n = int(round(math.sqrt(t.numel())))
    if n * n != t.numel():
        raise ValueError(f"tensor with {t.numel()} elements is not an n x n grid")
    return n


def check_grid(t: torch.Tensor, dtype=torch.float64, name="array") -> int:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (device memory)")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return grid_n(t)


def ptr(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


@dataclass
class Options:
    """Mirror of ``sbp_options`` (include/sbpmg.h)."""
    smoother: int = L.SBP_SMOOTH_JACOBI
    omega: float = 2.0 / 3.0
    nu_pre: int = 3
    nu_post: int = 3
    restriction: int = L.SBP_RESTRICT_GALERKIN
    coarse_n: int = 65
    precision: int = L.SBP_PREC_FP64

    def to_c(self) -> L.sbp_options:
        o = L.sbp_options()
        o.smoother = self.smoother
        o.omega = self.omega
        o.nu_pre = self.nu_pre
        o.nu_post = self.nu_post
        o.restriction = self.restriction
        o.coarse_n = self.coarse_n
        o.precision = self.precision
        return o

    @staticmethod
    def from_c(o: L.sbp_options) -> "Options":
        return Options(o.smoother, o.omega, o.nu_pre, o.nu_post, o.restriction, o.coarse_n,
                       o.precision)


def default_options(precision: int = L.SBP_PREC_FP64) -> Options:
    """V-cycle preconditioner of the N=4097 configuration (Jacobi 2/3, 3+3,
    SBP-compatible restriction, direct solve at 65^2)."""
    o = L.sbp_options()
    L.load().sbp_options_default(C.byref(o))
    out = Options.from_c(o)
    out.precision = precision
    return out


def reference_two_level_options(n: int) -> Options:
    """The reference's two-level GPU preconditioner
    (``matrix_free_Two_level_multigrid``, matrix_free_mg_cg.jl:143-176)."""
    o = L.sbp_options()
    L.load().sbp_options_reference_two_level(C.byref(o), n)
    return Options.from_c(o)


@dataclass
class SolveResult:
    iters: int
    status: int
    norms: list
    initial_norm: float
    final_norm: float
    threshold: float

    @property
    def converged(self) -> bool:
        return self.status == L.SBP_OK


class Solver:
    """A libsbpmg solver handle for n x n grids.

    ``options=None`` gives a plain-CG handle; otherwise the multigrid
    hierarchy, its buffers and the coarse inverse are built (this replaces
    the reference's ``lu(Assembling_matrix(level-1))``).
    """

    def __init__(self, n: int, options: Options | None = None):
        self.n = n
        self.options = options
        lib = L.load()
        h = C.c_void_p()
        oc = options.to_c() if options is not None else None
        L.check(lib.sbp_solver_create(C.byref(h), n,
                                      C.byref(oc) if oc is not None else None),
                "sbp_solver_create")
        self._h = h
        self._lib = lib

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sbp_solver_destroy(self._h)
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
        return L.check(self._lib.sbp_solver_levels(self._h), "sbp_solver_levels")

    @property
    def device_bytes(self) -> int:
        return int(self._lib.sbp_solver_device_bytes(self._h))

    @property
    def last_launches(self) -> int:
        """Kernel launches of the last solve (set-up + iteration graphs)."""
        return int(self._lib.sbp_solver_last_launches(self._h))

    def _run(self, call, name, maxiter, raise_on_fail):
        """call(res_ptr, norms_buf, cap) -> status."""
        res = L.sbp_result()
        cap = min(maxiter, 100000) + 1
        buf = (C.c_double * cap)()
        st = call(C.byref(res), buf, cap)
        if st < 0 and (raise_on_fail or st not in (L.SBP_ERR_MAXITER, L.SBP_ERR_BREAKDOWN)):
            L.check(st, name)
        cnt = min(cap, res.iters + 1)
        return SolveResult(res.iters, st, list(buf[:cnt]), res.initial_norm, res.final_norm,
                           res.threshold)

    def _check_pair(self, b, x):
        n = check_grid(b, name="b")
        check_grid(x, name="x")
        if n != self.n or x.numel() != b.numel():
            raise ValueError(f"grid size mismatch: solver n={self.n}, b has n={n}")
        if b.device != x.device:
            raise ValueError("b and x must be on the same device")
        return n

    def mgcg(self, b: torch.Tensor, x: torch.Tensor, abstol: float = 0.0, reltol: float = 0.0,
             maxiter: int | None = None, stream=None, raise_on_fail=False) -> SolveResult:
        """MGCG on A x = b; x (initial guess) is overwritten with the solution.
        Stops at ||r|| < abstol if abstol > 0, else ||r|| < reltol*||r0||."""
        n = self._check_pair(b, x)
        maxiter = n * n if maxiter is None else maxiter
        sp = _stream_ptr(stream)
        return self._run(lambda res, buf, cap: self._lib.sbp_mgcg_solve(
            self._h, ptr(b), ptr(x), abstol, reltol, maxiter, res, buf, cap, sp),
            "sbp_mgcg_solve", maxiter, raise_on_fail)

    def cg(self, b: torch.Tensor, x: torch.Tensor, sign: int = 1, abstol: float = 0.0,
           reltol: float = 0.0, maxiter: int | None = None, stream=None,
           raise_on_fail=False) -> SolveResult:
        """Matrix-free CG on (sign*A) x = b."""
        n = self._check_pair(b, x)
        maxiter = n * n if maxiter is None else maxiter
        sp = _stream_ptr(stream)
        return self._run(lambda res, buf, cap: self._lib.sbp_cg_solve(
            self._h, ptr(b), ptr(x), sign, abstol, reltol, maxiter, res, buf, cap, sp),
            "sbp_cg_solve", maxiter, raise_on_fail)

    def adjoint(self, gu: torch.Tensor, lam: torch.Tensor, df: torch.Tensor | None = None,
                dg: dict | None = None, fsign: float = 1.0, abstol: float = 0.0,
                reltol: float = 0.0, maxiter: int | None = None, stream=None,
                raise_on_fail=True) -> SolveResult:
        """Adjoint MGCG: lam = A^-1 gu (A is SPD), then the transposed
        right-hand-side map: df = dL/df and dg[side] = dL/dg_side for
        dL/du = gu (outputs written in place; df/dg may be None)."""
        n = self._check_pair(gu, lam)
        maxiter = n * n if maxiter is None else maxiter
        sp = _stream_ptr(stream)
        dg = dg or {}
        for k, t in dg.items():
            if t.dtype != torch.float64 or t.numel() != n or not t.is_contiguous():
                raise ValueError(f"dg[{k!r}] must be a contiguous float64 vector of length {n}")
        if df is not None:
            check_grid(df, name="df")
        outs = [ptr(df) if df is not None else None] + [
            ptr(dg[k]) if dg.get(k) is not None else None for k in ("W", "E", "S", "N")]
        res = L.sbp_result()
        st = self._lib.sbp_mgcg_adjoint_f64(self._h, ptr(gu), ptr(lam), *outs, fsign, abstol,
                                             reltol, maxiter, C.byref(res), sp)
        if st < 0 and (raise_on_fail or st not in (L.SBP_ERR_MAXITER, L.SBP_ERR_BREAKDOWN)):
            L.check(st, "sbp_mgcg_adjoint_f64")
        return SolveResult(res.iters, st, [], res.initial_norm, res.final_norm, res.threshold)

    def profile(self, b: torch.Tensor, x: torch.Tensor, kind: str = "mgcg", sign: int = 1,
                reltol: float = 1e-10, maxiter: int | None = None, stream=None):
        """One solve (``kind`` "mgcg" or "cg") launched without CUDA graphs,
        with CUDA events around every kernel launch.  Returns (SolveResult,
        [{"kernel", "launches", "total_ms", "ms_per_launch"}, ...]) sorted by
        total time; x is overwritten with the solution."""
        n = self._check_pair(b, x)
        maxiter = n * n if maxiter is None else maxiter
        cap = 64
        out = (L.sbp_kernel_time * cap)()
        cnt = C.c_int(0)
        res = L.sbp_result()
        st = self._lib.sbp_solver_profile(self._h, 0 if kind == "mgcg" else 1, ptr(b), ptr(x),
                                          sign, reltol, maxiter, C.byref(res), out, cap,
                                          C.byref(cnt), _stream_ptr(stream))
        if st < 0 and st not in (L.SBP_ERR_MAXITER, L.SBP_ERR_BREAKDOWN):
            L.check(st, "sbp_solver_profile")
        rows = [{"kernel": out[k].name.decode(), "launches": out[k].launches,
                 "total_ms": out[k].total_ms,
                 "ms_per_launch": out[k].total_ms / max(out[k].launches, 1)}
                for k in range(min(cnt.value, cap))]
        return SolveResult(res.iters, st, [], res.initial_norm, res.final_norm,
                           res.threshold), rows

    def vcycle(self, b: torch.Tensor, v: torch.Tensor, stream=None) -> torch.Tensor:
        """v = M b, one V-cycle from zero."""
        check_grid(b, name="b")
        check_grid(v, name="v")
        L.check(self._lib.sbp_vcycle_apply(self._h, ptr(b), ptr(v), _stream_ptr(stream)),
                "sbp_vcycle_apply")
        return v


class BatchSolver:
    """Batched MGCG over independent problems of any grid sizes (one solver
    per problem; the problems of one size share every kernel launch, sizes
    run as parallel graph branches).  ``options`` as for :class:`Solver`."""

    def __init__(self, ns, options: Options):
        self.ns = [int(n) for n in ns]
        lib = L.load()
        h = C.c_void_p()
        arr = (C.c_int * len(self.ns))(*self.ns)
        oc = options.to_c()
        L.check(lib.sbp_batch_create(C.byref(h), arr, len(self.ns), C.byref(oc)),
                "sbp_batch_create")
        self._h = h
        self._lib = lib
        self.options = options

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sbp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.ns)

    @property
    def device_bytes(self) -> int:
        return int(self._lib.sbp_batch_device_bytes(self._h))

    @property
    def last_launches(self) -> int:
        return int(self._lib.sbp_batch_last_launches(self._h))

    @property
    def classes(self) -> list:
        cnt = self._lib.sbp_batch_classes(self._h, None, 0)
        arr = (C.c_int * max(cnt, 1))()
        self._lib.sbp_batch_classes(self._h, arr, cnt)
        return list(arr[:cnt])

    def autotune(self, bs, xs, stream=None) -> dict:
        """Choose each grid size's CTA budget by timing a few iterations on
        these problems (xs are overwritten).  Returns {n: budget} (0 = one
        full wave)."""
        cnt = len(self.ns)
        bp = (C.c_void_p * cnt)(*[b.data_ptr() for b in bs])
        xp = (C.c_void_p * cnt)(*[x.data_ptr() for x in xs])
        cls = self.classes
        out = (C.c_int * len(cls))()
        L.check(self._lib.sbp_batch_autotune(self._h, bp, xp, out, _stream_ptr(stream)),
                "sbp_batch_autotune")
        return dict(zip(cls, list(out)))

    def mgcg(self, bs, xs, abstol: float = 0.0, reltol: float = 0.0, maxiter: int | None = None,
             stream=None, raise_on_fail=False):
        """MGCG on every problem: xs[k] (initial guesses) are overwritten.
        Returns one SolveResult per problem (norm histories not kept)."""
        if len(bs) != len(self.ns) or len(xs) != len(self.ns):
            raise ValueError("one b and one x per problem")
        for k, (b, x, n) in enumerate(zip(bs, xs, self.ns)):
            if check_grid(b, name=f"b[{k}]") != n or check_grid(x, name=f"x[{k}]") != n:
                raise ValueError(f"problem {k}: grid size differs from n={n}")
        cnt = len(self.ns)
        maxiter = max(n * n for n in self.ns) if maxiter is None else maxiter
        bp = (C.c_void_p * cnt)(*[b.data_ptr() for b in bs])
        xp = (C.c_void_p * cnt)(*[x.data_ptr() for x in xs])
        res = (L.sbp_result * cnt)()
        st = self._lib.sbp_batch_mgcg_solve(self._h, bp, xp, abstol, reltol, maxiter, res,
                                             _stream_ptr(stream))
        if st < 0 and (raise_on_fail or st not in (L.SBP_ERR_MAXITER, L.SBP_ERR_BREAKDOWN)):
            L.check(st, "sbp_batch_mgcg_solve")
        return [SolveResult(r.iters, r.status, [], r.initial_norm, r.final_norm, r.threshold)
                for r in res]
