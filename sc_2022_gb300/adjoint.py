"""Gradients through the MGCG solve: the adjoint path.

The reference has no adjoint.  Its solve composes the right-hand-side
assembly of ``Assembling_matrix`` (``level_2_multigrid_new.jl:169-185``) with
``matrix_free_MGCG`` (``preconditioned_CG/matrix_free_mg_cg.jl:281-324``):

    b = -H~ (f + sum_side SAT_side g_side),    u = A^-1 b,

linear in the source f (D2 convention, as :func:`problems.assemble_rhs`) and
in the boundary data g = (g_W, g_E, g_S, g_N).  For a loss L(u) with
g_u = dL/du the gradients are

    lam = A^-T g_u = A^-1 g_u            (A = -H~ (D2 + SAT) is SPD)
    dL/df = B_f^T lam,   dL/dg_side = B_side^T lam

i.e. one more MGCG solve with the same handle and the transposed
right-hand-side map (``sbp_mgcg_adjoint_f64``).

:class:`PoissonSolve` is the ``torch.autograd.Function`` form (the
counterpart of a ChainRulesCore ``rrule``); :func:`mgcg_rrule` returns
``(u, pullback)`` in the rrule shape; :class:`HMisfit` is the loss
L = 1/2 (u - u_t)' H~ (u - u_t) of the adjoint configuration on the GPU
(``sbp_h_misfit_f64``).  Every array is a float64 CUDA tensor; batches are a
leading dimension and share one solver handle.
"""
from __future__ import annotations

import torch

from . import _lib as L
from .solver import Solver, _stream_ptr, ptr

SIDES = ("W", "E", "S", "N")


def _batch(f: torch.Tensor, gs):
    """(f as (B, n, n), g list as (B, n) each, was_batched)."""
    batched = f.dim() == 3
    fb = f if batched else f.unsqueeze(0)
    gb = [g if g.dim() == 2 else g.unsqueeze(0) for g in gs]
    B, n = fb.shape[0], fb.shape[-1]
    if fb.shape[1:] != (n, n) or fb.dtype != torch.float64 or not fb.is_cuda:
        raise ValueError("f must be a float64 CUDA tensor of shape (n, n) or (B, n, n)")
    for g in gb:
        if g.shape != (B, n) or g.dtype != torch.float64 or g.device != fb.device:
            raise ValueError("boundary data must be float64 tensors of shape (n,) or (B, n)")
    return fb, gb, batched


def _rhs(f: torch.Tensor, gs, out: torch.Tensor, fsign: float, sp):
    n = f.shape[-1]
    L.check(L.load().sbp_rhs_f64(ptr(f), *[ptr(g) for g in gs], ptr(out), n, fsign, sp),
            "sbp_rhs_f64")


def solve_batch(solver: Solver, f: torch.Tensor, gs, reltol: float, fsign: float = 1.0,
                x0: torch.Tensor | None = None):
    """u[k] = A^-1 b(f[k], g[k]) for every batch member: MGCG from zero, or
    from x0[k] (then reltol is relative to the residual of x0)."""
    fb, gb, batched = _batch(f, gs)
    fb = fb.contiguous()
    gb = [g.contiguous() for g in gb]
    sp = _stream_ptr()
    if x0 is None:
        u = torch.zeros_like(fb)
    else:
        u = (x0 if x0.dim() == 3 else x0.unsqueeze(0)).detach().clone().contiguous()
        if u.shape != fb.shape:
            raise ValueError("x0 must have the shape of f")
    b = torch.empty_like(fb[0])
    for k in range(fb.shape[0]):
        _rhs(fb[k], [g[k] for g in gb], b, fsign, sp)
        solver.mgcg(b, u[k], reltol=reltol, raise_on_fail=True)
    return u if batched else u[0]


def adjoint_batch(solver: Solver, gu: torch.Tensor, reltol: float, fsign: float = 1.0):
    """(df, [dgW, dgE, dgS, dgN], lam) for dL/du = gu, per batch member."""
    batched = gu.dim() == 3
    gub = (gu if batched else gu.unsqueeze(0)).contiguous()
    B, n = gub.shape[0], gub.shape[-1]
    lam = torch.empty_like(gub)
    df = torch.empty_like(gub)
    dg = [torch.empty((B, n), dtype=torch.float64, device=gub.device) for _ in SIDES]
    for k in range(B):
        solver.adjoint(gub[k], lam[k], df[k], {s: dg[i][k] for i, s in enumerate(SIDES)},
                       fsign=fsign, reltol=reltol, raise_on_fail=True)
    if not batched:
        return df[0], [g[0] for g in dg], lam[0]
    return df, dg, lam


class PoissonSolve(torch.autograd.Function):
    """u = A^-1 b(f, g_W, g_E, g_S, g_N) with gradients for f and every g.

    ``PoissonSolve.apply(f, gW, gE, gS, gN, solver, reltol)``; f (n, n) or
    (B, n, n), each g (n,) or (B, n).  Backward runs the adjoint MGCG with the
    same handle and tolerance.
    """

    @staticmethod
    def forward(ctx, f, gW, gE, gS, gN, solver: Solver, reltol: float = 1e-12):
        ctx.solver = solver
        ctx.reltol = reltol
        return solve_batch(solver, f.detach(), [g.detach() for g in (gW, gE, gS, gN)], reltol)

    @staticmethod
    def backward(ctx, gu):
        df, dg, _ = adjoint_batch(ctx.solver, gu, ctx.reltol)
        return (df, *dg, None, None)


def mgcg_rrule(solver: Solver, f: torch.Tensor, g: dict, reltol: float = 1e-12):
    """rrule shape: returns (u, pullback) with pullback(du) -> (df, dg dict)."""
    gs = [g[s] for s in SIDES]
    u = solve_batch(solver, f, gs, reltol)

    def pullback(du: torch.Tensor):
        df, dg, _ = adjoint_batch(solver, du, reltol)
        return df, dict(zip(SIDES, dg))

    return u, pullback


class HMisfit(torch.autograd.Function):
    """L = sum over the batch of 1/2 (u - u_t)' H~ (u - u_t) (H~ = h^2 w_i w_j)."""

    @staticmethod
    def forward(ctx, u: torch.Tensor, ut: torch.Tensor):
        ub = (u if u.dim() == 3 else u.unsqueeze(0)).detach().contiguous()
        utb = (ut if ut.dim() == 3 else ut.unsqueeze(0)).detach().contiguous()
        if ub.shape != utb.shape or ub.dtype != torch.float64:
            raise ValueError("u and u_t must be float64 tensors of the same shape")
        n = ub.shape[-1]
        g = torch.empty_like(ub)
        losses = torch.empty(ub.shape[0], dtype=torch.float64, device=ub.device)
        sp = _stream_ptr()
        lib = L.load()
        for k in range(ub.shape[0]):
            L.check(lib.sbp_h_misfit_f64(ptr(ub[k]), ptr(utb[k]), ptr(g[k]), n,
                                         ptr(losses[k:k + 1]), sp), "sbp_h_misfit_f64")
        ctx.save_for_backward(g.reshape(u.shape))
        return losses.sum()

    @staticmethod
    def backward(ctx, grad):
        (g,) = ctx.saved_tensors
        return grad * g, -grad * g
