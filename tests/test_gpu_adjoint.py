"""GPU parity of the adjoint path: gradients of L = 1/2 |u - u_t|_H^2, with
u = A^-1 b(f, g), with respect to the source f and the four boundary
vectors, against the oracle's direct-solve gradient and against central
finite differences."""
import numpy as np
import pytest
import torch

from oracle import sbp_oracle as o

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device="cuda").contiguous()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().ravel()


def relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n,coarse", [(65, 17), (129, 33)])
def test_adjoint_matches_oracle(sbp, n, coarse):
    asm = o.assemble(n)
    rng = np.random.default_rng(5)
    f = rng.standard_normal(n * n)
    g = {s: rng.standard_normal(n) for s in "WESN"}
    ut = 0.01 * rng.standard_normal(n * n)
    L_ref, df_ref, dg_ref, u_ref, lam_ref = o.misfit_loss_grad(asm, f, g, ut)
    opts = sbp.default_options()
    opts.coarse_n = coarse
    s = sbp.Solver(n, opts)
    fv = dev(f).reshape(n, n).clone().requires_grad_()
    gv = {k: dev(g[k]).clone().requires_grad_() for k in "WESN"}
    u = sbp.PoissonSolve.apply(fv, gv["W"], gv["E"], gv["S"], gv["N"], s, 1e-14)
    loss = sbp.HMisfit.apply(u, dev(ut).reshape(n, n))
    loss.backward()
    assert relerr(host(u), u_ref) < 1e-10
    assert abs(loss.item() - L_ref) <= 1e-10 * abs(L_ref)
    assert relerr(host(fv.grad), df_ref) < 1e-9
    for k in "WESN":
        assert relerr(host(gv[k].grad), dg_ref[k]) < 1e-9


def test_rrule_pullback_and_lambda(sbp):
    # mgcg_rrule returns (u, pullback); the adjoint state is A^-1 g_u
    from sc_2022_gb300 import adjoint
    n = 65
    asm = o.assemble(n)
    rng = np.random.default_rng(8)
    f = rng.standard_normal(n * n)
    g = {s: rng.standard_normal(n) for s in "WESN"}
    s = sbp.Solver(n, sbp.default_options())
    u, pullback = sbp.mgcg_rrule(s, dev(f).reshape(n, n), {k: dev(g[k]) for k in "WESN"}, 1e-14)
    gu = rng.standard_normal(n * n)
    df, dg = pullback(dev(gu).reshape(n, n))
    lam = np.linalg.solve(asm.A.toarray(), gu)
    hl = asm.H_tilde @ lam
    assert relerr(host(df), -hl) < 1e-9
    for k in "WESN":
        assert relerr(host(dg[k]), -(asm.sat_r[k].T @ hl)) < 1e-9
    _, _, lam_gpu = adjoint.adjoint_batch(s, dev(gu).reshape(n, n), 1e-14)
    assert relerr(host(lam_gpu), lam) < 1e-10


def _config5(n, batch):
    from sc_2022_gb300 import problems
    fs, fts, gs = [], [], {k: [] for k in "WESN"}
    for b in range(batch):
        f, g = problems.bump_problem(n, seed=100 + b)
        fp, _ = problems.bump_problem(n, seed=1000 + b)
        fs.append(f)
        fts.append(f + 0.1 * fp)         # perturbed random-bump source of the target
        for k in "WESN":
            gs[k].append(g[k])
    F = dev(np.stack(fs)).reshape(batch, n, n)
    Ft = dev(np.stack(fts)).reshape(batch, n, n)
    G = {k: dev(np.stack(gs[k])) for k in "WESN"}
    return F, Ft, G


def test_gradient_n2049_batch16_finite_differences(sbp):
    # N = 2049, batch 16: gradients of L = sum_b 1/2 |u_b - u_t,b|_H^2 with
    # respect to f (2049^2 per problem) and the Dirichlet/Neumann vectors,
    # checked by central differences (step 1e-6) along 32 seeded directions
    # (FP64 solves; relative agreement 1e-7).
    from sc_2022_gb300 import adjoint
    n, batch = 2049, 16
    F, Ft, G = _config5(n, batch)
    s = sbp.Solver(n, sbp.default_options())
    tol = 1e-13
    Ut = adjoint.solve_batch(s, Ft, [G[k] for k in "WESN"], tol)
    Fv = F.clone().requires_grad_()
    Gv = {k: G[k].clone().requires_grad_() for k in "WESN"}
    u = sbp.PoissonSolve.apply(Fv, Gv["W"], Gv["E"], Gv["S"], Gv["N"], s, tol)
    L = sbp.HMisfit.apply(u, Ut)
    L.backward()

    u0 = u.detach()

    def loss_at(Fx, Gx):
        # warm start from the unperturbed solution: the solve then resolves
        # the 1e-6 perturbation itself to 1e-11 of its own residual
        ux = adjoint.solve_batch(s, Fx, [Gx[k] for k in "WESN"], 1e-11, x0=u0)
        return sbp.HMisfit.apply(ux, Ut).item()

    gen = torch.Generator(device="cuda").manual_seed(7)
    fscale = F.abs().mean().item()
    eps = 1e-6
    worst = 0.0
    for _ in range(32):
        dF = torch.randn(F.shape, generator=gen, device="cuda", dtype=torch.float64) * fscale
        dG = {k: torch.randn(G[k].shape, generator=gen, device="cuda", dtype=torch.float64)
              for k in "WESN"}
        lp = loss_at(F + eps * dF, {k: G[k] + eps * dG[k] for k in "WESN"})
        lm = loss_at(F - eps * dF, {k: G[k] - eps * dG[k] for k in "WESN"})
        fd = (lp - lm) / (2 * eps)
        an = (Fv.grad * dF).sum().item() + sum((Gv[k].grad * dG[k]).sum().item() for k in "WESN")
        worst = max(worst, abs(fd - an) / abs(an))
    assert worst < 1e-7, worst


def test_gradient_mixed_precision_matches_fp64(sbp):
    # the same gradients through the mixed-precision solver (FP32 V-cycle)
    from sc_2022_gb300 import _lib, adjoint
    n, batch = 1025, 2
    F, Ft, G = _config5(n, batch)
    grads = []
    for prec in (_lib.SBP_PREC_FP64, _lib.SBP_PREC_MIXED):
        s = sbp.Solver(n, sbp.default_options(prec))
        Ut = adjoint.solve_batch(s, Ft, [G[k] for k in "WESN"], 1e-12)
        Fv = F.clone().requires_grad_()
        Gv = {k: G[k].clone().requires_grad_() for k in "WESN"}
        u = sbp.PoissonSolve.apply(Fv, Gv["W"], Gv["E"], Gv["S"], Gv["N"], s, 1e-12)
        sbp.HMisfit.apply(u, Ut).backward()
        grads.append([host(Fv.grad)] + [host(Gv[k].grad) for k in "WESN"])
        s.close()
    for a, b in zip(grads[1], grads[0]):
        assert relerr(a, b) < 1e-7
