"""GPU parity of the higher-order (p = 4, 6) operators and solvers against
the assembled oracle matrices (Assembling_matrix(level; p)) and the oracle's
order-p multigrid."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

from oracle import sbp_oracle as o

pytestmark = pytest.mark.gpu

APPLY_RTOL = 1e-13   # FP64 operator apply, relative 2-norm
VCYCLE_RTOL = 1e-12  # one V-cycle vs the oracle's, relative 2-norm
SOL_RTOL = 1e-10     # solutions vs a sparse direct solve, relative 2-norm


def dev(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device="cuda").contiguous()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().ravel()


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def mg_options(sbp, coarse_n=33, smoother="jacobi"):
    opts = sbp.default_options()
    opts.coarse_n = coarse_n
    if smoother == "richardson":
        opts.smoother = 1
        opts.omega = 0.15
    return opts


@pytest.mark.parametrize("p,n", [(4, 8), (4, 9), (4, 10), (4, 17), (4, 65), (4, 257), (4, 300),
                                 (6, 12), (6, 13), (6, 17), (6, 65), (6, 257), (6, 301)])
def test_apply_vs_assembled(sbp, p, n):
    rng = np.random.default_rng(40 + n + p)
    u = rng.standard_normal(n * n)
    A = o.assemble(n, p).A
    ud = dev(u)
    out = torch.empty_like(ud)
    for sign in (-1, 1):
        sbp.matrix_free_A_high_order_GPU(ud, out, p=p, sign=sign)
        assert relerr(host(out), sign * (A @ u)) < APPLY_RTOL


@pytest.mark.parametrize("p,n", [(4, 7), (6, 11)])
def test_apply_rejects_small_grid(sbp, p, n):
    u = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        sbp.matrix_free_A_high_order_GPU(u, torch.empty_like(u), p=p)


@pytest.mark.parametrize("p", [4, 6])
def test_apply_large_symmetry(sbp, p):
    # size-independent property at the benchmark size: <v, A u> = <A v, u>, A SPD
    n = 4097
    g = torch.Generator(device="cuda").manual_seed(p)
    u = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    v = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    au, av = torch.empty_like(u), torch.empty_like(v)
    sbp.matrix_free_A_high_order_GPU(u, au, p=p, sign=1)
    sbp.matrix_free_A_high_order_GPU(v, av, p=p, sign=1)
    a, b = float(torch.dot(v, au)), float(torch.dot(av, u))
    assert abs(a - b) <= 1e-12 * float(au.norm() * v.norm())
    assert float(torch.dot(u, au)) > 0


@pytest.mark.parametrize("p,n", [(4, 17), (4, 65), (6, 33), (6, 65)])
def test_cg_matches_oracle(sbp, p, n):
    a = o.assemble(n, p)
    F, g, U = o.manufactured(n, "reference")
    b = a.rhs(F, g)
    tol = 1e-9 * np.linalg.norm(b)
    x_ref, it_ref, norms_ref = o.cg(a.A, b, abstol=tol)
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = sbp.CG_high_order_GPU(dev(b), x, p=p, sign=1, abstol=tol)
    assert res.converged
    assert abs(res.iters - it_ref) <= 1
    k = min(len(norms_ref), len(res.norms), 20)
    np.testing.assert_allclose(res.norms[:k], norms_ref[:k], rtol=1e-8)
    assert relerr(host(x), x_ref) < 1e-7


def test_cg_negative_sign_matches_positive(sbp):
    # (-A) x = -b has the solution of A x = b (the reference's GPU sign)
    n, p = 33, 4
    a = o.assemble(n, p)
    F, g, U = o.manufactured(n, "baseline")
    b = a.rhs(F, g)
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = sbp.CG_high_order_GPU(dev(-b), x, p=p, sign=-1, reltol=1e-12, maxiter=5000)
    assert res.converged
    assert relerr(host(x), spla.spsolve(a.A.tocsc(), b)) < 1e-9


@pytest.mark.parametrize("p,n,smoother", [(4, 129, "jacobi"), (6, 129, "jacobi"),
                                          (4, 65, "richardson"), (6, 257, "jacobi")])
def test_vcycle_matches_oracle(sbp, p, n, smoother):
    opts = mg_options(sbp, 33, smoother)
    hier = o.Hierarchy(n, o.MGOptions(smoother=smoother, omega=opts.omega, restriction="galerkin",
                                      coarse_n=33), p)
    rng = np.random.default_rng(7 + n + p)
    b = rng.standard_normal(n * n)
    want = hier.vcycle(b)
    s = sbp.HighOrderSolver(n, p, opts)
    assert s.levels == len(hier.ns)
    v = torch.empty(n * n, dtype=torch.float64, device="cuda")
    s.vcycle(dev(b), v)
    assert relerr(host(v), want) < VCYCLE_RTOL


@pytest.mark.parametrize("p,n", [(4, 65), (4, 257), (6, 129), (6, 257)])
def test_mgcg_matches_oracle(sbp, p, n):
    hier = o.Hierarchy(n, o.MGOptions(restriction="galerkin", coarse_n=33), p)
    a = hier.asm[0]
    F, g, U = o.manufactured(n, "baseline")
    b = a.rhs(F, g)
    x_ref, it_ref, norms_ref = o.mgcg(hier, b, reltol=1e-10)
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    s = sbp.HighOrderSolver(n, p, mg_options(sbp, 33))
    res = s.mgcg(dev(b), x, reltol=1e-10)
    assert res.converged
    assert abs(res.iters - it_ref) <= 1
    k = min(len(res.norms), len(norms_ref))
    np.testing.assert_allclose(res.norms[:k], norms_ref[:k], rtol=1e-7)
    xs = spla.spsolve(a.A.tocsc(), b)
    assert relerr(host(x), xs) < SOL_RTOL * 10
    # the same iterate as the oracle's MGCG
    assert relerr(host(x), x_ref) < 1e-8


def test_mgcg_single_direct_level(sbp):
    # n <= coarse_n: the whole problem is the fast-diagonalisation solve
    n, p = 33, 6
    a = o.assemble(n, p)
    b = np.random.default_rng(3).standard_normal(n * n)
    s = sbp.HighOrderSolver(n, p, mg_options(sbp, 65))
    assert s.levels == 1
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = s.mgcg(dev(b), x, reltol=1e-12)
    assert res.converged and res.iters <= 2
    assert relerr(host(x), spla.spsolve(a.A.tocsc(), b)) < SOL_RTOL


def test_cg_only_handle_for_ragged_grid(sbp):
    # a ragged grid below the coarse size is one direct level ...
    assert sbp.HighOrderSolver(50, 4).levels == 1
    # ... above it, not 2^k + 1, the handle does CG only
    n, p = 300, 4
    s = sbp.HighOrderSolver(n, p)
    assert s.levels == 0
    b = dev(np.ones(n * n))
    x = torch.zeros_like(b)
    with pytest.raises(sbp.SbpError):
        s.mgcg(b, x, reltol=1e-8)
    res = s.cg(b, x, reltol=1e-10, maxiter=20000)
    assert res.converged
    a = o.assemble(n, p)
    assert relerr(host(x), spla.spsolve(a.A.tocsc(), np.ones(n * n))) < 1e-8


@pytest.mark.parametrize("p", [4, 6])
def test_mgcg_n4097_residual(sbp, p):
    # full size: the true residual of the returned x, by an independent apply,
    # meets the 1e-10 relative tolerance; iterations stay h-independent
    n = 4097
    g = torch.Generator(device="cuda").manual_seed(11)
    b = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    x = torch.zeros_like(b)
    s = sbp.HighOrderSolver(n, p)
    res = s.mgcg(b, x, reltol=1e-10, maxiter=100)
    assert res.converged
    assert res.iters <= (12 if p == 4 else 16)
    ax = torch.empty_like(x)
    sbp.matrix_free_A_high_order_GPU(x, ax, p=p, sign=1)
    assert float((b - ax).norm() / b.norm()) < 2e-10


MIXED_VCYCLE_RTOL = 2e-5   # FP32 V-cycle vs the FP64 oracle's, relative 2-norm


@pytest.mark.parametrize("p,n", [(4, 129), (6, 257)])
def test_mixed_vcycle_close_to_fp64_oracle(sbp, p, n):
    opts = mg_options(sbp, 33)
    opts.precision = 1   # SBP_PREC_MIXED
    hier = o.Hierarchy(n, o.MGOptions(restriction="galerkin", coarse_n=33), p)
    b = np.random.default_rng(17 + p).standard_normal(n * n)
    want = hier.vcycle(b)
    s = sbp.HighOrderSolver(n, p, opts)
    v = torch.empty(n * n, dtype=torch.float64, device="cuda")
    s.vcycle(dev(b), v)
    assert relerr(host(v), want) < MIXED_VCYCLE_RTOL


@pytest.mark.parametrize("p,n", [(4, 257), (6, 257)])
def test_mixed_mgcg_matches_fp64(sbp, p, n):
    # the FP32 V-cycle inside FP64 PCG: the FP64 iteration count (+-1) and a
    # solution at the FP64 tolerance
    a = o.assemble(n, p)
    F, g, U = o.manufactured(n, "baseline")
    b = a.rhs(F, g)
    xs = spla.spsolve(a.A.tocsc(), b)
    its = {}
    for prec in (0, 1):
        opts = mg_options(sbp, 33)
        opts.precision = prec
        s = sbp.HighOrderSolver(n, p, opts)
        x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        res = s.mgcg(dev(b), x, reltol=1e-10)
        assert res.converged
        its[prec] = res.iters
        assert relerr(host(x), xs) < SOL_RTOL * 10
    assert abs(its[1] - its[0]) <= 1


@pytest.mark.parametrize("p", [4, 6])
def test_mixed_mgcg_n4097_residual(sbp, p):
    n = 4097
    g = torch.Generator(device="cuda").manual_seed(12)
    b = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    x = torch.zeros_like(b)
    opts = sbp.default_options(1)
    s = sbp.HighOrderSolver(n, p, opts)
    res = s.mgcg(b, x, reltol=1e-10, maxiter=100)
    assert res.converged
    assert res.iters <= (12 if p == 4 else 16)
    ax = torch.empty_like(x)
    sbp.matrix_free_A_high_order_GPU(x, ax, p=p, sign=1)
    assert float((b - ax).norm() / b.norm()) < 2e-10
