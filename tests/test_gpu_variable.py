"""GPU parity of the variable-coefficient operator (div(c grad u)) and its
solvers against the oracle's assembly of variable_diagonal_sbp_D2 per grid
line and the oracle's multigrid with harmonic-mean coarse coefficients."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

from oracle import sbp_oracle as o

pytestmark = pytest.mark.gpu

APPLY_RTOL = 1e-13
VCYCLE_RTOL = 1e-12
SOL_RTOL = 1e-10


def dev(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device="cuda").contiguous()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().ravel()


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def opts_for(sbp, coarse_n=17, precision=0, smoother="jacobi"):
    op = sbp.default_options(precision)
    op.coarse_n = coarse_n
    if smoother == "richardson":
        op.smoother = 1
        op.omega = 0.15
    return op


@pytest.mark.parametrize("n", [3, 4, 9, 17, 65, 257, 300])
@pytest.mark.parametrize("kind", ["smooth", "layered"])
def test_apply_vs_assembled(sbp, n, kind):
    c = o.coefficient_field(n, kind)
    A = o.assemble_variable(n, c).A
    u = np.random.default_rng(n).standard_normal(n * n)
    ud, cd = dev(u), dev(c)
    out = torch.empty_like(ud)
    for sign in (-1, 1):
        sbp.matrix_free_A_variable_GPU(ud, cd, out, sign=sign)
        assert relerr(host(out), sign * (A @ u)) < APPLY_RTOL


def test_apply_unit_coefficient_is_constant_operator(sbp):
    n = 513
    u = torch.randn(n * n, device="cuda", dtype=torch.float64,
                    generator=torch.Generator(device="cuda").manual_seed(5))
    a, b = torch.empty_like(u), torch.empty_like(u)
    sbp.matrix_free_A_variable_GPU(u, torch.ones_like(u), a)
    sbp.matrix_free_A_full_GPU(u, b)
    assert float((a - b).norm() / b.norm()) < 1e-15


def test_apply_large_symmetry(sbp):
    n = 4097
    g = torch.Generator(device="cuda").manual_seed(9)
    u = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    v = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    c = dev(o.coefficient_field(n, "layered"))
    au, av = torch.empty_like(u), torch.empty_like(v)
    sbp.matrix_free_A_variable_GPU(u, c, au, sign=1)
    sbp.matrix_free_A_variable_GPU(v, c, av, sign=1)
    assert abs(float(torch.dot(v, au)) - float(torch.dot(av, u))) <= 1e-12 * float(
        au.norm() * v.norm())
    assert float(torch.dot(u, au)) > 0


@pytest.mark.parametrize("n", [17, 65])
def test_cg_matches_oracle(sbp, n):
    c, F, g, U = o.manufactured_variable(n)
    a = o.assemble_variable(n, c)
    b = a.rhs(F, g)
    tol = 1e-9 * np.linalg.norm(b)
    x_ref, it_ref, norms_ref = o.cg(a.A, b, abstol=tol)
    s = sbp.VariableCoefficientSolver(n, dev(c))
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = s.cg(dev(b), x, abstol=tol)
    assert res.converged and abs(res.iters - it_ref) <= 1
    k = min(len(norms_ref), len(res.norms), 20)
    np.testing.assert_allclose(res.norms[:k], norms_ref[:k], rtol=1e-8)
    assert relerr(host(x), x_ref) < 1e-7


@pytest.mark.parametrize("n,kind,smoother", [(65, "smooth", "jacobi"), (129, "layered", "jacobi"),
                                             (65, "layered", "richardson")])
def test_vcycle_matches_oracle(sbp, n, kind, smoother):
    c = o.coefficient_field(n, kind)
    op = opts_for(sbp, 17, 0, smoother)
    hier = o.Hierarchy(n, o.MGOptions(smoother=smoother, omega=op.omega, restriction="galerkin",
                                      coarse_n=17), coef=c)
    b = np.random.default_rng(3).standard_normal(n * n)
    want = hier.vcycle(b)
    s = sbp.VariableCoefficientSolver(n, dev(c), op)
    assert s.levels == len(hier.ns)
    v = torch.empty(n * n, dtype=torch.float64, device="cuda")
    s.vcycle(dev(b), v)
    assert relerr(host(v), want) < VCYCLE_RTOL


@pytest.mark.parametrize("n,kind", [(65, "smooth"), (257, "layered")])
def test_mgcg_matches_oracle(sbp, n, kind):
    c = o.coefficient_field(n, kind)
    hier = o.Hierarchy(n, o.MGOptions(restriction="galerkin", coarse_n=17), coef=c)
    b = np.random.default_rng(4).standard_normal(n * n)
    x_ref, it_ref, norms_ref = o.mgcg(hier, b, reltol=1e-10)
    s = sbp.VariableCoefficientSolver(n, dev(c), opts_for(sbp, 17))
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = s.mgcg(dev(b), x, reltol=1e-10)
    assert res.converged and abs(res.iters - it_ref) <= 1
    k = min(len(res.norms), len(norms_ref))
    np.testing.assert_allclose(res.norms[:k], norms_ref[:k], rtol=1e-7)
    assert relerr(host(x), x_ref) < 1e-8
    xs = spla.spsolve(hier.A[0].tocsc(), b)
    assert relerr(host(x), xs) < SOL_RTOL * 100


def test_mgcg_manufactured_second_order(sbp):
    # div(c grad u) = f with u = sin(pi x) cos(pi y): the GPU MGCG solution
    # converges at second order (the H-norm error falls 4x per refinement)
    errs = []
    for n in (65, 129, 257):
        c, F, g, U = o.manufactured_variable(n)
        a = o.assemble_variable(n, c)
        s = sbp.VariableCoefficientSolver(n, dev(c), opts_for(sbp, 33))
        x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        res = s.mgcg(dev(a.rhs(F, g)), x, reltol=1e-12)
        assert res.converged
        errs.append(o.h_error(a, host(x), U))
    assert 3.8 < errs[0] / errs[1] < 4.2 and 3.8 < errs[1] / errs[2] < 4.2


@pytest.mark.parametrize("kind", ["smooth", "layered"])
def test_mixed_mgcg_matches_fp64(sbp, kind):
    n = 257
    c = o.coefficient_field(n, kind)
    b = dev(np.random.default_rng(6).standard_normal(n * n))
    its = {}
    xs = {}
    for prec in (0, 1):
        s = sbp.VariableCoefficientSolver(n, dev(c), opts_for(sbp, 33, prec))
        x = torch.zeros_like(b)
        res = s.mgcg(b, x, reltol=1e-10)
        assert res.converged
        its[prec], xs[prec] = res.iters, host(x)
    assert abs(its[1] - its[0]) <= 1
    assert relerr(xs[1], xs[0]) < 1e-8


def test_cg_only_handle_and_direct_level(sbp):
    c = o.coefficient_field(30, "smooth")
    s = sbp.VariableCoefficientSolver(30, dev(c))
    assert s.levels == 1          # n <= 33: one direct level
    b = np.random.default_rng(8).standard_normal(900)
    x = torch.zeros(900, dtype=torch.float64, device="cuda")
    res = s.mgcg(dev(b), x, reltol=1e-12)
    assert res.converged and res.iters <= 2
    assert relerr(host(x), spla.spsolve(o.assemble_variable(30, c).A.tocsc(), b)) < SOL_RTOL
    c2 = o.coefficient_field(100, "smooth")
    s2 = sbp.VariableCoefficientSolver(100, dev(c2))
    assert s2.levels == 0
    x2 = torch.zeros(10000, dtype=torch.float64, device="cuda")
    with pytest.raises(sbp.SbpError):
        s2.mgcg(dev(np.ones(10000)), x2, reltol=1e-8)
    assert s2.cg(dev(np.ones(10000)), x2, reltol=1e-10, maxiter=5000).converged


@pytest.mark.parametrize("precision", [0, 1])
def test_mgcg_n4097_residual(sbp, precision):
    n = 4097
    c = dev(o.coefficient_field(n, "layered"))
    g = torch.Generator(device="cuda").manual_seed(13)
    b = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    x = torch.zeros_like(b)
    s = sbp.VariableCoefficientSolver(n, c, sbp.default_options(precision))
    res = s.mgcg(b, x, reltol=1e-10, maxiter=200)
    assert res.converged
    ax = torch.empty_like(x)
    sbp.matrix_free_A_variable_GPU(x, c, ax, sign=1)
    assert float((b - ax).norm() / b.norm()) < 2e-10
