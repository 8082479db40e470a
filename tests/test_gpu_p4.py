"""GPU parity of the fourth-order (p = 4) operator and its CG against the
assembled oracle matrix (Assembling_matrix(level; p = 4))."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

from oracle import sbp_oracle as o

pytestmark = pytest.mark.gpu

APPLY_RTOL = 1e-13   # FP64 operator apply, relative 2-norm
SOL_RTOL = 1e-10     # CG solution vs the oracle's CG, relative 2-norm


def dev(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device="cuda").contiguous()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().ravel()


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("n", [9, 10, 17, 65, 257, 300])
def test_apply_p4_vs_assembled(sbp, n):
    rng = np.random.default_rng(40 + n)
    u = rng.standard_normal(n * n)
    A = o.assemble(n, 4).A
    ud = dev(u)
    out = torch.empty_like(ud)
    for sign in (-1, 1):
        sbp.matrix_free_A_p4_GPU(ud, out, sign=sign)
        assert relerr(host(out), sign * (A @ u)) < APPLY_RTOL


def test_apply_p4_rejects_small_grid(sbp):
    u = torch.zeros(8 * 8, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        sbp.matrix_free_A_p4_GPU(u, torch.empty_like(u))


def test_apply_p4_large_symmetry(sbp):
    # size-independent property at the benchmark size: <v, A u> = <A v, u>
    n = 4097
    g = torch.Generator(device="cuda").manual_seed(4)
    u = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    v = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    au, av = torch.empty_like(u), torch.empty_like(v)
    sbp.matrix_free_A_p4_GPU(u, au, sign=1)
    sbp.matrix_free_A_p4_GPU(v, av, sign=1)
    a, b = float(torch.dot(v, au)), float(torch.dot(av, u))
    assert abs(a - b) <= 1e-12 * float(au.norm() * v.norm())
    assert float(torch.dot(u, au)) > 0


@pytest.mark.parametrize("n", [17, 65])
def test_cg_p4_matches_oracle(sbp, n):
    a = o.assemble(n, 4)
    F, g, U = o.manufactured(n, "reference")
    b = a.rhs(F, g)
    r0 = np.linalg.norm(b)
    tol = 1e-9 * r0
    x_ref, it_ref, norms_ref = o.cg(a.A, b, abstol=tol)
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = sbp.CG_p4_GPU(dev(b), x, sign=1, abstol=tol)
    assert res.converged
    assert abs(res.iters - it_ref) <= 1
    k = min(len(norms_ref), len(res.norms), 20)
    np.testing.assert_allclose(res.norms[:k], norms_ref[:k], rtol=1e-8)
    xs = spla.spsolve(a.A.tocsc(), b)
    assert relerr(host(x), xs) < 1e-7
    assert relerr(host(x), x_ref) < 1e-7


def test_cg_p4_solution_to_1e10(sbp):
    n = 65
    a = o.assemble(n, 4)
    F, g, U = o.manufactured(n, "baseline")
    b = a.rhs(F, g)
    xs = spla.spsolve(a.A.tocsc(), b)
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = sbp.CG_p4_GPU(dev(b), x, sign=1, reltol=1e-13, maxiter=20000)
    assert res.converged
    assert relerr(host(x), xs) < SOL_RTOL
    # fourth-order discretisation: same H-norm error as the direct solve
    assert o.h_error(a, host(x), U) == pytest.approx(o.h_error(a, xs, U), rel=1e-6)
