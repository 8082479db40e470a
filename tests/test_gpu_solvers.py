"""GPU parity of the CG / MGCG solvers against the CPU oracle."""
import math

import numpy as np
import pytest
import torch

from oracle import sbp_oracle as o

pytestmark = pytest.mark.gpu

SQRT_EPS = math.sqrt(np.finfo(float).eps)


def dev(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device="cuda").contiguous()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().ravel()


def relerr(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def ref_problem(n, kind="reference"):
    a = o.assemble(n)
    F, g, U = o.manufactured(n, kind)
    return a, a.rhs(F, g), U


def test_cg_matches_oracle(sbp, golden):
    n = 33
    b = golden["ref33_b"]
    s = sbp.Solver(n)
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = s.cg(dev(b), x, sign=1, abstol=np.linalg.norm(b) * SQRT_EPS)
    ref = golden["ref33_cg_norms"]
    assert res.converged and res.iters == len(ref) - 1
    np.testing.assert_allclose(res.norms, ref, rtol=1e-6)
    assert relerr(host(x), golden["ref33_cg_x"]) < 1e-10


def test_cg_full_gpu_reference_semantics(sbp):
    # CG_full_GPU iterates with matrix_free_A_full_GPU (-A): solves (-A) x = b
    n = 65
    a, b, _ = ref_problem(n)
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    abstol = np.linalg.norm(b) * SQRT_EPS
    iters, tol, last = sbp.CG_full_GPU(dev(b), x, abstol=abstol)
    xr, itr, nr = o.cg(-a.A, b, abstol=abstol)
    # 187 CG iterations: rounding differences grow along the run, so the
    # iteration count and the solution are compared, and the last reported
    # norm to a few percent.
    assert abs(iters - itr) <= 1 and tol == abstol
    assert last == pytest.approx(nr[-2], rel=5e-2)
    assert relerr(host(x), xr) < 1e-8


@pytest.mark.parametrize("n,expect", [(33, 18), (65, 19), (129, 18), (257, 17), (513, 17),
                                      (1025, 15), (2049, 15)])
def test_mgcg_reference_two_level(sbp, n, expect):
    # the reference's matrix_free_MGCG with its two-level preconditioner and an
    # exact coarse solve at (n+1)/2 (coarse grids above 257 get their
    # fast-diagonalisation eigenbases from the GPU eigen-solver)
    a, b, U = ref_problem(n)
    hier = o.Hierarchy(n, o.MGOptions.reference_two_level(n))
    xr, itr, nr = o.mgcg(hier, b)
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    abstol = np.linalg.norm(b) * SQRT_EPS
    iters, norms, xo = sbp.matrix_free_MGCG(dev(b), x, abstol=abstol)
    assert iters == itr == expect
    np.testing.assert_allclose(norms, nr, rtol=1e-8)
    assert relerr(host(x), xr) < 1e-10


def test_two_level_vcycle_matches(sbp):
    n = 65
    a, b, _ = ref_problem(n)
    hier = o.Hierarchy(n, o.MGOptions.reference_two_level(n))
    z_ref = hier.vcycle(b)
    v, resnorm = sbp.matrix_free_Two_level_multigrid(dev(b))
    assert relerr(host(v), z_ref) < 1e-12
    assert resnorm == pytest.approx(np.linalg.norm(a.A @ z_ref - b), rel=1e-9)


def test_vcycle_mgcg_golden(sbp, golden):
    n = 65
    b = golden["base65_b"]
    opts = sbp.default_options()
    opts.coarse_n = 17
    s = sbp.Solver(n, opts)
    assert s.levels == 3
    z = torch.empty(n * n, dtype=torch.float64, device="cuda")
    s.vcycle(dev(b), z)
    assert relerr(host(z), golden["base65_vcycle17_z"]) < 1e-12
    x = torch.zeros_like(z)
    res = s.mgcg(dev(b), x, reltol=1e-10)
    ref = golden["base65_vcycle17_norms"]
    assert res.converged and res.iters == len(ref) - 1
    np.testing.assert_allclose(res.norms, ref, rtol=1e-7)
    assert relerr(host(x), golden["base65_vcycle17_x"]) < 1e-10


@pytest.mark.parametrize("n", [129, 257, 513])
def test_mgcg_vcycle_default(sbp, n):
    a, b, U = ref_problem(n, "baseline")
    hier = o.Hierarchy(n, o.MGOptions(coarse_n=65))
    xr, itr, nr = o.mgcg(hier, b, reltol=1e-10)
    s = sbp.Solver(n, sbp.default_options())
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = s.mgcg(dev(b), x, reltol=1e-10)
    assert res.converged and res.iters == itr
    np.testing.assert_allclose(res.norms, nr, rtol=1e-6)
    assert relerr(host(x), xr) < 1e-10


@pytest.mark.parametrize("n", [257, 1025])
def test_mgcg_mixed_precision(sbp, n):
    from sc_2022_gb300 import _lib
    a, b, U = ref_problem(n, "baseline")
    bd = dev(b)
    s64 = sbp.Solver(n, sbp.default_options())
    x64 = torch.zeros_like(bd)
    r64 = s64.mgcg(bd, x64, reltol=1e-10)
    s32 = sbp.Solver(n, sbp.default_options(_lib.SBP_PREC_MIXED))
    x32 = torch.zeros_like(bd)
    r32 = s32.mgcg(bd, x32, reltol=1e-10)
    assert r64.converged and r32.converged
    assert r32.iters <= r64.iters + 2
    # true FP64 residual of the mixed solution
    import ctypes as C
    lib = sbp.load_library()
    out = C.c_double()
    assert lib.sbp_residual_norm_f64(C.c_void_p(x32.data_ptr()), C.c_void_p(bd.data_ptr()), n, 1,
                                     C.byref(out), None) == 0
    assert out.value <= 2e-10 * np.linalg.norm(b)
    assert relerr(host(x32), host(x64)) < 1e-8


@pytest.mark.parametrize("n,smoother,nu,restriction", [
    (513, "jacobi", 3, "galerkin"),
    (513, "jacobi", 2, "normal"),
    (513, "richardson", 1, "sbp"),
    (1025, "jacobi", 3, "galerkin"),
    (1025, "richardson", 3, "normal"),
    (1025, "jacobi", 3, "sbp"),
    (257, "richardson", 3, "normal"),
])
def test_vcycle_mixed_matches_fp64_oracle(sbp, n, smoother, nu, restriction):
    # The FP32 V-cycle (fused pre/post-smoothing kernels on every level, with
    # the interior-tile and boundary-tile paths) against the oracle's FP64
    # V-cycle: FP32 accuracy, relative 2e-5 in the 2-norm.
    from sc_2022_gb300 import _lib
    a, b, _ = ref_problem(n, "baseline")
    om = 2.0 / 3.0 if smoother == "jacobi" else 0.15
    hier = o.Hierarchy(n, o.MGOptions(smoother=smoother, omega=om, nu_pre=nu, nu_post=nu,
                                      restriction=restriction, coarse_n=65))
    z_ref = hier.vcycle(b)
    kinds = {"normal": _lib.SBP_RESTRICT_NORMAL, "sbp": _lib.SBP_RESTRICT_SBP,
             "galerkin": _lib.SBP_RESTRICT_GALERKIN}
    opts = sbp.default_options(_lib.SBP_PREC_MIXED)
    opts.smoother = _lib.SBP_SMOOTH_JACOBI if smoother == "jacobi" else _lib.SBP_SMOOTH_RICHARDSON
    opts.omega = om
    opts.nu_pre = opts.nu_post = nu
    opts.restriction = kinds[restriction]
    s = sbp.Solver(n, opts)
    z = torch.empty(n * n, dtype=torch.float64, device="cuda")
    s.vcycle(dev(b), z)
    assert relerr(host(z), z_ref) < 2e-5


def test_mgcg_large_discretisation_error(sbp):
    # N = 4097 and 2049: MGCG to 1e-10 and second-order H-error of the
    # manufactured solution (size-independent property of the full solve)
    from sc_2022_gb300 import problems
    errs = {}
    for n in (2049, 4097):
        f, g, U = problems.manufactured(n, "baseline")
        bd = problems.assemble_rhs(f, g)
        s = sbp.Solver(n, sbp.default_options())
        x = torch.zeros_like(bd)
        res = s.mgcg(bd, x, reltol=1e-10)
        assert res.converged and res.iters <= 10
        d = host(x) - U.ravel()
        h = 1.0 / (n - 1)
        w = np.ones(n)
        w[0] = w[-1] = 0.5
        W = (h * h) * np.outer(w, w).ravel()
        errs[n] = math.sqrt(float(d @ (W * d)))
        s.close()
    assert 3.8 < errs[2049] / errs[4097] < 4.2


def test_status_codes(sbp):
    from sc_2022_gb300 import _lib
    n = 129
    a, b, _ = ref_problem(n)
    s = sbp.Solver(n, sbp.default_options())
    x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    res = s.mgcg(dev(b), x, reltol=1e-14, maxiter=2)
    assert res.status == _lib.SBP_ERR_MAXITER and res.iters == 2
    bad = b.copy()
    bad[100] = np.nan
    x.zero_()
    res = s.mgcg(dev(bad), x, reltol=1e-10)
    assert res.status == _lib.SBP_ERR_BREAKDOWN
    x.zero_()
    res = s.mgcg(torch.zeros(n * n, dtype=torch.float64, device="cuda"), x, reltol=1e-10)
    assert res.converged and res.iters == 0
    with pytest.raises(sbp.SbpError):
        s.mgcg(dev(b), x, reltol=1e-14, maxiter=2, raise_on_fail=True)


def test_deterministic(sbp):
    n = 257
    a, b, _ = ref_problem(n, "baseline")
    s = sbp.Solver(n, sbp.default_options())
    runs = []
    for _ in range(2):
        x = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        res = s.mgcg(dev(b), x, reltol=1e-10)
        runs.append((res.norms, host(x)))
    assert runs[0][0] == runs[1][0]
    assert np.array_equal(runs[0][1], runs[1][1])


def test_mixed_n8193_bump_against_fp64(sbp):
    # N = 8193 (67M unknowns), random Gaussian-bump source and trig boundary
    # data: FP32 V-cycle inside FP64 PCG to 1e-10, against the FP64 MGCG solve
    # of the same problem (the FP64 path is itself held to the oracle at
    # smaller N).
    from sc_2022_gb300 import _lib, problems
    n = 8193
    f, g = problems.bump_problem(n, seed=3)
    b = problems.assemble_rhs(f, g).reshape(-1)
    del f
    xs, its = {}, {}
    for prec in (_lib.SBP_PREC_FP64, _lib.SBP_PREC_MIXED):
        s = sbp.Solver(n, sbp.default_options(prec))
        x = torch.zeros_like(b)
        res = s.mgcg(b, x, reltol=1e-10)
        assert res.converged
        xs[prec], its[prec] = x, res.iters
        s.close()
    assert its[_lib.SBP_PREC_MIXED] <= its[_lib.SBP_PREC_FP64] + 1
    import ctypes as C
    lib = sbp.load_library()
    out = C.c_double()
    x32 = xs[_lib.SBP_PREC_MIXED]
    assert lib.sbp_residual_norm_f64(C.c_void_p(x32.data_ptr()), C.c_void_p(b.data_ptr()), n, 1,
                                     C.byref(out), None) == 0
    assert out.value <= 2e-10 * b.norm().item()
    err = ((x32 - xs[_lib.SBP_PREC_FP64]).norm() / xs[_lib.SBP_PREC_FP64].norm()).item()
    # and against the C oracle's FP64 MGCG solve of the same b (67M unknowns)
    import os
    from oracle import cpu_path
    cpu_path.set_threads(os.cpu_count() or 1)
    bh = host(b)
    m = cpu_path.CpuMG(n, smoother="jacobi", restriction="galerkin", coarse_n=65)
    xo, it_o, _ = m.mgcg(bh, np.zeros_like(bh), 1e-10 * float(np.linalg.norm(bh)))
    m.close()
    err_o = relerr(host(x32), xo)
    err_o64 = relerr(host(xs[_lib.SBP_PREC_FP64]), xo)
    print(f"N=8193 mixed vs FP64: iterations {its} (oracle {it_o}), relative solution "
          f"difference {err:.3e}, mixed vs oracle {err_o:.3e}, FP64 vs oracle {err_o64:.3e}, "
          f"true relative residual {out.value / b.norm().item():.3e}")
    assert err < 1e-8
    assert its[_lib.SBP_PREC_FP64] == it_o
    assert err_o <= 1e-10 and err_o64 <= 1e-10


@pytest.mark.parametrize("n", [65, 257])
def test_nested_iteration_matches_oracle(sbp, n):
    rhs = {}
    for m in (n, (n + 1) // 2, (n + 3) // 4):
        a = o.assemble(m)
        F, g, U = o.manufactured(m, "reference")
        rhs[m] = a.rhs(F, g)
    b = rhs[n]
    abstol = float(np.linalg.norm(b)) * SQRT_EPS
    xr, itr, nr = o.nested_cg(n, b, rhs[(n + 1) // 2], abstol)
    x, it, norms = sbp.initial_guess_interpolation_CG_GPU(dev(b), dev(rhs[(n + 1) // 2]),
                                                         abstol=abstol)
    assert abs(it - itr) <= 1
    assert relerr(host(x), xr) < 1e-8
    assert norms[0] == pytest.approx(nr[0], rel=1e-10)
    x3r, it2r, it1r, _, _ = o.nested_cg_three_level(n, b, rhs[(n + 1) // 2], rhs[(n + 3) // 4],
                                                    abstol)
    x3, it2, it1, n2, n1 = sbp.initial_guess_interpolation_three_level_CG_GPU(
        dev(b), dev(rhs[(n + 1) // 2]), dev(rhs[(n + 3) // 4]), abstol=abstol)
    assert abs(it2 - it2r) <= 1 and abs(it1 - it1r) <= 1
    assert relerr(host(x3), x3r) < 1e-8
