"""The headline sizes held to the C oracle: FP64 and mixed-precision MGCG at
N = 4097 and plain CG at N = 1025 against the C restatement of the
reference's CPU sparse path (oracle/sbp_cpu.c) solving the same problem, the
reference's CG at N = 4097 by its true residual, and the per-kernel profile
of a solve against the graph-launched solve."""
import os

import numpy as np
import pytest
import torch

from oracle import cpu_path

pytestmark = pytest.mark.gpu


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().ravel()


def relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def true_rel_residual(sbp, x, b, n, sign=1):
    import ctypes as C
    out = C.c_double()
    assert sbp.load_library().sbp_residual_norm_f64(C.c_void_p(x.data_ptr()),
                                                    C.c_void_p(b.data_ptr()), n, sign,
                                                    C.byref(out), None) == 0
    return out.value / b.norm().item()


@pytest.fixture(scope="module")
def threads():
    t = os.cpu_count() or 1
    cpu_path.set_threads(t)
    return t


def test_mgcg_n4097_pinned_to_c_oracle(sbp, threads):
    # matrix_free_MGCG (matrix_free_mg_cg.jl:281-324) with the benchmark
    # V-cycle at N = 4097, manufactured problem, tolerance 1e-10: the GPU FP64
    # and mixed solutions against the oracle's FP64 solve of the same b
    # (mg_preconditioned_CG, level_2_multigrid_new.jl:480-524)
    from sc_2022_gb300 import _lib, problems
    n = 4097
    f, g, _ = problems.manufactured(n, "baseline")
    b = problems.assemble_rhs(f, g).reshape(-1)
    bh = host(b)
    m = cpu_path.CpuMG(n, smoother="jacobi", restriction="galerkin", coarse_n=65)
    xo, it_o, _ = m.mgcg(bh, np.zeros_like(bh), 1e-10 * float(np.linalg.norm(bh)))
    m.close()
    for prec in (_lib.SBP_PREC_FP64, _lib.SBP_PREC_MIXED):
        s = sbp.Solver(n, sbp.default_options(prec))
        x = torch.zeros_like(b)
        res = s.mgcg(b, x, reltol=1e-10)
        assert res.converged
        err = relerr(host(x), xo)
        print(f"N=4097 precision {prec}: iterations {res.iters} (oracle {it_o}), "
              f"solution vs oracle {err:.3e}")
        if prec == _lib.SBP_PREC_FP64:
            assert res.iters == it_o
        else:
            assert abs(res.iters - it_o) <= 1
        assert err <= 1e-10
        s.close()


def test_cg_n1025_matches_c_oracle(sbp, threads):
    # CG_CPU (level_2_multigrid_new.jl:258-291) on A x = b to 1e-10 relative
    # residual at N = 1025 (about 2500 iterations): iterations within one,
    # solution within 1e-10
    from sc_2022_gb300 import problems
    n = 1025
    f, g, _ = problems.manufactured(n, "baseline")
    b = problems.assemble_rhs(f, g).reshape(-1)
    bh = host(b)
    abstol = 1e-10 * float(np.linalg.norm(bh))
    m = cpu_path.CpuMG(n, plain=True)
    xo, it_o, no = m.cg(bh, np.zeros_like(bh), abstol)
    m.close()
    s = sbp.Solver(n)
    x = torch.zeros_like(b)
    res = s.cg(b, x, sign=1, abstol=abstol, maxiter=20000)
    assert res.converged
    err = relerr(host(x), xo)
    print(f"N=1025 CG: iterations {res.iters} (oracle {it_o}), solution vs oracle {err:.3e}")
    assert abs(res.iters - it_o) <= 1
    assert err <= 1e-10
    assert res.norms[0] == pytest.approx(no[0], rel=1e-12)


def test_cg_n4097_true_residual(sbp):
    # the plain matrix-free CG of the reference's comparison at level 12
    # (CG_comparison/cg_comparison.jl:99-122) at N = 4097 to 1e-10: the true
    # residual of the returned x (the recurrence residual drifts from it by
    # rounding over ~10^4 iterations)
    from sc_2022_gb300 import problems
    n = 4097
    f, g, _ = problems.manufactured(n, "baseline")
    b = problems.assemble_rhs(f, g).reshape(-1)
    s = sbp.Solver(n)
    x = torch.zeros_like(b)
    res = s.cg(b, x, sign=1, reltol=1e-10, maxiter=100000)
    assert res.converged
    rel = true_rel_residual(sbp, x, b, n)
    print(f"N=4097 CG: {res.iters} iterations, true relative residual {rel:.3e}")
    assert rel <= 2e-10
    s.close()


@pytest.mark.parametrize("n", [513, 1025])
def test_profile_matches_graph_solve(sbp, n):
    # sbp_solver_profile launches the same kernels without graphs: the same
    # iterations and, with fixed-order reductions, the same solution bit for
    # bit; every kernel of the solve appears with its launches.  At N = 1025
    # the mixed direction pass is the one-launch register wave (interior
    # strips and SAT boundary CTAs meeting in one reduction), and the
    # smoothing waves run beside their staged boundary rings.
    from sc_2022_gb300 import _lib, problems
    f, g, _ = problems.manufactured(n, "baseline")
    b = problems.assemble_rhs(f, g).reshape(-1)
    for prec in (_lib.SBP_PREC_FP64, _lib.SBP_PREC_MIXED):
        s = sbp.Solver(n, sbp.default_options(prec))
        x = torch.zeros_like(b)
        res = s.mgcg(b, x, reltol=1e-10)
        xp = torch.zeros_like(b)
        rp, rows = s.profile(b, xp, kind="mgcg", reltol=1e-10)
        assert rp.iters == res.iters and rp.converged
        assert torch.equal(x, xp)
        assert rows and all(r["launches"] > 0 and r["total_ms"] > 0 for r in rows)
        assert [r["total_ms"] for r in rows] == sorted((r["total_ms"] for r in rows),
                                                       reverse=True)
        launches = sum(r["launches"] for r in rows)
        assert launches >= res.iters * 3
        if prec == _lib.SBP_PREC_MIXED and n == 1025:
            names = " ".join(r["kernel"] for r in rows)
            assert "k_dir_wave" in names and "CgDirF32Job" not in names
            assert "k_pre_wave" in names and "k_post_wave" in names
        s.close()


def test_fp64_fma_rate(sbp):
    import ctypes as C
    g = C.c_double()
    assert sbp.load_library().sbp_fp64_fma_rate(C.byref(g), None) == 0
    # GB300: about two FP64 lanes per clock per SM, 152 SMs at up to 2.07 GHz
    assert 50.0 < g.value < 5000.0


@pytest.mark.parametrize("n", [2049, 4097])
def test_vcycle_large_levels_match_c_oracle(sbp, threads, n):
    # One V-cycle of the benchmark hierarchy (matrix_free_Two_level_multigrid
    # generalised to 7 levels, matrix_free_mg_cg.jl:143-176) at the sizes
    # whose fine levels run the register-wave pre-smoothing in the mixed
    # form: FP64 against the C oracle's V-cycle to 1e-12, mixed to 2e-5
    from sc_2022_gb300 import _lib
    rng = np.random.default_rng(n)
    b = rng.standard_normal(n * n)
    m = cpu_path.CpuMG(n, smoother="jacobi", restriction="galerkin", coarse_n=65)
    zo = m.vcycle(b)
    m.close()
    bd = torch.tensor(b, dtype=torch.float64, device="cuda")
    for prec, tol in ((_lib.SBP_PREC_FP64, 1e-12), (_lib.SBP_PREC_MIXED, 2e-5)):
        s = sbp.Solver(n, sbp.default_options(prec))
        z = torch.empty_like(bd)
        s.vcycle(bd, z)
        err = relerr(host(z), zo)
        print(f"N={n} V-cycle precision {prec}: vs C oracle {err:.3e}")
        assert err <= tol
        s.close()
