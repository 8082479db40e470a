"""GPU parity of the single-grid operators (through the C ABI) against the
CPU oracle and the golden fixtures."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import sbp_oracle as o

pytestmark = pytest.mark.gpu

APPLY_RTOL = 1e-13   # FP64 operator apply, relative 2-norm


def dev(a, dtype=torch.float64):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda").contiguous()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().ravel().astype(np.float64)


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("n", [3, 5, 9, 17, 33])
def test_apply_golden(sbp, golden, n):
    u = dev(golden[f"apply_u_{n}"])
    out = torch.empty_like(u)
    sbp.matrix_free_A_full_GPU(u, out)
    assert relerr(host(out), golden[f"apply_negAu_{n}"]) < APPLY_RTOL


@pytest.mark.parametrize("n", [65, 129, 257, 513, 1025])
def test_apply_vs_assembled(sbp, n):
    rng = np.random.default_rng(n)
    u = rng.standard_normal(n * n)
    A = o.assemble(n).A
    ud = dev(u)
    out = torch.empty_like(ud)
    lib = sbp.load_library()
    for sign in (-1, 1):
        rc = lib.sbp_apply_f64(C.c_void_p(ud.data_ptr()), C.c_void_p(out.data_ptr()), n, sign,
                               None)
        assert rc == 0
        assert relerr(host(out), sign * (A @ u)) < APPLY_RTOL


def test_apply_large_linearity(sbp):
    # size-independent property at the benchmark size: A(a u + b v) = a Au + b Av
    n = 4097
    g = torch.Generator(device="cuda").manual_seed(1)
    u = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    v = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    au, av, aw = (torch.empty_like(u) for _ in range(3))
    sbp.matrix_free_A_full_GPU(u, au)
    sbp.matrix_free_A_full_GPU(v, av)
    sbp.matrix_free_A_full_GPU(2.0 * u - 3.0 * v, aw)
    torch.cuda.synchronize()
    d = (aw - (2.0 * au - 3.0 * av)).norm() / aw.norm()
    assert d.item() < 1e-14
    # symmetry u.Av == v.Au
    s1 = torch.dot(u, av).item()
    s2 = torch.dot(v, au).item()
    assert abs(s1 - s2) <= 1e-12 * (abs(s1) + 1e-300) * 100


@pytest.mark.parametrize("n", [9, 65, 1025])
def test_apply_f32(sbp, n):
    rng = np.random.default_rng(7)
    u = rng.standard_normal(n * n).astype(np.float32)
    A = o.assemble(n).A
    ud = dev(u, torch.float32)
    out = torch.empty_like(ud)
    sbp.matrix_free_A_full_GPU_f32(ud, out)
    ref = -(A @ u.astype(np.float64))
    assert relerr(host(out), ref) < 1e-6


@pytest.mark.parametrize("n", [5, 33, 257])
def test_apply_dot(sbp, n):
    rng = np.random.default_rng(3)
    u = rng.standard_normal(n * n)
    A = o.assemble(n).A
    ud = dev(u)
    out = torch.empty_like(ud)
    dot = torch.zeros(1, dtype=torch.float64, device="cuda")
    lib = sbp.load_library()
    rc = lib.sbp_apply_dot_f64(C.c_void_p(ud.data_ptr()), C.c_void_p(out.data_ptr()), n, 1,
                               C.c_void_p(dot.data_ptr()), None)
    assert rc == 0
    ref = u @ (A @ u)
    assert abs(host(dot)[0] - ref) <= 1e-12 * abs(ref)
    assert relerr(host(out), A @ u) < APPLY_RTOL


@pytest.mark.parametrize("n", [5, 9, 17, 33])
def test_restrict_golden(sbp, golden, n):
    lib = sbp.load_library()
    r = dev(golden[f"restrict_in_{n}"])
    nc = (n + 1) // 2
    f = torch.empty(nc * nc, dtype=torch.float64, device="cuda")
    for k, kind in enumerate(o.RESTRICT_KINDS):
        assert lib.sbp_restrict_f64(C.c_void_p(r.data_ptr()), C.c_void_p(f.data_ptr()), n, k,
                                    None) == 0
        np.testing.assert_allclose(host(f), golden[f"restrict_{kind}_{n}"], rtol=0, atol=1e-14)
    # the reference's entry point (NORMAL)
    sbp.matrix_free_restriction_2d_GPU(r, f)
    np.testing.assert_allclose(host(f), golden[f"restrict_normal_{n}"], rtol=0, atol=1e-14)


@pytest.mark.parametrize("nc", [3, 5, 9, 17])
def test_prolong_golden(sbp, golden, nc):
    e = dev(golden[f"prolong_in_{nc}"])
    nf = 2 * nc - 1
    out = torch.full((nf * nf,), float("nan"), dtype=torch.float64, device="cuda")
    sbp.matrix_free_prolongation_2d_GPU(e, out)
    np.testing.assert_allclose(host(out), golden[f"prolong_{nc}"], rtol=0, atol=1e-15)
    base = torch.ones_like(out)
    sbp.matrix_free_prolongation_2d_GPU(e, base, accumulate=True)
    np.testing.assert_allclose(host(base), golden[f"prolong_{nc}"] + 1.0, rtol=0, atol=1e-14)


@pytest.mark.parametrize("n", [1025, 4097])
def test_restrict_prolong_adjoint_large(sbp, n):
    # <P e, r> == <e, P^T r> with P^T = GALERKIN restriction, at full size
    lib = sbp.load_library()
    nc = (n + 1) // 2
    g = torch.Generator(device="cuda").manual_seed(5)
    r = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    e = torch.randn(nc * nc, generator=g, device="cuda", dtype=torch.float64)
    pe = torch.empty_like(r)
    rt = torch.empty_like(e)
    sbp.matrix_free_prolongation_2d_GPU(e, pe)
    assert lib.sbp_restrict_f64(C.c_void_p(r.data_ptr()), C.c_void_p(rt.data_ptr()), n, 2,
                                None) == 0
    torch.cuda.synchronize()
    a, b = torch.dot(pe, r).item(), torch.dot(e, rt).item()
    assert abs(a - b) <= 1e-11 * (abs(a) + abs(b))


@pytest.mark.parametrize("smoother", ["richardson", "jacobi"])
def test_smoothers(sbp, smoother):
    n = 33
    a = o.assemble(n)
    rng = np.random.default_rng(11)
    v0 = rng.standard_normal(n * n)
    b = rng.standard_normal(n * n)
    vd, td, bd = dev(v0), torch.empty(n * n, dtype=torch.float64, device="cuda"), dev(b)
    if smoother == "richardson":
        sbp.matrix_free_richardson(vd, td, bd, maxiter=3, omega=0.15)
        ref = o.richardson(v0, a.A, b, 3, 0.15)
    else:
        sbp.jacobi(vd, td, bd, maxiter=4, omega=2 / 3)
        ref = o.jacobi(v0, a.A, b, 4, 2 / 3)
    assert relerr(host(vd), ref) < 1e-13
    assert relerr(host(td), ref) < 1e-13


@pytest.mark.parametrize("n", [9, 17, 33])
def test_rhs_golden(sbp, golden, n):
    from sc_2022_gb300 import problems
    g = {k: golden[f"rhs_g{k}_{n}"] for k in "WESN"}
    b = problems.assemble_rhs(golden[f"rhs_f_{n}"], g)
    np.testing.assert_allclose(host(b), golden[f"rhs_b_{n}"], rtol=0, atol=1e-13)


def test_rhs_adjoint_dot_identity(sbp):
    from sc_2022_gb300 import problems
    n = 257
    rng = np.random.default_rng(2)
    f = rng.standard_normal(n * n)
    g = {k: rng.standard_normal(n) for k in "WESN"}
    lam = dev(rng.standard_normal(n * n))
    b = problems.assemble_rhs(f, g)
    df, dg = problems.rhs_adjoint(lam)
    lhs = torch.dot(lam.ravel(), b.ravel()).item()
    rhs = float(host(df) @ f) + sum(float(host(dg[k]) @ g[k]) for k in "WESN")
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + 1.0)


def test_residual_norm(sbp):
    n = 65
    a = o.assemble(n)
    rng = np.random.default_rng(4)
    x, b = rng.standard_normal(n * n), rng.standard_normal(n * n)
    lib = sbp.load_library()
    out = C.c_double()
    xd, bd = dev(x), dev(b)
    assert lib.sbp_residual_norm_f64(C.c_void_p(xd.data_ptr()), C.c_void_p(bd.data_ptr()), n, 1,
                                     C.byref(out), None) == 0
    ref = np.linalg.norm(b - a.A @ x)
    assert abs(out.value - ref) <= 1e-12 * ref


@pytest.mark.parametrize("field", ["wide", "smooth"])
def test_apply_f64_exact_integer_path(sbp, field):
    # Interior points of the FP64 apply on the caller's layout are summed
    # either on the integer pipe (odd warps: rows with (i mod 256) // 32 odd)
    # or with FP64 instructions (even warps).  Against the exact rational value of
    # (w + e + m + p) - 4c: the integer path is within 1 ulp of the result
    # plus 0.05 ulp of the largest term, the FP64 path within 3 ulp of it.
    import math
    from fractions import Fraction
    n = 257
    rng = np.random.default_rng(17)
    if field == "wide":
        u = rng.standard_normal(n * n) * 10.0 ** rng.uniform(-5, 5, n * n)
    else:
        x = np.linspace(0, 1, n)
        u = (np.sin(3 * x)[None, :] * np.cos(2 * x)[:, None]).ravel() + 1e-3 * rng.random(n * n)
    U = u.reshape(n, n)                      # U[j, i]
    out = torch.empty(n * n, dtype=torch.float64, device="cuda")
    lib = sbp.load_library()
    assert lib.sbp_apply_f64(C.c_void_p(dev(u).data_ptr()), C.c_void_p(out.data_ptr()), n, -1,
                             None) == 0
    got = host(out).reshape(n, n)
    checked = {0: 0, 1: 0}
    for _ in range(3000):
        i = int(rng.integers(1, n - 1))
        j = int(rng.integers(3, n - 3))
        c, w, e, m, p = U[j, i], U[j, i - 1], U[j, i + 1], U[j - 1, i], U[j + 1, i]
        exact = (Fraction(w) + Fraction(e) + Fraction(m) + Fraction(p)) - 4 * Fraction(c)
        ref = float(exact)
        big = max(abs(4 * c), abs(w), abs(e), abs(m), abs(p))
        err = abs(float(Fraction(got[j, i]) - exact))
        integer_path = ((i % 256) // 32) % 2 == 1
        if integer_path:
            assert err <= math.ulp(ref) + 0.05 * math.ulp(big), (i, j, err)
        else:
            assert err <= 3 * math.ulp(big), (i, j, err)
        checked[int(integer_path)] += 1
    assert checked[0] > 100 and checked[1] > 100


@pytest.mark.parametrize("n", [257, 1025])
def test_csr_spmv_matches_matrix_free(sbp, n):
    from sc_2022_gb300 import csr
    A = csr.CsrOperator(n)
    rng = np.random.default_rng(23)
    x = rng.standard_normal(n * n)
    xd = dev(x)
    y = A.matvec(xd)
    mf = torch.empty_like(xd)
    lib = sbp.load_library()
    assert lib.sbp_apply_f64(C.c_void_p(xd.data_ptr()), C.c_void_p(mf.data_ptr()), n, 1,
                             None) == 0
    rel = np.linalg.norm(host(y) - host(mf)) / np.linalg.norm(host(mf))
    assert rel < 1e-14
    if n == 257:
        ref = o.assemble(n).A @ x
        assert np.linalg.norm(host(y) - ref) / np.linalg.norm(ref) < 1e-14


@pytest.mark.parametrize("n", [2049, 4097])
def test_apply_large_vs_oracle(sbp, n):
    # The caller-layout applies at the benchmark sizes (many column runs and
    # row blocks per launch, the last row block holding one row), FP64 and
    # FP32, both signs, and the fused dot, against the oracle's matrix-free
    # restatement of matrix_free_A_full_GPU (split_matrix_free.jl:444-486).
    rng = np.random.default_rng(n)
    u = rng.standard_normal(n * n)
    ref = o.neg_A_matrix_free(u, n).ravel()
    lib = sbp.load_library()
    ud = dev(u)
    out = torch.empty_like(ud)
    for sign in (-1, 1):
        assert lib.sbp_apply_f64(C.c_void_p(ud.data_ptr()), C.c_void_p(out.data_ptr()), n, sign,
                                 None) == 0
        assert relerr(host(out), -sign * ref) < APPLY_RTOL
    u32 = u.astype(np.float32)
    ref32 = o.neg_A_matrix_free(u32.astype(np.float64), n).ravel()
    ud32 = dev(u32, torch.float32)
    out32 = torch.empty_like(ud32)
    assert lib.sbp_apply_f32(C.c_void_p(ud32.data_ptr()), C.c_void_p(out32.data_ptr()), n, -1,
                             None) == 0
    assert relerr(host(out32), ref32) < 1e-6
    dot = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.sbp_apply_dot_f64(C.c_void_p(ud.data_ptr()), C.c_void_p(out.data_ptr()), n, 1,
                                 C.c_void_p(dot.data_ptr()), None) == 0
    want = -float(u @ ref)
    assert abs(host(dot)[0] - want) <= 1e-11 * abs(want)


@pytest.mark.parametrize("n", [65, 1025])
def test_apply_unaligned_arrays(sbp, n):
    # arrays that start 8 (FP64) or 4 (FP32) bytes into a buffer: an offset
    # view is as valid a caller array as a fresh allocation
    rng = np.random.default_rng(5)
    u = rng.standard_normal(n * n)
    ref = o.neg_A_matrix_free(u, n).ravel()
    lib = sbp.load_library()
    buf = torch.zeros(n * n + 1, dtype=torch.float64, device="cuda")
    buf[1:] = dev(u)
    outb = torch.zeros(n * n + 1, dtype=torch.float64, device="cuda")
    assert lib.sbp_apply_f64(C.c_void_p(buf[1:].data_ptr()), C.c_void_p(outb[1:].data_ptr()), n,
                             -1, None) == 0
    assert relerr(host(outb[1:]), ref) < APPLY_RTOL
    assert host(outb)[0] == 0.0
    buf32 = torch.zeros(n * n + 1, dtype=torch.float32, device="cuda")
    buf32[1:] = dev(u.astype(np.float32), torch.float32)
    out32 = torch.zeros(n * n + 1, dtype=torch.float32, device="cuda")
    assert lib.sbp_apply_f32(C.c_void_p(buf32[1:].data_ptr()), C.c_void_p(out32[1:].data_ptr()),
                             n, -1, None) == 0
    ref32 = o.neg_A_matrix_free(u.astype(np.float32).astype(np.float64), n).ravel()
    assert relerr(host(out32[1:]), ref32) < 1e-6


def test_pair_to_f64_matches_fp64_add(sbp):
    # the direction pass forms -(hi + lo) of its float-float stencil without
    # FP64 arithmetic: the bits must be those of the FP64 add, over random bit
    # patterns, cancelling pairs and every exponent gap
    rng = np.random.default_rng(11)
    n = 1 << 22
    hi = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    lo = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    m = n // 4
    # cancellation: lo = -hi (1 + k 2^-23)
    k = rng.integers(-2048, 2048, m).astype(np.float32)
    lo[:m] = -hi[:m] * (np.float32(1) + k * np.float32(2.0 ** -23))
    # exponent gaps 0 .. 70 with both signs
    gap = rng.integers(0, 71, m)
    lo[m:2 * m] = (hi[m:2 * m].astype(np.float64) * np.ldexp(1.0, -gap)
                   * rng.choice([-1.0, 1.0], m) * rng.uniform(0.5, 2.0, m)).astype(np.float32)
    lo[2 * m + 5] = 0.0
    hi[2 * m + 6], lo[2 * m + 6] = 0.0, 0.0
    ok = np.isfinite(hi) & np.isfinite(lo)
    hi, lo = hi[ok], lo[ok]
    with np.errstate(all="ignore"):
        ref = -(hi.astype(np.float64) + lo.astype(np.float64))
    dh, dl = dev(hi, torch.float32), dev(lo, torch.float32)
    out = torch.empty(hi.size, dtype=torch.float64, device="cuda")
    lib = sbp.load_library()
    assert lib.sbp_test_pair_to_f64(C.c_void_p(dh.data_ptr()), C.c_void_p(dl.data_ptr()),
                                    C.c_void_p(out.data_ptr()), hi.size, None) == 0
    got = out.cpu().numpy()
    # the hardware add flushes float denormal inputs like the integer path
    # does not need to: compare where neither operand is a denormal
    normal = ((np.abs(hi) >= np.finfo(np.float32).tiny) | (hi == 0)) & \
             ((np.abs(lo) >= np.finfo(np.float32).tiny) | (lo == 0))
    assert normal.mean() > 0.95
    bad = np.flatnonzero(got[normal].view(np.uint64) != ref[normal].view(np.uint64))
    assert bad.size == 0, (hi[normal][bad[:4]], lo[normal][bad[:4]])


@pytest.mark.parametrize("n,offset", [(66, 0), (67, 1), (100, 1), (1025, 0), (1025, 1)])
def test_apply_f32_interior_bits(sbp, n, offset):
    # the FP32 apply's plain interior (rows 1..n-2, columns 3..n-4) is
    # fma(+-4, u0, -+((u_i-1 + u_i+1) + (u_j-1 + u_j+1))) in FP32: bit for bit
    # against the same operations emulated in numpy (4 u0 - s is exact in
    # FP64, so one rounding to FP32 is the FMA); the SAT boundary against the
    # oracle.  Odd and even n - 1 and arrays starting 4 bytes into a buffer.
    rng = np.random.default_rng(n + offset)
    u = rng.standard_normal((n, n)).astype(np.float32)   # [j, i]: column-major
    lib = sbp.load_library()
    buf = torch.zeros(n * n + offset, dtype=torch.float32, device="cuda")
    buf[offset:] = dev(u.ravel(), torch.float32)
    out = torch.full((n * n + offset,), np.nan, dtype=torch.float32, device="cuda")
    for sign in (-1, 1):
        assert lib.sbp_apply_f32(C.c_void_p(buf[offset:].data_ptr()),
                                 C.c_void_p(out[offset:].data_ptr()), n, sign, None) == 0
        got = out[offset:].cpu().numpy().reshape(n, n)
        c0 = u[3:n - 3, 1:n - 1]
        s = (u[3:n - 3, 0:n - 2] + u[3:n - 3, 2:n]) + (u[2:n - 4, 1:n - 1] + u[4:n - 2, 1:n - 1])
        if sign > 0:
            want = (4.0 * c0.astype(np.float64) - s.astype(np.float64)).astype(np.float32)
        else:
            want = (s.astype(np.float64) - 4.0 * c0.astype(np.float64)).astype(np.float32)
        assert np.array_equal(got[3:n - 3, 1:n - 1].view(np.uint32), want.view(np.uint32))
        ref = -sign * o.neg_A_matrix_free(u.ravel().astype(np.float64), n).reshape(n, n)
        assert np.isfinite(got).all()
        assert relerr(got.ravel().astype(np.float64), ref.ravel()) < 1e-6
