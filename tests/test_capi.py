"""CPU tests of the C ABI: the library loads, exports every function that
include/sbpmg.h declares, argument checks reject bad input before touching
the GPU, and the host-side coarse inverse is exact."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import sbp_oracle as o

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "sbpmg.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(sbp_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from sc_2022_gb300 import _lib
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), f"libsbpmg.so does not export {name}"


def test_python_binding_covers_header():
    from sc_2022_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_options(lib):
    from sc_2022_gb300 import _lib
    o1 = _lib.sbp_options()
    lib.sbp_options_default(C.byref(o1))
    assert (o1.smoother, o1.nu_pre, o1.nu_post, o1.restriction, o1.coarse_n, o1.precision) == (
        _lib.SBP_SMOOTH_JACOBI, 3, 3, _lib.SBP_RESTRICT_GALERKIN, 65, _lib.SBP_PREC_FP64)
    assert abs(o1.omega - 2 / 3) < 1e-15
    o2 = _lib.sbp_options()
    lib.sbp_options_reference_two_level(C.byref(o2), 129)
    assert (o2.smoother, o2.restriction, o2.coarse_n) == (_lib.SBP_SMOOTH_RICHARDSON,
                                                          _lib.SBP_RESTRICT_NORMAL, 65)
    assert o2.omega == 0.15


def test_argument_errors_without_gpu(lib):
    from sc_2022_gb300 import _lib
    assert lib.sbp_apply_f64(None, None, 5, -1, None) == _lib.SBP_ERR_ARGS
    assert lib.sbp_apply_f64(C.c_void_p(8), C.c_void_p(8), 2, -1, None) == _lib.SBP_ERR_ARGS
    assert lib.sbp_apply_f64(C.c_void_p(8), C.c_void_p(8), 5, 3, None) == _lib.SBP_ERR_ARGS
    assert lib.sbp_restrict_f64(C.c_void_p(8), C.c_void_p(8), 8, 0, None) == _lib.SBP_ERR_ARGS
    assert lib.sbp_restrict_f64(C.c_void_p(8), C.c_void_p(8), 9, 7, None) == _lib.SBP_ERR_ARGS
    h = C.c_void_p()
    assert lib.sbp_solver_create(C.byref(h), 2, None) == _lib.SBP_ERR_ARGS
    assert lib.sbp_mgcg_solve(None, None, None, 0, 0, 1, None, None, 0, None) == _lib.SBP_ERR_ARGS
    assert lib.sbp_status_string(_lib.SBP_ERR_MAXITER) == b"maximum iterations reached"


@pytest.mark.parametrize("nc", [5, 17, 33])
def test_coarse_inverse_host(lib, nc):
    N = nc * nc
    X = np.zeros(N * N)
    rc = lib.sbp_coarse_inverse_host(nc, X.ctypes.data_as(C.POINTER(C.c_double)), N * N)
    assert rc == 0
    A = o.assemble(nc).A.toarray()
    X = X.reshape(N, N)
    assert np.abs(X - X.T).max() == 0.0
    assert np.abs(X @ A - np.eye(N)).max() < 1e-11


def test_coarse_inverse_rejects_bad_size(lib):
    X = np.zeros(10)
    assert lib.sbp_coarse_inverse_host(6, X.ctypes.data_as(C.POINTER(C.c_double)), 10) < 0
    assert lib.sbp_coarse_inverse_host(5, X.ctypes.data_as(C.POINTER(C.c_double)), 10) < 0


@pytest.mark.parametrize("n", [5, 17, 33])
def test_csr_assembly_equals_oracle_matrix(lib, n):
    # the comparator's CSR matrix is Assembling_matrix's A, bit for bit
    from sc_2022_gb300 import csr
    rp, col, val = csr.assemble_csr_host(n)
    A = o.assemble(n).A.tocsr()
    A.sort_indices()
    A.eliminate_zeros()
    assert np.array_equal(A.indptr, rp)
    assert np.array_equal(A.indices, col)
    assert np.array_equal(A.data, val)


@pytest.mark.parametrize("n,kind", [(3, "smooth"), (4, "layered"), (9, "smooth"), (17, "layered"),
                                    (33, "smooth")])
def test_variable_assembly_equals_oracle_matrix(n, kind):
    # the library's per-point variable-coefficient stencil, as CSR, against
    # the oracle's assembly of variable_diagonal_sbp_D2 per grid line
    import sc_2022_gb300 as sbp
    from oracle import sbp_oracle as o
    import scipy.sparse as sp
    c = o.coefficient_field(n, kind)
    rp, col, val = sbp.assemble_variable_host(n, c)
    A = sp.csr_matrix((val, col, rp), shape=(n * n, n * n))
    ref = o.assemble_variable(n, c).A
    assert abs(A - ref).max() <= 1e-13 * abs(ref).max()
    # c = 1: the constant-coefficient matrix
    rp1, col1, val1 = sbp.assemble_variable_host(n, np.ones(n * n))
    A1 = sp.csr_matrix((val1, col1, rp1), shape=(n * n, n * n))
    assert abs(A1 - o.assemble(n).A).max() == 0.0


def test_new_entry_points_reject_bad_arguments_without_gpu():
    # argument checks run before any CUDA call
    import sc_2022_gb300 as sbp
    from sc_2022_gb300 import _lib as L
    lib = sbp.load_library()
    h = C.c_void_p()
    assert lib.sbp_ho_solver_create(C.byref(h), 65, 3, None) == L.SBP_ERR_ARGS   # p = 3
    assert lib.sbp_ho_solver_create(C.byref(h), 7, 4, None) == L.SBP_ERR_ARGS    # n < 8
    assert lib.sbp_ho_solver_create(C.byref(h), 11, 6, None) == L.SBP_ERR_ARGS   # n < 12
    assert lib.sbp_ho_solver_create(None, 65, 4, None) == L.SBP_ERR_ARGS
    assert lib.sbp_apply_ho_f64(None, None, 65, 4, 1, None) == L.SBP_ERR_ARGS
    assert lib.sbp_apply_ho_f64(C.c_void_p(8), C.c_void_p(8), 65, 5, 1, None) == L.SBP_ERR_ARGS
    assert lib.sbp_apply_ho_f64(C.c_void_p(8), C.c_void_p(8), 65, 4, 0, None) == L.SBP_ERR_ARGS
    assert lib.sbp_vc_solver_create(C.byref(h), 65, None, None) == L.SBP_ERR_ARGS   # no c
    assert lib.sbp_vc_solver_create(C.byref(h), 2, C.c_void_p(8), None) == L.SBP_ERR_ARGS
    assert lib.sbp_apply_vc_f64(C.c_void_p(8), None, C.c_void_p(8), 65, 1, None) == L.SBP_ERR_ARGS
    assert lib.sbp_apply_vc_f64(C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), 2, 1,
                                None) == L.SBP_ERR_ARGS
    for f in (lib.sbp_ho_mgcg_solve, lib.sbp_vc_mgcg_solve):
        assert f(None, None, None, 0.0, 1e-8, 10, None, None, 0, None) == L.SBP_ERR_ARGS
    assert lib.sbp_ho_solver_destroy(None) == 0 and lib.sbp_vc_solver_destroy(None) == 0
    assert lib.sbp_ho_solver_levels(None) == L.SBP_ERR_ARGS
    # host CSR assembly: too small a capacity reports the needed count
    nnz = C.c_longlong()
    c = np.ones(9 * 9)
    rp = np.zeros(82, dtype=np.int64)
    assert lib.sbp_vc_assemble_host(9, c.ctypes.data_as(C.POINTER(C.c_double)),
                                    rp.ctypes.data_as(C.POINTER(C.c_longlong)), None, None, 0,
                                    C.byref(nnz)) == L.SBP_ERR_ARGS
    assert nnz.value > 81


@pytest.mark.parametrize("p,nc", [(2, 17), (4, 8), (4, 17), (4, 33), (6, 12), (6, 17), (6, 33)])
def test_order_p_coarse_inverse_equals_oracle(p, nc):
    # the order-p fast-diagonalisation factors (the order-p solver's coarse
    # solve) against the inverse of the oracle's assembled operator
    import sc_2022_gb300 as sbp
    lib = sbp.load_library()
    N = nc * nc
    out = np.zeros(N * N)
    assert lib.sbp_coarse_inverse_order_host(nc, p, out.ctypes.data_as(C.POINTER(C.c_double)),
                                             N * N) == 0
    A = o.assemble(nc, p).A.toarray()
    Ainv = out.reshape(N, N)
    assert np.abs(Ainv @ A - np.eye(N)).max() < 1e-9
    assert np.abs(Ainv - Ainv.T).max() == 0.0
    assert lib.sbp_coarse_inverse_order_host(7, 4, out.ctypes.data_as(C.POINTER(C.c_double)),
                                             N * N) != 0   # below the minimum grid


@pytest.mark.parametrize("n,kind", [(3, "smooth"), (9, "layered"), (33, "smooth"),
                                    (65, "layered"), (129, "random")])
def test_variable_coarse_coefficients_equal_oracle_bitwise(n, kind):
    # the coarse coefficients of the variable-coefficient multigrid (the
    # device kernel's arithmetic, run on the host) are the oracle's doubles
    import sc_2022_gb300 as sbp
    if kind == "random":
        c = np.exp(np.random.default_rng(5).uniform(-3.0, 3.0, n * n))
    else:
        c = o.coefficient_field(n, kind)
    got = sbp.coarsen_coefficients_host(c)
    ref = o.coarsen_coefficients(c.reshape(n, n))
    assert got.shape == ref.shape
    np.testing.assert_array_equal(got, ref)


def _nine_point_matrix(st):
    """The symmetric matrix of a stored 9-point level (arrays [j, i])."""
    import scipy.sparse as sps
    m = st["D"].shape[0]
    rows, cols, vals = [], [], []
    for j in range(m):
        for i in range(m):
            k = j * m + i
            rows.append(k); cols.append(k); vals.append(st["D"][j, i])
            for key, di, dj in (("E", 1, 0), ("N", 0, 1), ("NE", 1, 1), ("NW", -1, 1)):
                ii, jj = i + di, j + dj
                if 0 <= ii < m and 0 <= jj < m:
                    q = jj * m + ii
                    rows += [k, q]; cols += [q, k]; vals += [-st[key][j, i]] * 2
                else:
                    assert st[key][j, i] == 0.0
    return sps.csr_matrix((vals, (rows, cols)), shape=(m * m, m * m))


@pytest.mark.parametrize("n,kind", [(3, "smooth"), (9, "layered"), (17, "smooth"),
                                    (33, "layered")])
def test_galerkin_coarse_operators_equal_oracle(n, kind):
    # P' A P of the variable-coefficient operator, level after level, built
    # by the library's set-up arithmetic, against the oracle's sparse products
    import sc_2022_gb300 as sbp
    c = o.coefficient_field(n, kind)
    levels = max(1, int(np.log2(n - 1)) - 1)
    got = sbp.galerkin_coarse_host(c, levels=levels)
    A = o.assemble_variable(n, c).A
    m = n
    for st in got:
        m = (m + 1) // 2
        P = o.prolongation_2d(m)
        A = (P.T @ A @ P).tocsr()
        B = _nine_point_matrix(st)
        scale = abs(A).max()
        assert abs(B - A).max() <= 1e-14 * scale


def test_variable_coarse_coefficients_arguments():
    import sc_2022_gb300 as sbp
    lib = sbp.load_library()
    dp = C.POINTER(C.c_double)
    buf = np.ones(9)
    assert lib.sbp_vc_coarsen_host(0, buf.ctypes.data_as(dp), buf.ctypes.data_as(dp)) < 0
    assert lib.sbp_vc_coarsen_host(2, None, buf.ctypes.data_as(dp)) < 0
    with pytest.raises(ValueError):
        sbp.coarsen_coefficients_host(np.ones(16))
    five = [buf.ctypes.data_as(dp)] * 5
    assert lib.sbp_vc_galerkin_coarse_host(4, buf.ctypes.data_as(dp), *five) < 0
    assert lib.sbp_galerkin9_coarse_host(1, *[buf.ctypes.data_as(dp)] * 10) < 0
    with pytest.raises(ValueError):
        sbp.galerkin_coarse_host(np.ones(16))


@pytest.mark.parametrize("nc,kind", [(5, "smooth"), (9, "layered"), (17, "smooth")])
def test_variable_coarse_inverse_equals_oracle(nc, kind):
    # the dense coarse inverse of the variable-coefficient solver (host
    # Cholesky) against the inverse of the oracle's assembled operator
    import sc_2022_gb300 as sbp
    lib = sbp.load_library()
    c = np.ascontiguousarray(o.coefficient_field(nc, kind))
    N = nc * nc
    out = np.zeros(N * N)
    dp = C.POINTER(C.c_double)
    assert lib.sbp_vc_coarse_inverse_host(nc, c.ctypes.data_as(dp), out.ctypes.data_as(dp),
                                          N * N) == 0
    A = o.assemble_variable(nc, c).A.toarray()
    assert np.abs(out.reshape(N, N) @ A - np.eye(N)).max() < 1e-10
