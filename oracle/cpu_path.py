"""ctypes wrapper of oracle/libsbp_cpu.so (the C restatement of the
reference's CPU sparse MGCG/CG path).  TEST INFRASTRUCTURE ONLY: used by
tests/ and by bench.py's CPU baseline legs.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle

_lib = None


class cpu_opts(C.Structure):
    _fields_ = [("smoother", C.c_int), ("omega", C.c_double), ("nu_pre", C.c_int),
                ("nu_post", C.c_int), ("restriction", C.c_int), ("coarse_n", C.c_int)]


def load():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        lib = C.CDLL(str(path))
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        lib.cpu_mg_create.restype = vp
        lib.cpu_mg_create.argtypes = [C.c_int, C.POINTER(cpu_opts)]
        lib.cpu_mg_destroy.argtypes = [vp]
        lib.cpu_mgcg.restype = C.c_int
        lib.cpu_mgcg.argtypes = [vp, dp, dp, C.c_double, C.c_int, dp]
        lib.cpu_cg.restype = C.c_int
        lib.cpu_cg.argtypes = [vp, dp, dp, C.c_double, C.c_int, dp]
        lib.cpu_apply.argtypes = [vp, dp, dp]
        lib.cpu_vcycle.argtypes = [vp, dp, dp]
        lib.cpu_nnz.restype = C.c_int
        lib.cpu_nnz.argtypes = [vp, C.c_int]
        lib.cpu_export_A.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), dp]
        lib.cpu_set_threads.argtypes = [C.c_int]
        lib.cpu_max_threads.restype = C.c_int
        _lib = lib
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class CpuMG:
    """Hierarchy + CG workspace of the C restatement."""

    def __init__(self, n: int, smoother="jacobi", omega=None, nu_pre=3, nu_post=3,
                 restriction="galerkin", coarse_n=65, plain=False):
        lib = load()
        self.n = n
        kinds = {"normal": 0, "sbp": 1, "galerkin": 2}
        if plain:
            self.h = lib.cpu_mg_create(n, None)
        else:
            o = cpu_opts(0 if smoother == "jacobi" else 1,
                         omega if omega is not None else (2 / 3 if smoother == "jacobi" else 0.15),
                         nu_pre, nu_post, kinds[restriction], coarse_n)
            self.h = lib.cpu_mg_create(n, C.byref(o))
        if not self.h:
            raise RuntimeError("cpu_mg_create failed")
        self.lib = lib

    def close(self):
        if self.h:
            self.lib.cpu_mg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def mgcg(self, b, x, abstol, maxiter=None):
        b = np.ascontiguousarray(b, dtype=np.float64).ravel()
        x = np.ascontiguousarray(x, dtype=np.float64).ravel().copy()
        maxiter = b.size if maxiter is None else maxiter
        norms = np.zeros(maxiter + 1)
        it = self.lib.cpu_mgcg(self.h, _dp(b), _dp(x), abstol, maxiter, _dp(norms))
        return x, it, norms[:it + 1]

    def cg(self, b, x, abstol, maxiter=None):
        b = np.ascontiguousarray(b, dtype=np.float64).ravel()
        x = np.ascontiguousarray(x, dtype=np.float64).ravel().copy()
        maxiter = b.size if maxiter is None else maxiter
        norms = np.zeros(maxiter + 1)
        it = self.lib.cpu_cg(self.h, _dp(b), _dp(x), abstol, maxiter, _dp(norms))
        return x, it, norms[:it + 1]

    def apply(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        out = np.empty_like(u)
        self.lib.cpu_apply(self.h, _dp(u), _dp(out))
        return out

    def vcycle(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64).ravel()
        out = np.empty_like(b)
        self.lib.cpu_vcycle(self.h, _dp(b), _dp(out))
        return out

    def csr(self, level=0):
        import scipy.sparse as sp
        nnz = self.lib.cpu_nnz(self.h, level)
        m = self.n
        for _ in range(level):
            m = (m + 1) // 2
        N = m * m
        rp = np.zeros(N + 1, dtype=np.int32)
        ci = np.zeros(nnz, dtype=np.int32)
        v = np.zeros(nnz)
        self.lib.cpu_export_A(self.h, level, rp.ctypes.data_as(C.POINTER(C.c_int)),
                              ci.ctypes.data_as(C.POINTER(C.c_int)), _dp(v))
        return sp.csr_matrix((v, ci, rp), shape=(N, N))


def set_threads(t: int):
    load().cpu_set_threads(t)


def max_threads() -> int:
    return load().cpu_max_threads()
