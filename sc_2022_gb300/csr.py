"""The assembled-operator comparator: A (``Assembling_matrix``) as a device
CSR matrix with this project's SpMV kernel, for the reference's
matrix-free vs SpMV comparison (``Poisson_CG.jl:217, 244-271``,
``kernel_comparisons/SPMV_test.jl``)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .solver import _stream_ptr, ptr


def assemble_csr_host(n: int):
    """(row_ptr int64, col int32, val float64) numpy arrays of A on n x n points."""
    lib = L.load()
    nnz = C.c_longlong()
    L.check(lib.sbp_csr_assemble_host(n, None, None, None, 0, C.byref(nnz)),
            "sbp_csr_assemble_host")
    rp = np.empty(n * n + 1, dtype=np.int64)
    col = np.empty(nnz.value, dtype=np.int32)
    val = np.empty(nnz.value, dtype=np.float64)
    got = C.c_longlong()
    L.check(lib.sbp_csr_assemble_host(
        n, rp.ctypes.data_as(C.POINTER(C.c_longlong)), col.ctypes.data_as(C.POINTER(C.c_int)),
        val.ctypes.data_as(C.POINTER(C.c_double)), nnz.value, C.byref(got)),
        "sbp_csr_assemble_host")
    return rp, col, val


class CsrOperator:
    """A on the device in CSR form; ``matvec(x, y)`` is y = A x."""

    def __init__(self, n: int, device="cuda"):
        self.n = n
        rp, col, val = assemble_csr_host(n)
        self.nnz = int(val.size)
        self.row_ptr = torch.from_numpy(rp).to(device)
        self.col = torch.from_numpy(col).to(device)
        self.val = torch.from_numpy(val).to(device)

    @property
    def device_bytes(self) -> int:
        return 8 * self.row_ptr.numel() + 4 * self.col.numel() + 8 * self.val.numel()

    def matvec(self, x: torch.Tensor, y: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        if x.dtype != torch.float64 or x.numel() != self.n * self.n or not x.is_contiguous():
            raise ValueError("x must be a contiguous float64 tensor of n*n entries")
        y = torch.empty_like(x) if y is None else y
        L.check(L.load().sbp_csr_spmv_f64(self.n * self.n, ptr(self.row_ptr), ptr(self.col),
                                          ptr(self.val), ptr(x), ptr(y), _stream_ptr(stream)),
                "sbp_csr_spmv_f64")
        return y
