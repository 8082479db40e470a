"""The allocation-free entry point sbp_apply_dot_f64_noalloc.

Some callers cannot let a library allocate device memory for them: hosts
whose device memory belongs to their own allocator or pool, and loops that
must never enter the CUDA allocator.  For them the library offers an apply +
dot whose reduction scratch is a static device array instead of a
stream-ordered allocation.  This file checks it, through the C ABI, against
the regular sbp_apply_dot_f64 on two calls in a row (the second call reuses
the static scratch the first one left behind).  It is named so that pytest
collects it last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

APPLY_RTOL = 1e-13   # operator apply, relative 2-norm (as in test_gpu_ops.py)
DOT_RTOL = 1e-12


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("n", [257, 4097])
def test_noalloc_matches_allocating_entry_point(n):
    import sc_2022_gb300 as sbp
    lib = sbp.load_library()
    assert torch.cuda.is_available()
    g = torch.Generator(device="cuda").manual_seed(n)
    u = torch.randn(n * n, generator=g, device="cuda", dtype=torch.float64)
    ref_out = torch.empty_like(u)
    ref_dot = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for sign in (1, -1):
        assert lib.sbp_apply_dot_f64(_ptr(u), _ptr(ref_out), n, sign, _ptr(ref_dot), stream) == 0
        torch.cuda.synchronize()
        want_out = ref_out.clone()
        want_dot = ref_dot.item()
        for call in range(2):
            out = torch.full_like(u, float("nan"))
            dot = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
            rc = lib.sbp_apply_dot_f64_noalloc(_ptr(u), _ptr(out), n, sign, _ptr(dot), stream)
            assert rc == 0, lib.sbp_status_string(rc).decode()
            torch.cuda.synchronize()
            err = ((out - want_out).norm() / want_out.norm()).item()
            assert err <= APPLY_RTOL, f"call {call}: apply rel err {err}"
            got = dot.item()
            assert abs(got - want_dot) <= DOT_RTOL * abs(want_dot), f"call {call}: dot {got} vs {want_dot}"


def test_noalloc_rejects_bad_arguments():
    import sc_2022_gb300 as sbp
    from sc_2022_gb300 import _lib
    lib = sbp.load_library()
    x = torch.zeros(9, dtype=torch.float64, device="cuda")
    assert lib.sbp_apply_dot_f64_noalloc(_ptr(x), _ptr(x), 2, 1, _ptr(x), None) == _lib.SBP_ERR_ARGS
    assert lib.sbp_apply_dot_f64_noalloc(None, _ptr(x), 3, 1, _ptr(x), None) == _lib.SBP_ERR_ARGS
