"""The bounded-wait failure path, made to happen without a GPU fault: a
test switch makes CTA 0 of every persistent stencil launch declare its first
tile's bytes to the tile's mbarrier without issuing the copy, and shortens
the bounded waits.  Nothing is read or written out of bounds and every wait
ends; the solve must report SBP_ERR_TIMEOUT and the same handle must then
solve exactly as before."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import sbp_oracle as o

pytestmark = pytest.mark.gpu


def test_lost_copy_reports_timeout_and_handle_recovers(sbp):
    from sc_2022_gb300 import _lib
    lib = sbp.load_library()
    n = 129
    a = o.assemble(n)
    F, g, _ = o.manufactured(n, "baseline")
    b = torch.tensor(a.rhs(F, g), dtype=torch.float64, device="cuda")
    for prec in (_lib.SBP_PREC_FP64, _lib.SBP_PREC_MIXED):
        s = sbp.Solver(n, sbp.default_options(prec))
        x0 = torch.zeros_like(b)
        ref = s.mgcg(b, x0, reltol=1e-10)
        assert ref.converged
        x1 = torch.zeros_like(b)
        assert lib.sbp_test_drop_copy(1, 1 << 10) == 0
        try:
            with pytest.raises(sbp.SbpError) as err:
                s.mgcg(b, x1, reltol=1e-10)
        finally:
            assert lib.sbp_test_drop_copy(0, 0) == 0
        assert err.value.status == _lib.SBP_ERR_TIMEOUT
        assert "bounded wait" in str(err.value)
        # the flag was read and cleared: the handle solves as before, bit for bit
        x2 = torch.zeros_like(b)
        again = s.mgcg(b, x2, reltol=1e-10)
        assert again.converged and again.iters == ref.iters
        assert torch.equal(x2, x0)
        s.close()
    # and the single-grid entry points are unaffected
    out = torch.empty_like(b)
    assert lib.sbp_apply_f64(C.c_void_p(b.data_ptr()), C.c_void_p(out.data_ptr()), n, -1,
                             None) == 0
    torch.cuda.synchronize()
    ref_out = -(a.A @ b.cpu().numpy())
    assert np.linalg.norm(out.cpu().numpy() - ref_out) <= 1e-13 * np.linalg.norm(ref_out)
