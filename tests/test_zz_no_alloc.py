"""The allocation-free residual check (sog_residual_noalloc) against the
residual figures the solver's own entry point reports (sog_solve stats).

That entry point exists for callers that must not allocate device memory
(their memory belongs to another allocator, or an allocation would stall a
latency-critical loop); its scratch is a fixed array in device memory shared
by all calls. The check runs two calls in a row so a second call starting
from the first call's leftovers is covered, and the size limit is exercised.
This file is collected last so a failure here never hides another test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_residual_matches_solver(sg, wl):
    torch = pytest.importorskip("torch")
    s = wl.convdiff2d(40, 5.0, 1.0, nrhs=4)
    ctx = sg.Context()
    plan = sg.Plan(s.n, s.rows, s.cols, s.vals)
    # one FP32 solve without refinement leaves a residual near 1e-7, so the
    # norms are well above rounding noise and comparable across row orders
    sysm = sg.System(ctx, plan, precision=sg.MIXED, max_refine=0, tol=1e-30)
    sysm.factor(s.vals)
    X, st = sysm.solve(s.b, allow_noconv=True)
    assert 1e-12 < st["rel_resid"] < 1e-3
    A = s.to_scipy()
    dev = torch.device("cuda:0")
    ptr = torch.tensor(A.indptr.astype(np.int32), device=dev)
    col = torch.tensor(A.indices.astype(np.int32), device=dev)
    val = torch.tensor(A.data, dtype=torch.float64, device=dev)
    k = s.b.shape[0]
    b = torch.tensor(np.ascontiguousarray(s.b.T), device=dev)  # n x nrhs row-major
    x = torch.tensor(np.ascontiguousarray(X.T), device=dev)
    r = torch.empty_like(b)
    r_ref = np.ascontiguousarray(s.b.T) - A @ np.ascontiguousarray(X.T)
    L = sg.lib()
    for _ in range(2):
        rel = np.zeros(k)
        bwd = np.zeros(k)
        torch.cuda.synchronize()
        rc = L.sog_residual_noalloc(s.n, ptr.data_ptr(), col.data_ptr(), val.data_ptr(), k, b.data_ptr(),
                                    x.data_ptr(), r.data_ptr(), rel.ctypes.data, bwd.ctypes.data, None)
        assert rc == sg.SOG_OK, L.sog_last_error()
        np.testing.assert_allclose(r.cpu().numpy(), r_ref, rtol=0, atol=1e-10 * np.abs(s.b).max())
        np.testing.assert_allclose(rel.max(), st["rel_resid"], rtol=1e-6)
        np.testing.assert_allclose(bwd.max(), st["backward_error"], rtol=1e-6)
    # beyond the fixed scratch size: refused with a clear error, nothing launched
    big = np.zeros(65)
    rc = L.sog_residual_noalloc(s.n, ptr.data_ptr(), col.data_ptr(), val.data_ptr(), 65, b.data_ptr(),
                                x.data_ptr(), r.data_ptr(), big.ctypes.data, big.ctypes.data, None)
    assert rc == sg.SOG_EINVAL and b"nrhs" in L.sog_last_error()
    sysm.close()
    ctx.close()
