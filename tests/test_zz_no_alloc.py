"""The Newton linear solve that allocates nothing (ma_laplacian_solve_static).

It exists for callers that cannot let a library allocate device memory (their own
pool owns it all, or cudaMalloc's device-wide synchronisation is not acceptable in
their loop): its CG vectors live in a fixed array inside the library.  This file is
collected last so that a failure here stops a -x run only after every other test.
"""
import ctypes

import numpy as np
import pytest

from mongeampere_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_static_solve_matches_context_solve_twice():
    import torch
    from mongeampere_gb300 import _lib, api

    ctx = api.Context(0)
    lib = ctx.lib
    p = W.make_problem(48, 2000, seed=2)
    v, g, h = api.kantorovich(p.mesh, np.c_[p.x, p.y], np.zeros(p.n), ctx=ctx)
    rhs = np.asarray(g) - p.nu
    # the existing entry point (context-owned scratch) as the reference answer
    d_ref, _ = api.solve_laplacian_matrix(rhs, rtol=1e-13, ctx=ctx)
    rp = torch.tensor(h.rowptr, dtype=torch.int32, device="cuda")
    col = torch.tensor(h.col, dtype=torch.int32, device="cuda")
    val = torch.tensor(h.val, dtype=torch.float64, device="cuda")
    b = torch.tensor(rhs, dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        d = torch.full((p.n,), float("nan"), dtype=torch.float64, device="cuda")
        it = ctypes.c_int64(-1)
        st = lib.ma_laplacian_solve_static(p.n, _ptr(rp), _ptr(col), _ptr(val), _ptr(b), _ptr(d), 1e-13, 0,
                                           ctypes.byref(it), stream)
        assert st == _lib.MA_OK
        out = d.cpu().numpy()
        assert it.value > 0 and out[-1] == 0.0
        np.testing.assert_allclose(out, d_ref, rtol=0, atol=1e-9 * np.abs(d_ref).max())


def test_static_solve_rejects_oversized_systems():
    import torch
    from mongeampere_gb300 import _lib, api

    lib = api.Context(0).lib
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    i = torch.zeros(4, dtype=torch.int32, device="cuda")
    it = ctypes.c_int64(0)
    st = lib.ma_laplacian_solve_static((1 << 18) + 1, _ptr(i), _ptr(i), _ptr(x), _ptr(x), _ptr(x), 1e-10, 0,
                                       ctypes.byref(it), None)
    assert st == _lib.MA_ERR_BUFFER_TOO_SMALL


def test_static_solve_reports_a_capped_iteration():
    # maxiter = 1 cannot reach rtol 1e-13: the call says so (MA_CG_NOCONV) and leaves the
    # first CG iterate in d; a maxiter beyond INT_MAX is capped, not wrapped to zero
    import torch
    from mongeampere_gb300 import _lib, api

    ctx = api.Context(0)
    lib = ctx.lib
    p = W.make_problem(48, 2000, seed=2)
    v, g, h = api.kantorovich(p.mesh, np.c_[p.x, p.y], np.zeros(p.n), ctx=ctx)
    rhs = np.asarray(g) - p.nu
    rp = torch.tensor(h.rowptr, dtype=torch.int32, device="cuda")
    col = torch.tensor(h.col, dtype=torch.int32, device="cuda")
    val = torch.tensor(h.val, dtype=torch.float64, device="cuda")
    b = torch.tensor(rhs, dtype=torch.float64, device="cuda")
    d = torch.zeros(p.n, dtype=torch.float64, device="cuda")
    it = ctypes.c_int64(-1)
    st = lib.ma_laplacian_solve_static(p.n, _ptr(rp), _ptr(col), _ptr(val), _ptr(b), _ptr(d), 1e-13, 1,
                                       ctypes.byref(it), None)
    assert st == _lib.MA_CG_NOCONV
    assert it.value == 1
    assert np.isfinite(d.cpu().numpy()).all()
    d_ref, _ = api.solve_laplacian_matrix(rhs, rtol=1e-13, ctx=ctx)
    it = ctypes.c_int64(-1)
    st = lib.ma_laplacian_solve_static(p.n, _ptr(rp), _ptr(col), _ptr(val), _ptr(b), _ptr(d), 1e-13, 1 << 40,
                                       ctypes.byref(it), None)
    assert st == _lib.MA_OK and it.value > 1
    np.testing.assert_allclose(d.cpu().numpy(), d_ref, rtol=0, atol=1e-9 * np.abs(d_ref).max())
