"""The allocation-free dense Sinkhorn entry point against the allocating one.

``otg_sinkhorn_dense_noalloc`` serves callers that cannot allocate device
memory at solve time (a host whose allocator owns the device pool, or a
latency-bound loop that must not pay cudaMalloc/cudaFree): its scratch is a
static device array inside the library.  Both entry points are called here
through the C ABI on the same problem; the allocation-free one is called
twice, with a call on a different problem (other shape, other form) in
between, because every call reuses the array and must not depend on what
the previous call left in it.  Tolerances are the float64 ones of the dense
parity tests (potentials rtol 1e-8, error history rtol 1e-6) and an
identical status and last iteration index.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import golden
from pot_gb300 import _lib
from pot_gb300.bregman import _hist_cap, default_grid

pytestmark = pytest.mark.gpu


def _problem(M, a, b, reg, method, max_iter, stop):
    n, m = M.shape
    out_u = torch.empty(n, dtype=M.dtype, device=M.device)
    out_v = torch.empty(m, dtype=M.dtype, device=M.device)
    p = _lib.OtgDenseProblem(dtype=_lib.dtype_code(M.dtype), method=method, M=M.data_ptr(), n=n, m=m,
                             ldm=M.stride(0), a=a.data_ptr(), b=b.data_ptr(), warm_u=None, warm_v=None,
                             reg=reg, max_iter=max_iter, hist_cap=_hist_cap(max_iter), stop_thr=stop,
                             out_u=out_u.data_ptr(), out_v=out_v.data_ptr(), workspace_bytes=0,
                             grid=default_grid(n, m), timeout_ms=0)
    return p, out_u, out_v


def _with_alloc(lib, M, a, b, reg, method, max_iter, stop):
    p, u, v = _problem(M, a, b, reg, method, max_iter, stop)
    wsb = lib.otg_dense_workspace_bytes(p.dtype, p.n, p.m, p.hist_cap, p.grid)
    ws = torch.zeros(wsb, dtype=torch.uint8, device=M.device)
    p.workspace_bytes = wsb
    st = _lib.stream_handle(M.device)
    assert lib.otg_sinkhorn_dense(ctypes.byref(p), ctypes.c_void_p(ws.data_ptr()), st) == 0
    torch.cuda.synchronize()
    off = lib.otg_dense_info_offset(p.dtype, p.n, p.m, p.hist_cap, p.grid)
    ctrl = (off + 8 * p.hist_cap + 255) // 256 * 256
    hist = ws[off:off + 8 * p.hist_cap].cpu().numpy().view(np.float64)
    info = ws[ctrl:ctrl + 32].cpu().numpy().view(np.int32)
    return u.cpu().numpy(), v.cpu().numpy(), hist.copy(), info.copy()


def _no_alloc(lib, M, a, b, reg, method, max_iter, stop):
    p, u, v = _problem(M, a, b, reg, method, max_iter, stop)
    hist = torch.full((p.hist_cap,), -1.0, dtype=torch.float64, device=M.device)
    info = torch.full((8,), -7, dtype=torch.int32, device=M.device)
    rc = lib.otg_sinkhorn_dense_noalloc(ctypes.byref(p), ctypes.c_void_p(hist.data_ptr()),
                                        ctypes.c_void_p(info.data_ptr()), _lib.stream_handle(M.device))
    assert rc == 0, rc
    torch.cuda.synchronize()
    return u.cpu().numpy(), v.cpu().numpy(), hist.cpu().numpy(), info.cpu().numpy()


CASES = [("dense_127x129_reg0.05", torch.float64, _lib.OTG_METHOD_LOG, 1e-9),
         ("dense_127x129_reg0.05", torch.float64, _lib.OTG_METHOD_KNOPP, 1e-9),
         ("dense_5x300_reg0.5", torch.float64, _lib.OTG_METHOD_LOG, 1e-9),
         ("dense_100x100_reg0.05", torch.float32, _lib.OTG_METHOD_LOG, 1e-6)]


@pytest.mark.parametrize("name,dtype,method,stop", CASES)
def test_no_alloc_matches_allocating_entry_point(cuda, name, dtype, method, stop):
    lib = _lib.load()
    g = golden(name)
    M = torch.tensor(g["M"], dtype=dtype, device=cuda)
    a = torch.tensor(g["a"], dtype=dtype, device=cuda)
    b = torch.tensor(g["b"], dtype=dtype, device=cuda)
    reg = float(g["reg"])
    ref_u, ref_v, ref_h, ref_i = _with_alloc(lib, M, a, b, reg, method, 2000, stop)
    rtol = 1e-8 if dtype == torch.float64 else 1e-5
    # another problem that leaves different contents in the shared array
    g2 = golden("dense_31x33_reg0.5")
    M2 = torch.tensor(g2["M"], dtype=dtype, device=cuda)
    a2 = torch.tensor(g2["a"], dtype=dtype, device=cuda)
    b2 = torch.tensor(g2["b"], dtype=dtype, device=cuda)
    other = _lib.OTG_METHOD_KNOPP if method == _lib.OTG_METHOD_LOG else _lib.OTG_METHOD_LOG
    for k in range(2):  # two checked calls share the static scratch
        if k == 1:
            _no_alloc(lib, M2, a2, b2, float(g2["reg"]), other, 37, 1e-12)
        u, v, h, info = _no_alloc(lib, M, a, b, reg, method, 2000, stop)
        assert list(info[:4]) == list(ref_i[:4])
        nchk = int(info[2])
        np.testing.assert_allclose(h[:nchk], ref_h[:nchk], rtol=1e-6 if dtype == torch.float64 else 1e-4)
        np.testing.assert_allclose(u, ref_u, rtol=rtol, atol=1e-30)
        np.testing.assert_allclose(v, ref_v, rtol=rtol, atol=1e-30)


def test_no_alloc_rejects_problems_beyond_the_static_scratch(cuda):
    lib = _lib.load()
    n, m = 4, 1 << 22  # the state vectors alone exceed the static array
    M = torch.rand(n, m, dtype=torch.float32, device=cuda)
    a = torch.full((n,), 1.0 / n, dtype=torch.float32, device=cuda)
    b = torch.full((m,), 1.0 / m, dtype=torch.float32, device=cuda)
    p, _, _ = _problem(M, a, b, 1.0, _lib.OTG_METHOD_LOG, 10, 1e-6)
    hist = torch.zeros(p.hist_cap, dtype=torch.float64, device=cuda)
    info = torch.zeros(8, dtype=torch.int32, device=cuda)
    rc = lib.otg_sinkhorn_dense_noalloc(ctypes.byref(p), ctypes.c_void_p(hist.data_ptr()),
                                        ctypes.c_void_p(info.data_ptr()), _lib.stream_handle(cuda))
    assert rc == -6
