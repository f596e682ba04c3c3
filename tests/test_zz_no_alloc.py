"""The allocation-free 1D entry point, topeExec1DNoAlloc (GPU).

Callers that may not allocate device memory while running (a host
framework owning the memory pool, a fixed budget, a latency-critical path
where cudaMalloc would synchronise the device) pass their own device input
and output buffers; the scratch and the twiddle tables are static device
arrays of the library.  This test allocates the buffers itself (the test is
not such a caller), then checks the entry point, on the same input, against
the FP64 oracle and against the allocating entry point tope1DExec, within
the FP64 gate, for two calls in a row (the second call runs on the state
the first one left in the shared scratch).  It is collected last and also
passes alone in a fresh process, where its first call performs the one-time
table set-up.
"""
import ctypes

import numpy as np
import pytest

from conftest import SEED0, tol_fp64

pytestmark = pytest.mark.gpu


def _reference_result(T, x, n, dir_):
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.check(f)
    T.topeSetArith(f, T.TOPE_ARITH_FP64)
    d = x.copy()
    t = T.TopePlan1D()
    T.tope1DPlanInit(f, t, n, T.C2C, d)
    T.tope1DExec(f, t, d, dir_)
    T.check(f)
    T.tope1DDestroy(f, t)
    T.topeFFTDestroy(f)
    return d


@pytest.mark.parametrize("n", [1, 2, 4, 64, 512, 1024, 4096, 8192, 1 << 14, 1 << 17, 1 << 20])
def test_no_alloc_matches_allocating_entry_point(T, orc, n):
    import torch
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):  # two calls in a row, different inputs
        x = orc.uniform(n, SEED0 + 77 * n + call)
        src = torch.from_numpy(x).to(dev)
        dst = torch.full_like(src, float("nan"))
        for dir_ in (T.FORWARD, T.INVERSE):
            st = T.lib.topeExec1DNoAlloc(ctypes.c_void_p(src.data_ptr()),
                                         ctypes.c_void_p(dst.data_ptr()), n, dir_,
                                         ctypes.c_void_p(stream.cuda_stream))
            assert st == T.TOPE_SUCCESS
            torch.cuda.synchronize(dev)
            got = dst.cpu().numpy()
            assert np.all(np.isfinite(got))
            # the long-double oracle (the restatement keeps the reference's
            # two-point inverse, which halves only the real parts)
            want = x if n == 1 else orc.fft_ld(x, n, dir_=dir_)
            assert orc.rel_l2(got, want) <= tol_fp64(n)
            assert orc.rel_l2(got, _reference_result(T, x, n, dir_)) <= tol_fp64(n)


def test_no_alloc_in_place_and_limits(T, orc):
    import torch
    dev = torch.device("cuda", 0)
    s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    n = 1 << 16
    x = orc.uniform(n, SEED0 + 5)
    buf = torch.from_numpy(x).to(dev)
    p = ctypes.c_void_p(buf.data_ptr())
    assert T.lib.topeExec1DNoAlloc(p, p, n, T.FORWARD, s) == T.TOPE_SUCCESS
    assert T.lib.topeExec1DNoAlloc(p, p, n, T.INVERSE, s) == T.TOPE_SUCCESS
    torch.cuda.synchronize(dev)
    assert orc.rel_l2(buf.cpu().numpy(), x) <= tol_fp64(n)
    # beyond the static scratch, or not a power of two: rejected, nothing queued
    assert T.lib.topeExec1DNoAlloc(p, p, 1 << 21, T.FORWARD, s) == T.TOPE_ERR_INVALID_SIZE
    assert T.lib.topeExec1DNoAlloc(p, p, 3000, T.FORWARD, s) == T.TOPE_ERR_INVALID_SIZE
    assert T.lib.topeExec1DNoAlloc(p, p, 0, T.FORWARD, s) == T.TOPE_ERR_INVALID_SIZE
    assert T.lib.topeExec1DNoAlloc(None, p, 16, T.FORWARD, s) == T.TOPE_ERR_INVALID_ARG
