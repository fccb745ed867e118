"""The no-allocation entry point, af_exec_c2c_noalloc.

Callers that cannot call cudaMalloc (code inside another owner's memory pool,
work that must not touch the CUDA allocator during capture or timing,
embedders that forbid allocation after start-up) use this entry point; its
scratch lives in static device arrays of the library.  The test calls it
through the C ABI twice in a row and compares each result with
af_exec_c2c on the same input, within the tolerance the other parity tests
use.  It runs last (file name) so that a failure here comes after every other
test, and it passes both alone in a fresh process and after the others.
"""
import ctypes

import numpy as np
import pytest

from _util import crand, fp32_bound, rel_l2


def _lib():
    from accelerate_fourier import _lib
    return _lib


def test_rejects_sizes_beyond_the_static_workspace():
    L = _lib().load()
    buf = ctypes.c_void_p(16)
    rc = L.af_exec_c2c_noalloc(1 << 22, -1, buf, buf, 1, None)
    assert rc == _lib().AF_ERR_INVALID
    assert b"exceeds the static workspace" in L.af_last_error()
    assert L.af_exec_c2c_noalloc(12, -1, buf, buf, 1, None) == _lib().AF_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("n,batch", [(1 << 16, 2), (1 << 20, 1), (4096, 64)])
def test_noalloc_matches_exec_c2c_on_two_calls(n, batch):
    import torch
    lib = _lib()
    L = lib.load()
    plan = lib.Plan(n, -1, "auto")
    rng = np.random.default_rng(n)
    s = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row: the second reuses the static arrays
        x = crand(rng, (batch, n), "normal").astype(np.complex64)
        xd = torch.from_numpy(x).cuda()
        y_ref = torch.empty_like(xd)
        y = torch.empty_like(xd)
        plan.exec_ptr(xd.data_ptr(), None, y_ref.data_ptr(), None, batch, s)
        rc = L.af_exec_c2c_noalloc(n, -1, xd.data_ptr(), y.data_ptr(), batch, s)
        assert rc == 0, L.af_last_error()
        torch.cuda.synchronize()
        a, b = y.cpu().numpy(), y_ref.cpu().numpy()
        assert rel_l2(a, b) <= fp32_bound(n, 2.0), (call, rel_l2(a, b))
