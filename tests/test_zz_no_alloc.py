"""The no-allocation entry point, af_exec_c2c_noalloc.

Callers that cannot call cudaMalloc (code inside another owner's memory pool,
work that must not touch the CUDA allocator during timing, embedders that
forbid allocation after start-up) use this entry point; its scratch lives in
static device arrays of the library.  The tests call it through the C ABI,
twice in a row, and compare each result with af_exec_c2c on the same input
(and one case with the oracle), within the tolerance the other parity tests
use; they check that the second call allocates no device memory, both signs,
in-place use, n = 1 and the largest allowed n * batch; and that a call on a
capturing stream is refused.  The file runs last (by name) so that a failure
here comes after every other test; it passes both alone in a fresh process and
after the others.
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


def test_rejects_products_that_would_overflow():
    L = _lib().load()
    buf = ctypes.c_void_p(16)
    # 2^21 * 2^43 wraps to 0 in 64 bits: still refused
    assert L.af_exec_c2c_noalloc(1 << 21, -1, buf, buf, 1 << 43, None) == _lib().AF_ERR_INVALID
    assert b"exceeds the static workspace" in L.af_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("n,batch,sign,inplace", [
    (1 << 16, 2, -1, False), (1 << 20, 1, -1, False), (4096, 64, -1, False),
    (4096, 64, 1, False), (1024, 32, -1, True), (1, 7, -1, False), (1 << 21, 1, 1, False),
    (1 << 11, 1 << 10, -1, True)])
def test_noalloc_matches_exec_c2c_on_two_calls(n, batch, sign, inplace):
    import torch
    lib = _lib()
    L = lib.load()
    plan = lib.Plan(n, sign, "auto")
    rng = np.random.default_rng(n + batch)
    s = torch.cuda.current_stream().cuda_stream
    xs = [crand(rng, (batch, n), "normal").astype(np.complex64) for _ in range(2)]
    xds = [torch.from_numpy(x).cuda() for x in xs]
    refs = [torch.empty_like(xd) for xd in xds]
    outs = [xd.clone() if inplace else torch.empty_like(xd) for xd in xds]
    torch.cuda.synchronize()
    free_after_first = None
    for call in range(2):  # two calls in a row: the second reuses the static arrays
        plan.exec_ptr(xds[call].data_ptr(), None, refs[call].data_ptr(), None, batch, s)
        src = outs[call] if inplace else xds[call]
        rc = L.af_exec_c2c_noalloc(n, sign, src.data_ptr(), outs[call].data_ptr(), batch, s)
        assert rc == 0, L.af_last_error()
        torch.cuda.synchronize()
        free = torch.cuda.mem_get_info()[0]
        if call == 0:
            free_after_first = free
        else:
            assert free == free_after_first, "the second call allocated device memory"
        a, b = outs[call].cpu().numpy(), refs[call].cpu().numpy()
        assert rel_l2(a, b) <= fp32_bound(n, 2.0), (call, rel_l2(a, b))


@pytest.mark.gpu
def test_noalloc_matches_the_oracle():
    import torch
    from oracle import oracle
    L = _lib().load()
    n, batch = 1 << 12, 3
    x = crand(np.random.default_rng(3), (batch, n), "normal")
    xd = torch.from_numpy(x.astype(np.complex64)).cuda()
    y = torch.empty_like(xd)
    assert L.af_exec_c2c_noalloc(n, -1, xd.data_ptr(), y.data_ptr(), batch,
                                 torch.cuda.current_stream().cuda_stream) == 0, L.af_last_error()
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), oracle.planned(x, -1)) <= fp32_bound(n, 4.0)


@pytest.mark.gpu
def test_noalloc_refuses_a_capturing_stream():
    import torch
    lib = _lib()
    L = lib.load()
    n = 1024
    xd = torch.ones(n, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(xd)
    g = torch.cuda.CUDAGraph()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(g, stream=stream):
            rc = L.af_exec_c2c_noalloc(n, -1, xd.data_ptr(), y.data_ptr(), 1, stream.cuda_stream)
    assert rc == lib.AF_ERR_UNSUPPORTED
    assert b"cannot be captured" in L.af_last_error()
