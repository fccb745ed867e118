"""Gradients of the spectral-power loss L = sum_k w_k |FFT(x)_k|^2 (w ~ U[0, 1])
through the CUDA forward transforms and their VJPs.

The reference has no AD.  The reference gradient is 2 F^H (w . F x) computed in
FP64 with the oracle (F^H = the unscaled transform of the opposite sign); for
the real transform it is Re of that.  Central finite differences (FP64) of the oracle loss along random directions check the gradient
independently.  Bounds: relative L2 <= c * eps32 * log2 N against the FP64
gradient; directional derivatives agree to 1e-5 relative.
"""
import numpy as np
import pytest

from _util import crand, fp32_bound, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def O():
    from oracle import oracle
    return oracle


def c64(x):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).astype(np.complex64))).cuda()


def f32(x):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).astype(np.float32))).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().astype(np.complex128 if t.is_complex() else np.float64)


def _fd_check(loss, x, grad, rng, dirs=3, h=1e-3):
    """Central differences of loss (FP64) along random unit directions vs
    Re <grad, v> (grad = dL/dRe x + i dL/dIm x for complex x).  L is quadratic,
    so central differences have no truncation error; h = 1e-3 keeps the FP64
    rounding of L (about 1e10 at these sizes) far below the derivative."""
    for _ in range(dirs):
        if np.iscomplexobj(x):
            v = crand(rng, x.shape, "normal")
        else:
            v = rng.standard_normal(x.shape)
        v /= np.linalg.norm(v)
        fd = (loss(x + h * v) - loss(x - h * v)) / (2 * h)
        an = float(np.real(np.vdot(grad, v)))
        assert abs(fd - an) <= 1e-5 * max(abs(fd), np.linalg.norm(grad) * 1e-3), (fd, an)


def _c2c_case(n, batch, algo, mode, seed):
    from accelerate_fourier import planned
    rng = np.random.default_rng(seed)
    x = crand(rng, (batch, n), "normal")
    w = rng.uniform(0, 1, (batch, n))
    t = planned.Transform(-1, n, algo)
    X = t(c64(x))
    Xh = host(X)
    Xref = O().planned(x, -1, mode)
    assert rel_l2(Xh, Xref) <= fp32_bound(n, 4.0)
    g = 2 * w * Xh                                   # the cotangent dL/dconj(X) * 2
    grad = host(t.vjp(c64(g)))
    ref = 2 * O().planned(w * Xref, 1, mode)         # 2 F^H (w . F x), FP64
    assert rel_l2(grad, ref) <= fp32_bound(n, 6.0)

    sub = slice(0, 2)                                # FD on two rows keeps the oracle calls short
    _fd_check(lambda z: float(np.sum(w[sub] * np.abs(O().planned(z, -1, mode)) ** 2)), x[sub], grad[sub], rng)


def test_vjp_c2c_2p16_batch256():
    """Batch 256 x c64 2^16."""
    from oracle import oracle
    _c2c_case(1 << 16, 256, "auto", oracle.AUTO, 51)


@pytest.mark.parametrize("algo", ["chirp2", "chirp235"])
def test_vjp_bluestein_99991_batch32(algo):
    """Batch 32 x Bluestein 99991 (transformChirp2 / transformChirp235; plain
    transform would pick Rader for this prime)."""
    from oracle import oracle
    _c2c_case(99991, 32, algo, oracle.CHIRP2 if algo == "chirp2" else oracle.CHIRP235, 52)


def test_vjp_rader_65537():
    from oracle import oracle
    _c2c_case(65537, 4, "auto", oracle.AUTO, 53)


def test_vjp_real_2p18_batch32():
    """Batch 32 x real FFT 2^18: L = sum w |toSpectrum x|^2, grad = Re F^H (2 w X)."""
    from accelerate_fourier import planned, real
    N, batch = 1 << 18, 32
    rng = np.random.default_rng(54)
    x = rng.standard_normal((batch, N))
    w = rng.uniform(0, 1, (batch, N))
    sub = planned.transform(planned.forward, N // 2)
    X = host(real.toSpectrum(sub, f32(x)))
    Xref = O().to_spectrum(x)
    assert rel_l2(X, Xref) <= fp32_bound(N, 4.0)
    grad = host(real.toSpectrum_vjp(sub, c64(2 * w * X)))
    ref = 2 * np.real(O().planned(w * Xref, 1))
    assert rel_l2(grad, ref) <= fp32_bound(N, 6.0)
    sub2 = slice(0, 2)
    _fd_check(lambda z: float(np.sum(w[sub2] * np.abs(O().to_spectrum(z)) ** 2)), x[sub2], grad[sub2], rng)
