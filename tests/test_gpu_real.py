"""GPU parity of the real transforms, the two-real-signal functions, the
cyclic convolution, the 2-D/3-D transforms and Cyclic.reverse2d against the
oracle (FP64 restatement of Real.hs, Planned.convolveCyclic, Cyclic.hs).

Floating-point bound: relative L2 <= c * eps32 * log2 N (eps32 = 2^-24), with
c stated per test.  Index maps (reverse, reverse2d) are compared exactly.
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


REAL_N = [2, 4, 6, 8, 10, 30, 64, 200, 1000, 1024, 2 * 1009, 2 * 4099, 2 * 65537, 1 << 18]


@pytest.mark.parametrize("N", REAL_N)
def test_to_spectrum(N):
    from accelerate_fourier import planned, real
    rng = np.random.default_rng(N)
    batch = 3 if N < (1 << 17) else 2
    x = rng.standard_normal((batch, N))
    ref = O().to_spectrum(x)                       # Real.toSpectrum, FP64
    np.testing.assert_allclose(ref, np.fft.fft(x, axis=-1), atol=1e-8 * N)
    sub = planned.transform(planned.forward, N // 2)
    y = host(real.toSpectrum(sub, f32(x)))
    assert rel_l2(y, ref) <= fp32_bound(N, 4.0)
    yh = host(real.toSpectrum(sub, f32(x), half=True))
    assert yh.shape[-1] == N // 2 + 1
    assert rel_l2(yh, ref[:, : N // 2 + 1]) <= fp32_bound(N, 4.0)


@pytest.mark.parametrize("N", REAL_N)
def test_from_spectrum(N):
    from accelerate_fourier import planned, real
    rng = np.random.default_rng(N + 7)
    x = rng.standard_normal((2, N))
    spec = np.fft.fft(x, axis=-1)                 # self-adjoint spectrum
    ref = O().from_spectrum(spec)                 # Real.fromSpectrum = N x (unscaled)
    np.testing.assert_allclose(ref, N * x, atol=1e-7 * N)
    sub = planned.transform(planned.inverse, N // 2)
    y = host(real.fromSpectrum(sub, c64(spec)))
    assert rel_l2(y, ref) <= fp32_bound(N, 4.0)
    yp = host(real.fromSpectrum(sub, (f32(spec.real), f32(spec.imag))))
    assert rel_l2(yp, ref) <= fp32_bound(N, 4.0)


def test_to_spectrum_config_r2c_2p24_batch8():
    """R2C, Float32 N = 2^24, batch 8: vs numpy's FP64 FFT (the oracle is
    pinned to numpy at smaller sizes), plus Parseval."""
    from accelerate_fourier import planned, real
    N, batch = 1 << 24, 8
    rng = np.random.default_rng(3)
    x = rng.standard_normal((batch, N)).astype(np.float32)
    sub = planned.transform(planned.forward, N // 2)
    y = real.toSpectrum(sub, f32(x))
    for b in range(batch):
        ref = np.fft.fft(x[b].astype(np.float64))
        yb = y[b].cpu().numpy().astype(np.complex128)
        assert rel_l2(yb, ref) <= fp32_bound(N, 4.0)
        # Parseval: sum |X|^2 = N sum x^2
        p = float(np.sum(np.abs(yb) ** 2))
        assert abs(p - N * float(np.sum(x[b].astype(np.float64) ** 2))) <= 1e-5 * p
    del y
    torch.cuda.empty_cache()


@pytest.mark.parametrize("N", [2, 8, 30, 1024, 2 * 1009, 1 << 18])
def test_to_spectrum_vjp(N):
    """Adjoint identity <toSpectrum x, g> = <x, vjp g> (real part), and the
    value Re(DFT^H g) in FP64."""
    from accelerate_fourier import planned, real
    rng = np.random.default_rng(N + 11)
    batch = 2
    g = crand(rng, (batch, N), "normal")
    ref = np.real(np.fft.ifft(g, axis=-1) * N)
    sub = planned.transform(planned.forward, N // 2)
    v = host(real.toSpectrum_vjp(sub, c64(g)))
    assert rel_l2(v, ref) <= fp32_bound(N, 4.0)


@pytest.mark.parametrize("n", [1, 2, 5, 16, 100, 1001, 4099, 30011])
def test_two_to_spectrum(n):
    from accelerate_fourier import planned, real
    rng = np.random.default_rng(n)
    f, g = rng.standard_normal((2, 3, n))
    spec = O().planned(f + 1j * g, -1)
    ra, rb = O().untangle(spec)                   # Real.untangleSpectra, FP64
    np.testing.assert_allclose(ra, np.fft.fft(f, axis=-1), atol=1e-8 * max(n, 1))
    t = planned.transform(planned.forward, n)
    a, b = real.twoToSpectrum(t, (f32(f), f32(g)))
    assert rel_l2(host(a), ra) <= fp32_bound(n, 4.0)
    assert rel_l2(host(b), rb) <= fp32_bound(n, 4.0)
    # standalone untangle of a given spectrum
    a2, b2 = real.untangleSpectra(c64(spec))
    assert rel_l2(host(a2), ra) <= 1e-6 and rel_l2(host(b2), rb) <= 1e-6
    # twoFromSpectrum inverts it (unscaled: n f, n g)
    ti = planned.transform(planned.inverse, n)
    f2, g2 = real.twoFromSpectrum(ti, (c64(ra), c64(rb)))
    assert rel_l2(host(f2), n * f) <= fp32_bound(n, 4.0)
    assert rel_l2(host(g2), n * g) <= fp32_bound(n, 4.0)


def test_entangle_matches_oracle():
    from accelerate_fourier import real
    rng = np.random.default_rng(5)
    c, d = crand(rng, (2, 4, 33))
    ref = O().entangle(c, d)
    out = host(real.entangleSpectra((c64(c), c64(d))))
    assert rel_l2(out, ref) <= 1e-7
    a, b = real.untangleCoefficient(1 + 2j, 3 - 1j)
    assert abs(a - ((1 + 2j) + (3 + 1j)) / 2) < 1e-12


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 3, 5), (1, 16, 32), (2, 7, 100), (1, 64, 1001), (1, 257, 12)])
def test_two_to_spectrum_2d(shape):
    from accelerate_fourier import planned, preprocessed, real
    rng = np.random.default_rng(sum(shape))
    f, g = rng.standard_normal((2,) + shape)
    h, w = shape[-2:]
    t2 = preprocessed.transform2d(planned.transform(-1, w), planned.transform(-1, h))
    a, b = real.twoToSpectrum2d(t2, (f32(f), f32(g)))
    ra, rb = np.fft.fft2(f), np.fft.fft2(g)
    bound = fp32_bound(h * w, 4.0)
    assert rel_l2(host(a), ra) <= bound and rel_l2(host(b), rb) <= bound
    ti = preprocessed.transform2d(planned.transform(1, w), planned.transform(1, h))
    f2, g2 = real.twoFromSpectrum2d(ti, (c64(ra), c64(rb)))
    assert rel_l2(host(f2), h * w * f) <= bound and rel_l2(host(g2), h * w * g) <= bound


@pytest.mark.parametrize("n", [1, 2, 7, 64, 1001, 1024, 4099, 65537, 1 << 20])
def test_convolve_cyclic(n):
    from accelerate_fourier import planned
    rng = np.random.default_rng(n + 3)
    batch = 2 if n <= 65537 else 1
    x = crand(rng, (batch, n), "normal")
    y = crand(rng, (batch, n), "normal")
    conv = planned.convolveCyclic(n)
    if n <= 65537:
        ref = O().convolve_cyclic(x, y)          # Planned.convolveCyclic, FP64
    else:
        ref = np.fft.ifft(np.fft.fft(x) * np.fft.fft(y))
    np.testing.assert_allclose(ref, np.fft.ifft(np.fft.fft(x) * np.fft.fft(y)), atol=1e-9 * n)
    out = host(conv(c64(x), c64(y)))
    assert rel_l2(out, ref) <= fp32_bound(n, 6.0)
    outp = conv((f32(x.real), f32(x.imag)), (f32(y.real), f32(y.imag)))
    assert rel_l2(host(outp[0]) + 1j * host(outp[1]), ref) <= fp32_bound(n, 6.0)


def test_convolve_cyclic_real_2p20_pair():
    """Two Float32 2^20 real signals (zero imaginary parts)."""
    from accelerate_fourier import planned
    n = 1 << 20
    rng = np.random.default_rng(33)
    x, y = rng.standard_normal((2, 1, n))
    ref = np.fft.ifft(np.fft.fft(x) * np.fft.fft(y))
    out = host(planned.convolveCyclic(n)(c64(x), c64(y)))
    assert rel_l2(out, ref) <= fp32_bound(n, 6.0)
    assert np.abs(out.imag).max() <= 1e-5 * np.abs(out.real).max()


ND_SHAPES = [(1, 1, 1), (2, 4, 8), (3, 5, 7), (1, 16, 1024), (2, 100, 64), (1, 1001, 16), (1, 4099, 4),
             (2, 17, 4099), (1, 30011, 2), (2, 65537, 1), (1, 12, 65536)]


@pytest.mark.parametrize("shape", ND_SHAPES)
def test_transform2d(shape):
    from accelerate_fourier import adhoc, planned, preprocessed
    rng = np.random.default_rng(sum(shape))
    x = crand(rng, shape)
    h, w = shape[-2:]
    bound = fp32_bound(h * w, 5.0)
    for sign in (-1, 1):
        ref = np.fft.fft2(x) if sign < 0 else np.fft.ifft2(x) * h * w
        t2 = preprocessed.transform2d(planned.transform(sign, w), planned.transform(sign, h))
        assert rel_l2(host(t2(c64(x))), ref) <= bound
    # oracle per axis (Planned.transform on the last axis, then on the other)
    o = O().planned(x, -1)
    o = np.swapaxes(O().planned(np.ascontiguousarray(np.swapaxes(o, -1, -2)), -1), -1, -2)
    assert rel_l2(o, np.fft.fft2(x)) <= 1e-12
    assert rel_l2(host(adhoc.transform2d(-1, c64(x))), o) <= bound
    # planar, mixed signs per axis
    t2 = preprocessed.transform2d(planned.transform(-1, w), planned.transform(1, h))
    re, im = t2((f32(x.real), f32(x.imag)))
    ref = np.fft.ifft(np.fft.fft(x, axis=-1), axis=-2) * h
    assert rel_l2(host(re) + 1j * host(im), ref) <= bound


@pytest.mark.parametrize("shape", [(1, 2, 3, 4), (2, 8, 16, 32), (1, 7, 11, 13), (1, 5, 64, 257), (1, 64, 64, 64)])
def test_transform3d(shape):
    from accelerate_fourier import adhoc, planned, preprocessed
    rng = np.random.default_rng(sum(shape))
    x = crand(rng, shape)
    d, h, w = shape[-3:]
    ref = np.fft.fftn(x, axes=(-3, -2, -1))
    bound = fp32_bound(d * h * w, 5.0)
    t3 = preprocessed.transform3d(planned.transform(-1, w), planned.transform(-1, h), planned.transform(-1, d))
    assert rel_l2(host(t3(c64(x))), ref) <= bound
    assert rel_l2(host(adhoc.transform3d(-1, c64(x))), ref) <= bound


def test_transform2d_in_place_and_chirp_axis():
    from accelerate_fourier import planned, preprocessed
    rng = np.random.default_rng(9)
    x = crand(rng, (2, 1009, 24))
    t2 = preprocessed.transform2d(planned.transform(-1, 24), planned.transformChirp2(-1, 1009))
    X = c64(x)
    t2(X, out=X)
    assert rel_l2(host(X), np.fft.fft2(x)) <= fp32_bound(1009 * 24, 6.0)


@pytest.mark.parametrize("shape", [(1, 1), (3, 1), (1, 5), (4, 6), (2, 7, 9)])
def test_reverse2d(shape):
    from accelerate_fourier import cyclic
    rng = np.random.default_rng(len(shape))
    x = crand(rng, shape).astype(np.complex64)
    y = host(cyclic.reverse2d(c64(x)))
    h, w = shape[-2:]
    ref = x[..., (-np.arange(h)) % h, :][..., (-np.arange(w)) % w]
    assert np.array_equal(y, ref.astype(np.complex128))


def test_axis_entry_matches_strided_transform():
    """af_exec_c2c_axis along the middle axis of (outer, n, inner)."""
    import ctypes  # noqa: F401
    from accelerate_fourier import _lib, _tensor, planned
    rng = np.random.default_rng(12)
    outer, n, inner = 3, 1000, 7
    x = crand(rng, (outer, n, inner))
    X = c64(x)
    Y = torch.empty_like(X)
    t = planned.transform(-1, n)
    _lib.check(_lib.load().af_exec_c2c_axis(t.plan.handle, _lib.INTERLEAVED, X.data_ptr(), None, Y.data_ptr(), None,
                                            outer, inner, _tensor.stream_ptr()))
    assert rel_l2(host(Y), np.fft.fft(x, axis=1)) <= fp32_bound(n, 4.0)
