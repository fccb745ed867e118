"""GPU parity of the Complex Double (FP64) transforms.

The reference's transforms are polymorphic over the element type, and its own
test suite runs them on Complex Double with an absolute tolerance of 1e-10
(test/Test/Data/Array/Accelerate/Fourier.hs:34-35).  Here the FP64 build of
the kernels is checked (1) against the oracle (the FP64 CPU restatement of
the reference algorithm) and numpy's FFT with a c * eps64 * log2 N relative
L2 bound, and (2) through the reference's own properties at its own
tolerance: impulse to basis vector, inverse round trip, double transform =
n * reverse, isometry (Fourier.hs:219-223,367-417).
"""
import numpy as np
import pytest

from _util import crand, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = 1e-10  # Fourier.hs:34-35


def O():
    from oracle import oracle
    return oracle


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.complex128))).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def fp64_bound(n, c=64.0):
    """c * eps64 * log2 N relative-L2 bound for an FP64 transform of length n."""
    return c * 2.0 ** -53 * max(1.0, np.log2(max(n, 2)))


def transform(sign, n, algo="auto"):
    from accelerate_fourier import planned
    return planned.Transform(sign, n, algo)


SMALL = list(range(1, 41)) + [47, 49, 64, 81, 97, 100]
MEDIUM = [127, 128, 243, 256, 360, 1000, 1001, 1024, 2310, 3125, 4096, 4097, 6144, 6250, 7776, 8192,
          9973, 10007, 12288, 16384, 16385, 30030]
LARGE = [65536, 65537, 99991, 1 << 20, 3 ** 12, 1001 * 1024]


@pytest.mark.parametrize("n", SMALL + MEDIUM + LARGE)
def test_f64_planned_vs_oracle(n):
    rng = np.random.default_rng(n)
    batch = 3 if n <= 20000 else 1
    x = crand(rng, (batch, n))
    for sign in (-1, 1):
        t = transform(sign, n)
        y = host(t(dev(x)))
        assert y.dtype == np.complex128
        np_ref = np.fft.fft(x, axis=-1) if sign < 0 else np.fft.ifft(x, axis=-1) * n
        assert rel_l2(y, np_ref) <= fp64_bound(n), (n, sign, rel_l2(y, np_ref))
        # The oracle computes chirp phases pi k^2 / N in floating point, as the
        # reference does (Private.hs:428-436): a phase error near eps64 * k^2 / N,
        # up to about eps64 * N.  The kernels reduce k^2 mod 2N exactly.
        bound = fp64_bound(n) + (8 * 2.0 ** -53 * n if "BL" in t.describe() else 0.0)
        err = rel_l2(y, O().planned(x, sign, 0))
        assert err <= bound, f"n={n} sign={sign} plan={t.describe()} rel_l2={err:.3e}"


def test_f64_bluestein_1000003():
    """The chirp-z size of the benchmark (pad 2025000): against numpy (the
    oracle's chirp phase follows the reference's floating-point formula)."""
    n = 1000003
    rng = np.random.default_rng(2)
    x = rng.standard_normal((1, n)) + 1j * rng.standard_normal((1, n))
    y = host(transform(-1, n)(dev(x)))
    assert rel_l2(y, np.fft.fft(x, axis=-1)) <= fp64_bound(n)


@pytest.mark.parametrize("algo,sizes", [
    ("decompose", [17, 1009, 4099]),
    ("chirp2", [2, 17, 100, 1009, 4099, 16385]),
    ("chirp235", [3, 17, 100, 1009, 4099, 16385]),
    ("prep_splitradix", [1, 2, 64, 1024, 8192]),
    ("prep_dit2", [2, 256, 4096]),
    ("prep_dif2", [2, 256, 4096]),
    ("adhoc_auto", [7, 100, 1009, 4099]),
    ("adhoc_dit235", [6, 360, 3125, 7776]),
])
def test_f64_algorithms(algo, sizes):
    for n in sizes:
        rng = np.random.default_rng(n + 7)
        x = crand(rng, (2, n))
        y = host(transform(-1, n, algo)(dev(x)))
        assert rel_l2(y, np.fft.fft(x, axis=-1)) <= fp64_bound(n), (algo, n)


def test_f64_reference_properties():
    """Fourier.hs properties at the reference's own tolerance (absolute 1e-10
    per element, Complex Double, genComplex inputs U[-1,1]^2)."""
    rng = np.random.default_rng(11)
    lengths = list(range(1, 101)) + [128, 1000, 1024, 4099]
    for n in lengths:
        fwd, inv = transform(-1, n), transform(1, n)
        x = crand(rng, (n,))
        X = dev(x)
        F = fwd(X)
        # inverse round trip: inverse (forward x) = n x   (Fourier.hs:377-382)
        assert np.max(np.abs(host(inv(F)) - n * x)) <= TOL * n, n
        # double transform = n * cyclic reverse            (Fourier.hs:383-390)
        rev = np.roll(x[::-1], 1)
        assert np.max(np.abs(host(fwd(F)) - n * rev)) <= TOL * n, n
        # isometry: |F x|^2 = n |x|^2                       (Fourier.hs:403-417)
        f = host(F)
        assert abs(np.vdot(f, f).real - n * np.vdot(x, x).real) <= TOL * n * n, n
        # impulse at k -> basis vector                      (Fourier.hs:219-223,367-376)
        k = int(rng.integers(n))
        e = np.zeros(n, complex)
        e[k] = 1
        expect = np.exp(-2j * np.pi * k * np.arange(n) / n)
        assert np.max(np.abs(host(fwd(dev(e))) - expect)) <= TOL, n


def test_f64_vjp_and_planar():
    n, batch = 3000, 4
    rng = np.random.default_rng(5)
    x = crand(rng, (batch, n))
    t = transform(-1, n)
    g = host(t.vjp(dev(x)))
    assert rel_l2(g, np.fft.ifft(x, axis=-1) * n) <= fp64_bound(n)
    re = torch.from_numpy(x.real.copy()).cuda()
    im = torch.from_numpy(x.imag.copy()).cuda()
    yr, yi = t((re, im))
    assert yr.dtype == torch.float64
    y = host(yr) + 1j * host(yi)
    assert rel_l2(y, np.fft.fft(x, axis=-1)) <= fp64_bound(n)


@pytest.mark.parametrize("shape", [(2, 48, 30), (1, 100, 257), (3, 16, 4099)])
def test_f64_transform2d(shape):
    from accelerate_fourier import planned
    rng = np.random.default_rng(sum(shape))
    x = crand(rng, shape)
    t = planned.TransformND(transform(-1, shape[-1]), transform(-1, shape[-2]))
    y = host(t(dev(x)))
    assert rel_l2(y, np.fft.fft2(x, axes=(-2, -1))) <= fp64_bound(shape[-1] * shape[-2])


def test_f64_transform3d():
    from accelerate_fourier import planned
    shape = (2, 12, 20, 17)
    rng = np.random.default_rng(3)
    x = crand(rng, shape)
    t = planned.TransformND(transform(1, 17), transform(1, 20), transform(1, 12))
    y = host(t(dev(x)))
    ref = np.fft.ifftn(x, axes=(-3, -2, -1)) * (12 * 20 * 17)
    assert rel_l2(y, ref) <= fp64_bound(12 * 20 * 17)


def test_f64_and_f32_plans_refuse_each_other():
    import ctypes
    from accelerate_fourier import _lib
    L = _lib.load()
    p32, p64 = _lib.Plan(64, -1), _lib.Plan(64, -1, double=True)
    a = torch.zeros(64, dtype=torch.complex128, device="cuda")
    b = torch.zeros(64, dtype=torch.complex128, device="cuda")
    assert L.af_exec_c2c(p64.handle, 0, a.data_ptr(), None, b.data_ptr(), None, 1, None) == _lib.AF_ERR_INVALID
    assert b"Complex Double" in L.af_last_error()
    assert L.af_exec_c2c_f64(p32.handle, 0, a.data_ptr(), None, b.data_ptr(), None, 1, None) == _lib.AF_ERR_INVALID
    # interleaved Complex Double data must be 16-byte aligned
    assert L.af_exec_c2c_f64(p64.handle, 0, a.data_ptr() + 8, None, b.data_ptr(), None, 1,
                             None) == _lib.AF_ERR_INVALID
    n = ctypes.c_int64()
    assert L.af_plan_launches(p64.handle, 4, ctypes.byref(n)) == 0 and n.value >= 1


# ---------------------------------------------------------------- real, two-real, convolution, maps
def f64(x):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64))).cuda()


@pytest.mark.parametrize("N", [2, 6, 64, 1000, 2 * 1009, 2 * 4099, 2 * 65537, 1 << 18])
def test_f64_to_from_spectrum(N):
    from accelerate_fourier import real
    rng = np.random.default_rng(N)
    x = rng.standard_normal((2, N))
    sub = transform(-1, N // 2)
    y = host(real.toSpectrum(sub, f64(x)))
    assert y.dtype == np.complex128
    ref = np.fft.fft(x, axis=-1)
    assert rel_l2(y, ref) <= fp64_bound(N)
    # the oracle's chirp phases carry about eps64 * N (see test_f64_planned_vs_oracle)
    chirp = 8 * 2.0 ** -53 * N if "BL" in sub.describe() else 0.0
    assert rel_l2(y, O().to_spectrum(x)) <= fp64_bound(N) + chirp
    yh = host(real.toSpectrum(sub, f64(x), half=True))
    assert rel_l2(yh, ref[:, : N // 2 + 1]) <= fp64_bound(N)
    # fromSpectrum (unscaled inverse) of the full spectrum: N x
    z = host(real.fromSpectrum(transform(1, N // 2), dev(ref)))
    assert z.dtype == np.float64
    assert rel_l2(z, N * x) <= fp64_bound(N)
    # VJP of toSpectrum: Re(DFT^H g)
    g = crand(rng, (2, N))
    v = host(real.toSpectrum_vjp(sub, dev(g)))
    assert rel_l2(v, (np.fft.ifft(g, axis=-1) * N).real) <= fp64_bound(N)


@pytest.mark.parametrize("n", [1, 7, 100, 1009, 4096])
def test_f64_two_real(n):
    from accelerate_fourier import real
    rng = np.random.default_rng(n)
    f, g = rng.standard_normal((3, n)), rng.standard_normal((3, n))
    t = transform(-1, n)
    a, b = real.twoToSpectrum(t, (f64(f), f64(g)))
    a, b = host(a), host(b)
    assert rel_l2(a, np.fft.fft(f, axis=-1)) <= fp64_bound(n)
    assert rel_l2(b, np.fft.fft(g, axis=-1)) <= fp64_bound(n)
    ff, gg = real.twoFromSpectrum(transform(1, n), (dev(a), dev(b)))
    assert rel_l2(host(ff), n * f) <= fp64_bound(n) and rel_l2(host(gg), n * g) <= fp64_bound(n)
    # untangle / entangle are inverse element-wise maps
    s = crand(rng, (3, n))
    u, w = real.untangleSpectra(dev(s))
    back = host(real.entangleSpectra((u, w)))
    assert rel_l2(back, s) <= 1e-15


def test_f64_two_real_2d():
    from accelerate_fourier import planned, real
    rng = np.random.default_rng(9)
    f, g = rng.standard_normal((2, 24, 30)), rng.standard_normal((2, 24, 30))
    t2 = planned.TransformND(transform(-1, 30), transform(-1, 24))
    a, b = real.twoToSpectrum2d(t2, (f64(f), f64(g)))
    assert rel_l2(host(a), np.fft.fft2(f)) <= fp64_bound(720)
    assert rel_l2(host(b), np.fft.fft2(g)) <= fp64_bound(720)


@pytest.mark.parametrize("n", [1, 12, 1000, 4099, 1 << 16])
def test_f64_convolve_cyclic(n):
    from accelerate_fourier import planned
    rng = np.random.default_rng(n)
    x, y = crand(rng, (2, n)), crand(rng, (2, n))
    z = host(planned.convolveCyclic(n)(dev(x), dev(y)))
    ref = np.fft.ifft(np.fft.fft(x, axis=-1) * np.fft.fft(y, axis=-1), axis=-1)
    assert z.dtype == np.complex128
    assert rel_l2(z, ref) <= fp64_bound(n)
    zp = planned.convolveCyclic(n)((f64(x.real), f64(x.imag)), (f64(y.real), f64(y.imag)))
    assert rel_l2(host(zp[0]) + 1j * host(zp[1]), ref) <= fp64_bound(n)


def test_f64_reverse_and_scale_down():
    from accelerate_fourier import cyclic, utility
    rng = np.random.default_rng(4)
    x = crand(rng, (3, 17, 10))
    r = host(cyclic.reverse(dev(x)))
    assert np.array_equal(r, np.roll(x[..., ::-1], 1, axis=-1))
    r2 = host(cyclic.reverse2d(dev(x)))
    assert np.array_equal(r2, np.roll(np.roll(x[..., ::-1, ::-1], 1, axis=-1), 1, axis=-2))
    s = host(utility.scaleDown(dev(x)))
    assert s.dtype == np.complex128
    np.testing.assert_allclose(s, x / 10, rtol=4e-16, atol=0)
