"""GPU parity of the Karatsuba convolutions (Convolution/Adhoc.hs,
Convolution/Preprocessed.hs) against the oracle's restatement.

Integer results must be bit-exact (the oracle is itself checked against the
naive int64 convolution).  Floating-point results are bit-exact as well: the
kernels do the reference's additions and leaf products in the reference's
order, exactly as the oracle's loop does in the same precision.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def O():
    from oracle import oracle
    return oracle


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def naive(x, y):
    return np.stack([np.convolve(a.astype(np.int64), b.astype(np.int64)) for a, b in
                     zip(x.reshape(-1, x.shape[-1]), y.reshape(-1, y.shape[-1]))]).reshape(
        x.shape[:-1] + (max(0, 2 * x.shape[-1] - 1),))


LENGTHS = [1, 2, 3, 4, 5, 7, 8, 9, 17, 31, 33, 100, 255, 257, 1000, 1025]


def test_config_int32_4096_to_int64():
    """Int32 length 4096, uniform integers in [-1000, 1000], batch 1, Int64 out."""
    from accelerate_fourier import convolution
    rng = np.random.default_rng(3)
    x = rng.integers(-1000, 1001, (1, 4096)).astype(np.int32)
    y = rng.integers(-1000, 1001, (1, 4096)).astype(np.int32)
    z = host(convolution.karatsuba(dev(x), dev(y)))
    assert z.dtype == np.int64 and z.shape == (1, 8191)
    ref = O().karatsuba(x, y)
    assert np.array_equal(ref, naive(x, y))
    assert np.array_equal(z, ref)


@pytest.mark.parametrize("L", LENGTHS)
def test_karatsuba_int64_exact(L):
    from accelerate_fourier import convolution
    rng = np.random.default_rng(L)
    for batch in (1, 3):
        x = rng.integers(-10 ** 6, 10 ** 6, (batch, L)).astype(np.int64)
        y = rng.integers(-10 ** 6, 10 ** 6, (batch, L)).astype(np.int64)
        z = host(convolution.karatsuba(dev(x), dev(y)))
        assert np.array_equal(z, O().karatsuba(x, y))
        assert np.array_equal(z, O().karatsuba(x, y, recursive=True))
        assert np.array_equal(z, naive(x, y))


def test_karatsuba_int64_wraparound():
    """Products past 2^63 wrap like the reference's Int arithmetic."""
    from accelerate_fourier import convolution
    rng = np.random.default_rng(1)
    x = rng.integers(-2 ** 62, 2 ** 62, (2, 37)).astype(np.int64)
    y = rng.integers(-2 ** 62, 2 ** 62, (2, 37)).astype(np.int64)
    z = host(convolution.karatsuba(dev(x), dev(y)))
    with np.errstate(over="ignore"):
        assert np.array_equal(z, O().karatsuba(x, y))


def test_karatsuba_empty():
    from accelerate_fourier import convolution
    x = torch.zeros((2, 0), dtype=torch.int64, device="cuda")
    z = convolution.karatsuba(x, x)
    assert tuple(z.shape) == (2, 0)


@pytest.mark.parametrize("L", [1, 2, 3, 17, 100, 1000, 4096])
def test_karatsuba_float_bit_exact(L):
    from accelerate_fourier import convolution
    rng = np.random.default_rng(L + 5)
    x = rng.standard_normal((2, L))
    y = rng.standard_normal((2, L))
    z32 = host(convolution.karatsuba(dev(x.astype(np.float32)), dev(y.astype(np.float32))))
    assert np.array_equal(z32, O().karatsuba_f32(x, y))
    z64 = host(convolution.karatsuba(dev(x), dev(y)))
    assert np.array_equal(z64, O().karatsuba_f64(x, y))
    np.testing.assert_allclose(z64, np.stack([np.convolve(a, b) for a, b in zip(x, y)]), atol=1e-9 * L)


@pytest.mark.parametrize("L", [1, 2, 5, 64, 1000])
def test_cyclic_and_complex(L):
    from accelerate_fourier import convolution
    rng = np.random.default_rng(L + 9)
    x = rng.integers(-1000, 1001, (2, L)).astype(np.int64)
    y = rng.integers(-1000, 1001, (2, L)).astype(np.int64)
    cyc = convolution.cyclic(convolution.karatsuba)
    z = host(cyc(dev(x), dev(y)))
    assert np.array_equal(z, O().cyclic_fold(O().karatsuba(x, y), L))
    # complex over linear and cyclic karatsuba, int64 exact
    xi = rng.integers(-1000, 1001, (2, L)).astype(np.int64)
    yi = rng.integers(-1000, 1001, (2, L)).astype(np.int64)
    for cyclic in (False, True):
        conv = convolution.complex(cyc if cyclic else convolution.karatsuba)
        zr, zi = conv((dev(x), dev(xi)), (dev(y), dev(yi)))
        ref = O().karatsuba_complex(x + 1j * xi, y + 1j * yi, cyclic=cyclic)
        assert np.array_equal(host(zr), np.rint(ref.real).astype(np.int64))
        assert np.array_equal(host(zi), np.rint(ref.imag).astype(np.int64))
    # float32 complex: the three products and the combination in float32
    xr32, xi32 = rng.standard_normal((2, 2, L)).astype(np.float32)
    yr32, yi32 = rng.standard_normal((2, 2, L)).astype(np.float32)
    zr, zi = convolution.complex(convolution.karatsuba)((dev(xr32), dev(xi32)), (dev(yr32), dev(yi32)))
    k = O().karatsuba_f32
    rr, ii, mm = k(xr32, yr32), k(xi32, yi32), k(xr32 + xi32, yr32 + yi32)
    assert np.array_equal(host(zr), rr - ii)
    assert np.array_equal(host(zi), mm - (rr + ii))


def test_preprocessed_karatsuba_matches():
    from accelerate_fourier import convolution
    rng = np.random.default_rng(2)
    x = rng.integers(-50, 50, (4, 300)).astype(np.int64)
    y = rng.integers(-50, 50, (4, 300)).astype(np.int64)
    conv = convolution.karatsuba_preprocessed(300)
    assert np.array_equal(host(conv(dev(x), dev(y))), O().karatsuba(x, y, recursive=True))
