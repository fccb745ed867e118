"""CPU tests of the oracle (the restatement of the reference algorithms).

1. Pins: the permutation tables written in the reference's source comments,
   the reference's known-answer test (inverse transform of a unit impulse is
   a basis vector, test/Test/Data/Array/Accelerate/Fourier.hs:219-223,367-376),
   a long-double naive DFT, and numpy's FFT.
2. The reference's 38 QuickCheck properties (Fourier.hs:298-587), ported to
   seeded examples with the reference's tolerance: |x - y| <= 1e-10 absolute
   per element (Fourier.hs:34-47), lengths 0..100 like QuickCheck's lists.
"""
import os

import numpy as np
import pytest

from _util import crand

TOL = 1e-10


def O():
    from oracle import oracle
    return oracle


def close(a, b, tol=TOL):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and (a.size == 0 or np.max(np.abs(a - b)) <= tol)


def lengths(seed, count=24, lo=0, hi=100):
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.integers(lo, hi + 1, count)]


def floor_pow2(n):
    return 1 << (int(n).bit_length() - 1)


def floor_5smooth(n):
    best = 1
    p2 = 1
    while p2 <= n:
        p3 = p2
        while p3 <= n:
            p5 = p3
            while p5 <= n:
                best = max(best, p5)
                p5 *= 5
            p3 *= 3
        p2 *= 2
    return best


# ------------------------------------------------------------------ pins
def reference_tables():
    """Tables the reference documents in its source comments (fixture made by
    tests/golden/make_reference_tables.py from the reference tree)."""
    import json
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "reference_tables.json")) as f:
        return json.load(f)


def test_rader_permutation_of_7_matches_reference_comment():
    """Planned.hs:621-643: generator 3, powers 1 3 2 6 4 5, inverse 1 3 2 5 6 4."""
    t = reference_tables()["rader7"]
    assert O().multiplicative_generator(7) == t["generator"] == 3
    perm, rev, inv = O().rader_perms(7)
    assert list(perm + 1) == t["powers"]
    assert list(inv + 1) == t["inverse"]
    assert list(rev) == [perm[(-i) % 6] for i in range(6)]


def test_rader_exponent_matrix_of_7_matches_reference_comment():
    """Planned.hs:621-643: the exponent matrix j*k mod 7, then rows and columns
    permuted by powers of the generator."""
    t = reference_tables()["rader7"]
    assert t["exponent_matrix"] == [[j * k % 7 for k in range(7)] for j in range(7)]
    perm, _, _ = O().rader_perms(7)
    order = [0] + [int(v) + 1 for v in perm]
    assert t["permuted_matrix"] == [[order[a] * order[b] % 7 for b in range(7)] for a in range(7)]


def test_small5_permutation_matches_reference_comment():
    """Private.hs:185-202: transform5's Rader permutation 0 1 2 4 3 (powers of
    the generator 2 mod 5) and the permuted exponent matrix."""
    t = reference_tables()["small5"]
    assert t["exponent_matrix"] == [[j * k % 5 for k in range(5)] for j in range(5)]
    perm, _, _ = O().rader_perms(5)
    order = [0] + [int(v) + 1 for v in perm]
    assert order == t["permutation"]
    assert t["permuted_matrix"] == [[order[a] * order[b] % 5 for b in range(5)] for a in range(5)]


def test_number_theory():
    assert O().fermat_factors(1001) == [(13, 77), (11, 91), (7, 143), (1, 1001)]
    assert O().fermat_factors(25) == [(5, 5), (1, 25)]
    assert O().ceiling_pow2(0) == 1 and O().ceiling_pow2(1) == 1 and O().ceiling_pow2(1025) == 2048
    assert O().ceiling_5smooth(2 * 1000003 - 1) == 2025000
    for n in range(1, 3000):
        c = O().ceiling_5smooth(n)
        assert c >= n and floor_5smooth(c) == c
        assert all(floor_5smooth(m) != m for m in range(n, c))
    for p in [3, 5, 7, 11, 13, 17, 101, 65537, 99991]:
        g = O().multiplicative_generator(p)
        assert len({pow(g, i, p) for i in range(p - 1)}) == p - 1
        assert all(len({pow(c, i, p) for i in range(p - 1)}) < p - 1 for c in range(1, g))


def test_plan_trees_of_benchmark_sizes():
    assert O().plan_string(1024) == "SR1024(SR512(SR256(SR128(SR64(SR32(SR16(SR8(S4))))))))"
    assert O().plan_string(1001).startswith("GT1001(P13(")
    assert O().plan_string(531441).startswith("CT531441(CT729(")
    assert O().plan_string(65537).startswith("P65537(SR65536(")
    assert O().plan_string(1000003).startswith("BL1000003(SR2025000(")
    assert O().plan_string(99991, 0).startswith("P99991(")
    assert O().plan_string(99991, 2).startswith("BL99991(SR262144(")
    assert O().plan_string(99991, 3).startswith("BL99991(SR200000(")


@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 7, 12, 16, 47, 97, 100, 128, 243, 360, 1001, 1024])
def test_known_answer_basis_vector(n):
    """Fourier.hs:367-376: inverse transform of e_k is the basis vector cis(2 pi j k / n)."""
    for k in sorted({k % n for k in (0, 1, n // 2, n - 1)} if n else set()):
        e = np.zeros(n, dtype=np.complex128)
        e[k] = 1
        basis = np.exp(2j * np.pi * (np.arange(n) * k % n) / n)
        assert close(O().planned(e, +1), basis)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 9, 11, 13, 17, 30, 47, 64, 97, 100, 101,
                               210, 243, 256, 1001, 1024, 2310, 4096])
def test_oracle_vs_long_double_dft(n):
    rng = np.random.default_rng(n)
    x = crand(rng, (2, n))
    for sign in (-1, 1):
        ref = O().naive_dft(x, sign)
        for mode in range(4):
            y = O().planned(x, sign, mode)
            assert np.max(np.abs(y - ref)) <= 1e-9 * max(1.0, np.sqrt(n)), (n, sign, mode)


@pytest.mark.parametrize("n", [65536, 65537, 99991, 1 << 20, 3 ** 12, 1001 * 1024])
def test_oracle_vs_numpy_large(n):
    rng = np.random.default_rng(2)
    x = crand(rng, (1, n), "normal")
    y = O().planned(x, -1)
    ref = np.fft.fft(x)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-12


def test_oracle_bluestein_1000003_vs_numpy():
    rng = np.random.default_rng(2)
    x = crand(rng, (1, 1000003), "normal")
    y = O().planned(x, -1)
    ref = np.fft.fft(x)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-9


# ------------------------------------------------------- reference properties
P = O  # readability below


def rand(rng, n, count=1):
    return crand(rng, (n,)) if count == 1 else [crand(rng, (n,)) for _ in range(count)]


@pytest.mark.parametrize("code,name", [(0, "prep dit2"), (1, "prep dif2"), (2, "prep ditSplitRadix"),
                                       (3, "adhoc dit2"), (4, "adhoc ditSplitRadix")])
def test_generic_vs_pow2_variants(code, name):
    """Fourier.hs:300-324 (properties 1-5)."""
    rng = np.random.default_rng(code)
    for L in lengths(code, lo=1):
        n = floor_pow2(L)
        x = rand(rng, n)
        for sign in (-1, 1):
            assert close(P().planned(x, sign), P().variant(x, sign, code)), (name, n)


def test_generic_vs_adhoc_dit235():
    """Fourier.hs:325-329 (property 6)."""
    rng = np.random.default_rng(6)
    for L in lengths(6, lo=1):
        n = floor_5smooth(L)
        x = rand(rng, n)
        for sign in (-1, 1):
            assert close(P().planned(x, sign), P().variant(x, sign, 5))


@pytest.mark.parametrize("prop", ["adhoc chirp2 vs chirp235", "generic vs adhoc auto",
                                  "generic vs adhoc chirp235", "generic vs chirp2", "generic vs chirp235"])
def test_generic_vs_chirps(prop):
    """Fourier.hs:330-354 (properties 7-11)."""
    rng = np.random.default_rng(len(prop))
    for n in lengths(len(prop)):
        x = rand(rng, n)
        for sign in (-1, 1):
            g = P().planned(x, sign)
            if prop == "adhoc chirp2 vs chirp235":
                assert close(P().variant(x, sign, 6), P().variant(x, sign, 7))
            elif prop == "generic vs adhoc auto":
                assert close(g, P().variant(x, sign, 8))
            elif prop == "generic vs adhoc chirp235":
                assert close(g, P().variant(x, sign, 7))
            elif prop == "generic vs chirp2":
                assert close(g, P().planned(x, sign, 2))
            else:
                assert close(g, P().planned(x, sign, 3))


def test_homogeneity_and_additivity():
    """Fourier.hs:355-366 (properties 12-13)."""
    rng = np.random.default_rng(12)
    for n in lengths(12):
        a = rng.uniform(-1, 1) + 1j * rng.uniform(-1, 1)
        x, y = rand(rng, n, 2)
        for sign in (-1, 1):
            assert close(P().planned(a * x, sign), a * P().planned(x, sign))
            assert close(P().planned(x, sign) + P().planned(y, sign), P().planned(x + y, sign))


def test_inverse_double_reverse_conjugate():
    """Fourier.hs:377-402 (properties 15-18)."""
    rng = np.random.default_rng(15)
    for n in lengths(15):
        x = rand(rng, n)
        assert close(x, P().scale_down(P().planned(P().planned(x, 1), -1)))
        for sign in (-1, 1):
            assert close(x, P().cyclic_reverse(P().scale_down(P().planned(P().planned(x, sign), sign))))
            assert close(P().cyclic_reverse(P().planned(x, sign)), P().planned(P().cyclic_reverse(x), sign))
            assert close(np.conj(P().planned(x, sign)), P().planned(np.conj(P().cyclic_reverse(x)), sign))


def test_isometry_unitarity():
    """Fourier.hs:403-417 (properties 19-20)."""
    rng = np.random.default_rng(19)
    for n in lengths(19):
        x, y = rand(rng, n, 2)
        for sign in (-1, 1):
            fx, fy = P().planned(x, sign), P().planned(y, sign)
            assert abs(np.linalg.norm(fx) - np.sqrt(n) * np.linalg.norm(x)) <= TOL
            assert abs(np.sum(fx * np.conj(fy)) - n * np.sum(x * np.conj(y))) <= TOL


def test_convolution_laws():
    """Fourier.hs:418-435 (properties 21-23)."""
    rng = np.random.default_rng(21)
    for n in lengths(21, lo=1):
        x, y, z = rand(rng, n, 3)
        c = P().convolve_cyclic
        assert close(c(x, y), c(y, x))
        assert close(c(c(x, y), z), c(x, c(y, z)))
        assert close(c(x, y + z), c(x, y) + c(x, z))


def test_karatsuba_rec_vs_loop_and_fft():
    """Fourier.hs:436-462 (properties 24-26)."""
    rng = np.random.default_rng(24)
    for n in lengths(24):
        xy = rand(rng, n)
        xr, xi = xy.real, xy.imag
        # 24: recursive vs loop (on the ring of doubles; both exact on integers)
        ir = np.round(xr * 1000).astype(np.int64)
        ii = np.round(xi * 1000).astype(np.int64)
        assert np.array_equal(P().karatsuba(ir, ii, recursive=True), P().karatsuba(ir, ii))
        assert close(P().karatsuba_f64(xr, xi), np.convolve(xr, xi) if n else np.zeros(0))
        # 25: complex karatsuba vs FFT cyclic convolution of the zero-padded signals
        x, y = rand(rng, n, 2)
        rl = max(0, 2 * n - 1)
        if rl:
            px = np.concatenate([x, np.zeros(rl - n)])
            py = np.concatenate([y, np.zeros(rl - n)])
            assert close(P().karatsuba_complex(x, y), P().convolve_cyclic(px, py))
            # 26: cyclic karatsuba vs convolveCyclic of length n
            assert close(P().karatsuba_complex(x, y, cyclic=True), P().convolve_cyclic(x, y))


def test_karatsuba_int_exact_4096():
    """Config 3: Int32 length 4096 in [-1000, 1000], Int64 result, exact."""
    rng = np.random.default_rng(3)
    x = rng.integers(-1000, 1001, 4096)
    y = rng.integers(-1000, 1001, 4096)
    z = P().karatsuba(x, y)
    assert np.array_equal(z, np.convolve(x.astype(np.int64), y.astype(np.int64)))


def self_adjoint(x):
    return x + np.conj(P().cyclic_reverse(x))


def test_real_transforms():
    """Fourier.hs:463-496 (properties 27-30)."""
    rng = np.random.default_rng(27)
    for L in lengths(27):
        n = 2 * L
        x = rand(rng, n)
        xr = x.real.copy()
        assert close(P().to_spectrum(xr), P().planned(xr.astype(np.complex128), -1))
        sa = self_adjoint(x)
        assert close(P().from_spectrum(sa).astype(np.complex128), P().planned(sa, 1))
        if n:
            back = P().from_spectrum(P().to_spectrum(xr)) / n
            assert close(back, xr)
            assert close(P().to_spectrum(P().from_spectrum(sa)) / n, sa)


def test_two_real_spectra():
    """Fourier.hs:497-536 (properties 31-34)."""
    rng = np.random.default_rng(31)
    for L in lengths(31):
        n = 2 * L
        x = rand(rng, n)
        xr, xi = x.real.copy(), x.imag.copy()
        a, b = P().untangle(P().planned(x, -1))
        assert close(P().to_spectrum(xr), a) and close(P().to_spectrum(xi), b)
    for n in lengths(32):
        x = rand(rng, n)
        a, b = P().untangle(P().planned(x, -1))
        assert close(P().planned(x.real.astype(complex), -1), a)
        assert close(P().planned(x.imag.astype(complex), -1), b)
        y = rand(rng, n)
        # entangle then untangle is the identity on coefficient pairs
        e = P().entangle(x, y)
        c = e
        d = np.conj(x - 1j * y)
        bc = np.conj(d)
        assert close((c + bc) / 2, x) and close((c - bc) * (-0.5j), y)
        # twoFromSpectrum: one inverse transform gives both real signals
        xs = self_adjoint(x)
        ys = self_adjoint(1j * x)
        both = P().planned(P().entangle(xs, ys), 1)
        assert close(P().planned(xs, 1), both.real.astype(complex))
        assert close(P().planned(ys, 1), both.imag.astype(complex))


def transform_axis(x, sign, axis):
    x = np.moveaxis(x, axis, -1)
    y = P().planned(np.ascontiguousarray(x), sign)
    return np.moveaxis(y, -1, axis)


def test_transform2d_3d_vs_transposition():
    """Fourier.hs:537-586 (properties 35-38): per-axis transforms commute with
    transposition."""
    rng = np.random.default_rng(35)
    for _ in range(10):
        h, w = int(rng.integers(1, 9)), int(rng.integers(1, 12))
        x = crand(rng, (h, w))
        for sign in (-1, 1):
            t2 = transform_axis(transform_axis(x, sign, 1), sign, 0)
            t2T = transform_axis(transform_axis(x.T, sign, 1), sign, 0)
            assert close(t2.T, t2T)
            ref = np.fft.fft2(x) if sign < 0 else np.fft.ifft2(x) * h * w
            assert close(t2, ref, 1e-9)
        d, h, w = (int(v) for v in rng.integers(1, 6, 3))
        x = crand(rng, (d, h, w))
        t3 = transform_axis(transform_axis(transform_axis(x, -1, 2), -1, 1), -1, 0)
        assert close(t3, np.fft.fftn(x), 1e-9)
