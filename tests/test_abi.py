"""CPU-only checks of the C ABI library: it loads, exports every symbol that
include/af.h declares, and its planner reproduces the reference plan trees
(compared with the oracle's restatement of Planned.hs:201-293)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "af.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(af_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    from accelerate_fourier import _lib
    L = _lib.load()
    syms = header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(L, s), s
    # the Python binding declares exactly the header's entry points
    assert set(_lib.SIGNATURES) == set(syms)


def test_version_string():
    from accelerate_fourier import _lib
    assert b"sm_103a" in _lib.load().af_version()


SIZES = list(range(0, 200)) + [243, 1001, 1024, 2025, 4096, 30030, 49995, 65537, 99990, 99991,
                               1 << 20, 3 ** 12, 1001 * 1024, 1000003, 2025000, 123457, 524287]


@pytest.mark.parametrize("mode,algo", [(0, "auto"), (1, "decompose"), (2, "chirp2"), (3, "chirp235")])
def test_plan_trees_match_oracle(mode, algo):
    from accelerate_fourier import _lib
    from oracle import oracle as O
    for n in SIZES:
        assert _lib.plan_tree(n, algo) == O.plan_string(n, mode), (n, algo)


def test_plan_examples():
    """Trees for the sizes the benchmark configurations name."""
    from accelerate_fourier import _lib
    assert _lib.plan_tree(1024) == "SR1024(SR512(SR256(SR128(SR64(SR32(SR16(SR8(S4))))))))"
    assert _lib.plan_tree(1001 * 1024).endswith(
        "GT1001(P13(SR12(SR6(S3))),GT77(P7(SR6(S3)),P11(SR10(S5))))))))))))))")
    assert _lib.plan_tree(65537).startswith("P65537(SR65536(")
    assert _lib.plan_tree(1000003).startswith("BL1000003(SR2025000(")
    assert _lib.plan_tree(99991).startswith("P99991(SR99990(GT49995(P101(")


def test_invalid_arguments_are_reported():
    import ctypes
    from accelerate_fourier import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.af_plan_create(ctypes.byref(h), -1, -1, 0) == _lib.AF_ERR_INVALID
    assert b"negative" in L.af_last_error()
    assert L.af_plan_create(ctypes.byref(h), 16, 0, 0) == _lib.AF_ERR_INVALID
    with pytest.raises(_lib.AfError):
        _lib.plan_tree(12, "prep_dit2")  # not a power of two
    assert L.af_exec_c2c(None, 0, None, None, None, None, 1, None) == _lib.AF_ERR_INVALID


def test_invalid_arguments_of_the_f64_entry_points():
    """Complex Double entry points: the same checks before any device work."""
    import ctypes
    from accelerate_fourier import _lib
    L = _lib.load()
    INV = _lib.AF_ERR_INVALID
    h = ctypes.c_void_p()
    assert L.af_plan_create_f64(ctypes.byref(h), -1, -1, 0) == INV
    assert b"negative" in L.af_last_error()
    assert L.af_plan_create_f64(ctypes.byref(h), 16, 2, 0) == INV
    assert L.af_plan_create_f64(None, 16, -1, 0) == INV
    assert L.af_plan_create_f64(ctypes.byref(h), 1 << 31, -1, 0) == _lib.AF_ERR_UNSUPPORTED
    assert L.af_exec_c2c_f64(None, 0, None, None, None, None, 1, None) == INV
    assert L.af_vjp_c2c_f64(None, 0, None, None, None, None, 1, None) == INV
    assert L.af_exec_c2c_2d_f64(None, None, 0, None, None, None, None, 1, None) == INV
    assert L.af_exec_c2c_3d_f64(None, None, None, 0, None, None, None, None, 1, None) == INV


def test_invalid_arguments_of_the_other_entry_points():
    """Argument checks that fail before any device work (no GPU needed)."""
    from accelerate_fourier import _lib
    L = _lib.load()
    INV = _lib.AF_ERR_INVALID
    # null plans
    assert L.af_exec_c2c_axis(None, 0, None, None, None, None, 1, 1, None) == INV
    assert L.af_exec_c2c_2d(None, None, 0, None, None, None, None, 1, None) == INV
    assert L.af_exec_c2c_3d(None, None, None, 0, None, None, None, None, 1, None) == INV
    assert L.af_to_spectrum(None, None, 0, 0, None, None, 1, None) == INV
    assert L.af_from_spectrum(None, 0, None, None, None, 1, None) == INV
    assert L.af_vjp_to_spectrum(None, 0, None, None, None, 1, None) == INV
    assert L.af_two_to_spectrum(None, None, None, 0, None, None, None, None, 1, None) == INV
    assert L.af_two_from_spectrum(None, 0, None, None, None, None, None, None, 1, None) == INV
    assert L.af_convolve_cyclic(None, 0, None, None, None, None, None, None, 1, None) == INV
    # negative sizes
    assert L.af_karatsuba_i64(None, None, None, -1, 1, None) == INV
    assert L.af_karatsuba_f32(None, None, None, 4, -1, None) == INV
    assert L.af_conv_cyclic_fold_i64(None, None, -2, 1, None) == INV
    assert L.af_untangle_spectra(0, None, None, None, None, None, None, -1, 1, None) == INV
    assert L.af_untangle_spectra_2d(0, None, None, None, None, None, None, 2, -1, 1, None) == INV
    assert L.af_entangle_spectra(0, None, None, None, None, None, None, 4, -1, None) == INV
    assert L.af_cyclic_reverse_2d(0, None, None, None, None, -1, 2, 1, None) == INV
    # null data with work to do
    assert L.af_karatsuba_i32_i64(None, None, None, 8, 1, None) == INV
    assert b"null" in L.af_last_error()
    assert L.af_conv_complex_f64(0, None, None, None, None, None, None, 8, 1, None) == INV
    # empty work is a no-op
    assert L.af_karatsuba_i64(None, None, None, 0, 5, None) == _lib.AF_OK
    assert L.af_untangle_spectra(0, None, None, None, None, None, None, 0, 3, None) == _lib.AF_OK


def test_python_mirror_rejects_host_arrays():
    """No CPU fallback: the transforms refuse arrays that are not on a GPU."""
    torch = pytest.importorskip("torch")
    from accelerate_fourier import _tensor, convolution, real
    x = torch.zeros(8, dtype=torch.complex64)
    with pytest.raises(ValueError):
        _tensor.as_c64(x)
    with pytest.raises(ValueError):
        convolution.karatsuba(torch.zeros(1, 4, dtype=torch.int64), torch.zeros(1, 4, dtype=torch.int64))

    class _Sub:
        length = 4
    with pytest.raises(ValueError):
        real.toSpectrum(_Sub(), torch.zeros(1, 8))
