"""CPU checks of every launch program's memory addressing (no GPU needed).

The library builds its programs in a dry-run mode and replays every global
load and store address of the tile and map kernels against the buffer sizes;
every output element must be written exactly once, which also proves the
Good-Thomas CRT maps and the Rader permutations are bijections.  These checks
run before any program reaches a GPU.
"""
import ctypes

import numpy as np
import pytest


def _lib():
    from accelerate_fourier import _lib
    L = _lib.load()
    for sfx in ("", "_f64"):
        f = getattr(L, "afx_check_plan" + sfx)
        f.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_char_p, ctypes.c_size_t]
        f.restype = ctypes.c_int
        f = getattr(L, "afx_check_axis" + sfx)
        f.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_char_p,
                      ctypes.c_size_t]
        f.restype = ctypes.c_int
    L.afx_check_batch.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
    L.afx_check_batch.restype = ctypes.c_int
    return L, _lib.ALGO


def check_plan(n, sign=-1, algo="auto", batch=1, double=False):
    """double: the programs of the Complex Double engine (smaller tiles, so
    other splits), checked by its own build of the checker."""
    L, ALGO = _lib()
    msg = ctypes.create_string_buffer(1024)
    f = L.afx_check_plan_f64 if double else L.afx_check_plan
    rc = f(n, sign, ALGO[algo], batch, msg, len(msg))
    assert rc == 0, (n, algo, batch, double, msg.value.decode())


def check_axis(n, outer, inner, sign=-1, algo="auto", double=False):
    L, ALGO = _lib()
    msg = ctypes.create_string_buffer(1024)
    f = L.afx_check_axis_f64 if double else L.afx_check_axis
    rc = f(n, sign, ALGO[algo], outer, inner, msg, len(msg))
    assert rc == 0, (n, outer, inner, double, msg.value.decode())


def check_batch(sizes, sign=-1):
    L, _ = _lib()
    a = np.ascontiguousarray(np.asarray(sizes, dtype=np.int64))
    msg = ctypes.create_string_buffer(1024)
    rc = L.afx_check_batch(a.ctypes.data, len(a), sign, msg, len(msg))
    assert rc == 0, msg.value.decode()


# single tiles, four-step, two-pass Good-Thomas (plain and Rader factors),
# Rader convolutions (smooth and zero-padded), Bluestein, peel schemes, the
# generic recursive lowering
SIZES = ([1, 2, 3, 4, 5, 7, 8, 13, 16, 17, 47, 83, 100, 257, 307, 1001, 1009, 1031, 4096, 4099, 8192,
          12288, 12289, 13007, 15015, 16384, 16385, 19683, 20000, 26701, 30011, 49999, 65536, 65537,
          11326, 36316, 47978, 39729, 2738, 99991, 1 << 20, 3 ** 12, 1001 * 1024]
         + list(range(101, 140)))


@pytest.mark.parametrize("n", SIZES)
def test_plan_addressing(n):
    check_plan(n, -1, "auto", 1)
    if n <= 20000:
        check_plan(n, 1, "auto", 3)


@pytest.mark.parametrize("algo", ["decompose", "chirp2", "chirp235", "adhoc_auto", "adhoc_chirp2",
                                  "adhoc_chirp235"])
def test_algorithm_addressing(algo):
    for n in [2, 3, 17, 100, 1009, 4099, 16385, 30011]:
        check_plan(n, -1, algo, 2)


def test_large_sizes_addressing():
    for n in [1000003, 1 << 21, 1 << 22]:
        check_plan(n, -1, "auto", 1)


def test_batch_addressing_mixed():
    check_batch(SIZES)
    check_batch([0, 64, 64, 0, 1000, 64, 65537, 65537, 3], +1)


def test_batch_addressing_benchmark_workload():
    import bench
    check_batch(bench.workload_sizes())


# strided-axis programs of the 2-D/3-D transforms: single tiles with
# line-fast loads, multi-pass schemes through copies (outer > 1) or directly
@pytest.mark.parametrize("n", [1, 2, 3, 16, 17, 100, 257, 1001, 4096, 4099, 16384, 30011, 65537, 99991])
def test_axis_addressing(n):
    for outer, inner in [(1, 1), (1, 7), (3, 5), (2, 64), (1, 256)]:
        if n * outer * inner <= (1 << 23):
            check_axis(n, outer, inner)
    check_axis(n, 2, 3, sign=1)


# Complex Double programs: tiles hold at most 6200 elements, so lengths
# between that and 13000 take the multi-pass schemes in FP64
@pytest.mark.parametrize("n", SIZES + [6144, 6200, 6201, 6250, 7776, 9973, 10007, 12289 * 2])
def test_plan_addressing_f64(n):
    check_plan(n, -1, "auto", 1, double=True)
    if n <= 20000:
        check_plan(n, 1, "auto", 3, double=True)


def test_algorithm_addressing_f64():
    for algo in ["decompose", "chirp2", "chirp235", "adhoc_auto"]:
        for n in [2, 3, 17, 100, 1009, 4099, 16385, 30011]:
            check_plan(n, -1, algo, 2, double=True)


@pytest.mark.parametrize("n", [1, 16, 17, 100, 1001, 4096, 6250, 16384, 30011, 65537])
def test_axis_addressing_f64(n):
    for outer, inner in [(1, 1), (1, 7), (3, 5), (2, 64)]:
        if n * outer * inner <= (1 << 22):
            check_axis(n, outer, inner, double=True)


def describe_batch(sizes, double=False, which=0):
    """Dry-run text of a batch program: one line per launch with its tiles."""
    from accelerate_fourier import _lib
    L = _lib.load()
    f = L.afx_describe_batch_f64 if double else L.afx_describe_batch
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
    f.restype = ctypes.c_int
    a = np.ascontiguousarray(np.asarray(sizes, dtype=np.int64))
    buf = ctypes.create_string_buffer(1 << 16)
    assert f(a.ctypes.data, len(a), -1, which, buf, len(buf)) == 0, buf.value.decode()
    return buf.value.decode()


def test_f64_tiles_hold_half_the_elements():
    """A Complex Double tile holds at most 6200 elements (twice the shared
    memory per element): 8192 and 7776 are single tiles in FP32 and four-step
    transforms in FP64; 4096 is a single tile in both."""
    f32, f64 = describe_batch([8192, 7776, 4096]), describe_batch([8192, 7776, 4096], double=True)
    for n in (8192, 7776):
        assert f"n{n} s{n} " in f32
        assert f"n{n} s{n} " not in f64
    assert "n4096 s4096 " in f32 and "n4096 s4096 " in f64
    # the FP64 four-step passes: columns with the twiddle on the store, then rows
    assert " tw lf " in f64 and " tw lf " not in f32
