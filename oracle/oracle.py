"""ctypes wrapper of the oracle -- TEST INFRASTRUCTURE ONLY.

The oracle is a CPU restatement of accelerate-fourier's algorithms (C++ in
``af_oracle.cpp``).  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg may import this module; the CUDA library never
does.  Parity with a Haskell build of the reference is unpinned at the bit
level (no Haskell toolchain); the oracle itself is pinned by the reference's
known-answer test, the permutation tables in the reference's source comments,
the reference's 38 properties and a long-double naive DFT (see ``tests/``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_SRC = os.path.join(_HERE, "af_oracle.cpp")
_lock = threading.Lock()
_lib = None

I64 = ctypes.c_longlong
PTR = ctypes.c_void_p

# plan modes (Planned.hs:103-130,704-729)
AUTO, DECOMPOSE, CHIRP2, CHIRP235 = 0, 1, 2, 3
# variant algorithms (Preprocessed.hs / Adhoc.hs)
PREP_DIT2, PREP_DIF2, PREP_SPLITRADIX = 0, 1, 2
ADHOC_DIT2, ADHOC_SPLITRADIX, ADHOC_DIT235 = 3, 4, 5
ADHOC_CHIRP2, ADHOC_CHIRP235, ADHOC_AUTO = 6, 7, 8


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    with _lock:
        stale = (not os.path.exists(_LIB_PATH)
                 or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC))
        if force or stale:
            subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        sig = {
            "or_version": ([], ctypes.c_int),
            "or_max_threads": ([], ctypes.c_int),
            "or_ceiling_pow2": ([I64], I64),
            "or_ceiling_5smooth": ([I64], I64),
            "or_adhoc_ceiling_5smooth": ([I64], I64),
            "or_multiplicative_generator": ([I64], I64),
            "or_modular_power": ([I64, I64, I64], I64),
            "or_fermat_factors": ([I64, PTR, ctypes.c_int], ctypes.c_int),
            "or_plan_string": ([ctypes.c_int, I64, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
            "or_plan_count_primes": ([I64], ctypes.c_int),
            "or_rader_perms": ([I64, PTR, PTR, PTR], None),
            "or_skew_grid": ([I64, I64, PTR, PTR, PTR], None),
            "or_handle_create": ([ctypes.c_int, ctypes.c_int, I64], PTR),
            "or_handle_destroy": ([PTR], None),
            "or_handle_exec_f64": ([PTR, I64, PTR, PTR, ctypes.c_int], None),
            "or_handle_exec_f32": ([PTR, I64, PTR, PTR, ctypes.c_int], None),
            "or_planned": ([ctypes.c_int, ctypes.c_int, I64, I64, PTR, PTR], None),
            "or_variant": ([ctypes.c_int, ctypes.c_int, I64, I64, PTR, PTR], None),
            "or_naive_dft": ([ctypes.c_int, I64, I64, PTR, PTR], None),
            "or_scale_down": ([I64, I64, PTR], None),
            "or_cyclic_reverse": ([I64, I64, PTR, PTR], None),
            "or_to_spectrum": ([I64, I64, PTR, PTR], None),
            "or_from_spectrum": ([I64, I64, PTR, PTR], None),
            "or_untangle": ([I64, I64, PTR, PTR, PTR], None),
            "or_entangle": ([I64, I64, PTR, PTR, PTR], None),
            "or_convolve_cyclic": ([I64, I64, PTR, PTR, PTR], None),
            "or_karatsuba_loop_i64": ([I64, I64, PTR, PTR, PTR], None),
            "or_karatsuba_rec_i64": ([I64, I64, PTR, PTR, PTR], None),
            "or_karatsuba_loop_f64": ([I64, I64, PTR, PTR, PTR], None),
            "or_karatsuba_loop_f32": ([I64, I64, PTR, PTR, PTR], None),
            "or_cyclic_fold_i64": ([I64, I64, PTR, PTR], None),
            "or_mixed_create": ([ctypes.c_int, ctypes.c_int, I64, PTR], PTR),
            "or_mixed_destroy": ([PTR], None),
            "or_mixed_exec_f32": ([PTR, I64, I64, PTR, PTR, PTR, ctypes.c_int], None),
            "or_mixed_exec_f64": ([PTR, I64, I64, PTR, PTR, PTR, ctypes.c_int], None),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c128(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128))


def _rows(x: np.ndarray):
    n = x.shape[-1] if x.ndim else 0
    batch = int(np.prod(x.shape[:-1])) if x.ndim > 1 else 1
    return n, batch


# ----------------------------------------------------------------- number theory
def ceiling_pow2(n: int) -> int:
    return lib().or_ceiling_pow2(n)


def ceiling_5smooth(n: int) -> int:
    return lib().or_ceiling_5smooth(n)


def adhoc_ceiling_5smooth(n: int) -> int:
    return lib().or_adhoc_ceiling_5smooth(n)


def multiplicative_generator(p: int) -> int:
    return lib().or_multiplicative_generator(p)


def fermat_factors(n: int):
    buf = np.zeros(2 * 4096, dtype=np.int64)
    cnt = lib().or_fermat_factors(n, _p(buf), 4096)
    return [(int(buf[2 * i]), int(buf[2 * i + 1])) for i in range(min(cnt, 4096))]


def plan_string(n: int, mode: int = AUTO) -> str:
    buf = ctypes.create_string_buffer(1 << 16)
    r = lib().or_plan_string(mode, n, buf, len(buf))
    if r < 0:
        raise ValueError("plan string too long")
    return buf.value.decode()


def rader_perms(p: int):
    perm = np.zeros(p - 1, dtype=np.int64)
    rev = np.zeros(p - 1, dtype=np.int64)
    inv = np.zeros(p - 1, dtype=np.int64)
    lib().or_rader_perms(p, _p(perm), _p(rev), _p(inv))
    return perm, rev, inv


def skew_grid(n: int, m: int):
    fwd = np.zeros(n * m, dtype=np.int64)
    iq = np.zeros(n * m, dtype=np.int64)
    ip = np.zeros(n * m, dtype=np.int64)
    lib().or_skew_grid(n, m, _p(fwd), _p(iq), _p(ip))
    return fwd.reshape(m, n), iq, ip


# ------------------------------------------------------------------ transforms
def planned(x, sign: int, mode: int = AUTO) -> np.ndarray:
    """Planned.transform (mode AUTO), transformDecompose, transformChirp2/235.
    Transforms the last axis; leading axes are the batch."""
    x = _c128(x)
    out = np.empty_like(x)
    n, batch = _rows(x)
    if x.size:
        lib().or_planned(mode, sign, n, batch, _p(x), _p(out))
    return out


def variant(x, sign: int, algo: int) -> np.ndarray:
    """Preprocessed.dit2/dif2/ditSplitRadix and Adhoc.* transforms."""
    x = _c128(x)
    out = np.empty_like(x)
    n, batch = _rows(x)
    if x.size:
        lib().or_variant(algo, sign, n, batch, _p(x), _p(out))
    return out


def naive_dft(x, sign: int) -> np.ndarray:
    x = _c128(x)
    out = np.empty_like(x)
    n, batch = _rows(x)
    if x.size:
        lib().or_naive_dft(sign, n, batch, _p(x), _p(out))
    return out


def scale_down(x) -> np.ndarray:
    x = _c128(x).copy()
    n, batch = _rows(x)
    if x.size:
        lib().or_scale_down(n, batch, _p(x))
    return x


def cyclic_reverse(x) -> np.ndarray:
    x = _c128(x)
    out = np.empty_like(x)
    n, batch = _rows(x)
    if x.size:
        lib().or_cyclic_reverse(n, batch, _p(x), _p(out))
    return out


def to_spectrum(x) -> np.ndarray:
    """Real.toSpectrum (Planned.transform forward (n/2)); x real, even length."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    n, batch = _rows(x)
    out = np.empty(x.shape, dtype=np.complex128)
    if x.size:
        lib().or_to_spectrum(n, batch, _p(x), _p(out))
    return out


def from_spectrum(spec) -> np.ndarray:
    """Real.fromSpectrum (Planned.transform inverse (n/2)); unscaled."""
    spec = _c128(spec)
    n, batch = _rows(spec)
    out = np.empty(spec.shape, dtype=np.float64)
    if spec.size:
        lib().or_from_spectrum(n, batch, _p(spec), _p(out))
    return out


def untangle(spec):
    spec = _c128(spec)
    n, batch = _rows(spec)
    a = np.empty_like(spec)
    b = np.empty_like(spec)
    if spec.size:
        lib().or_untangle(n, batch, _p(spec), _p(a), _p(b))
    return a, b


def entangle(c, d) -> np.ndarray:
    c = _c128(c)
    d = _c128(d)
    out = np.empty_like(c)
    n, batch = _rows(c)
    if c.size:
        lib().or_entangle(n, batch, _p(c), _p(d), _p(out))
    return out


def convolve_cyclic(x, y) -> np.ndarray:
    x = _c128(x)
    y = _c128(y)
    out = np.empty_like(x)
    n, batch = _rows(x)
    if x.size:
        lib().or_convolve_cyclic(n, batch, _p(x), _p(y), _p(out))
    return out


def karatsuba(x, y, recursive: bool = False) -> np.ndarray:
    """Convolution.Adhoc.karatsuba (loop) or Convolution.Preprocessed.karatsuba
    over int64 rows; returns rows of length max 0 (2L-1)."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.int64))
    y = np.ascontiguousarray(np.asarray(y, dtype=np.int64))
    L, batch = _rows(x)
    zl = max(0, 2 * L - 1)
    out = np.zeros(x.shape[:-1] + (zl,), dtype=np.int64)
    if x.size:
        f = lib().or_karatsuba_rec_i64 if recursive else lib().or_karatsuba_loop_i64
        f(L, batch, _p(x), _p(y), _p(out))
    return out


def karatsuba_f64(x, y) -> np.ndarray:
    """Convolution.Adhoc.karatsuba over Double rows (loop form)."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    y = np.ascontiguousarray(np.asarray(y, dtype=np.float64))
    L, batch = _rows(x)
    out = np.zeros(x.shape[:-1] + (max(0, 2 * L - 1),), dtype=np.float64)
    if x.size:
        lib().or_karatsuba_loop_f64(L, batch, _p(x), _p(y), _p(out))
    return out


def karatsuba_f32(x, y) -> np.ndarray:
    """Convolution.Adhoc.karatsuba over Float rows (loop form, float arithmetic)."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    y = np.ascontiguousarray(np.asarray(y, dtype=np.float32))
    L, batch = _rows(x)
    out = np.zeros(x.shape[:-1] + (max(0, 2 * L - 1),), dtype=np.float32)
    if x.size:
        lib().or_karatsuba_loop_f32(L, batch, _p(x), _p(y), _p(out))
    return out


def karatsuba_complex(x, y, cyclic: bool = False) -> np.ndarray:
    """Convolution.Adhoc.complex (3 real products, Convolution/Adhoc.hs:118-133)
    of karatsuba, optionally through Convolution.Adhoc.cyclic (104-111)."""
    x = _c128(x)
    y = _c128(y)
    xr, xi, yr, yi = x.real.copy(), x.imag.copy(), y.real.copy(), y.imag.copy()
    xm, ym = xr + xi, yr + yi

    def conv(a, b):
        z = karatsuba_f64(a, b)
        if cyclic:
            L = a.shape[-1]
            if L == 0:
                return z
            w = z[..., :L].copy()
            w[..., :L - 1] += z[..., L:]
            return w
        return z
    rr, ii, mm = conv(xr, yr), conv(xi, yi), conv(xm, ym)
    return (rr - ii) + 1j * (mm - (rr + ii))


def cyclic_fold(z, L: int) -> np.ndarray:
    """Convolution.Adhoc.cyclic on an already computed linear convolution."""
    z = np.ascontiguousarray(np.asarray(z, dtype=np.int64))
    batch = int(np.prod(z.shape[:-1])) if z.ndim > 1 else 1
    out = np.zeros(z.shape[:-1] + (L,), dtype=np.int64)
    if L:
        lib().or_cyclic_fold_i64(L, batch, _p(z), _p(out))
    return out


class Handle:
    """Plan + cache built once (Planned.transform sign len), executed many times."""

    def __init__(self, n: int, sign: int, mode: int = AUTO):
        self.n = n
        self.h = lib().or_handle_create(mode, sign, n)

    def exec_f32(self, x: np.ndarray, threads: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.complex64)
        out = np.empty_like(x)
        lib().or_handle_exec_f32(self.h, x.size // self.n, _p(x), _p(out), threads)
        return out

    def exec_f64(self, x: np.ndarray, threads: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.complex128)
        out = np.empty_like(x)
        lib().or_handle_exec_f64(self.h, x.size // self.n, _p(x), _p(out), threads)
        return out

    def __del__(self):
        try:
            lib().or_handle_destroy(self.h)
        except Exception:
            pass


class Mixed:
    """Many transforms of different lengths stored back to back."""

    def __init__(self, ns, sign: int, mode: int = AUTO):
        self.ns = np.ascontiguousarray(np.asarray(ns, dtype=np.int64))
        self.offsets = np.ascontiguousarray(
            np.concatenate([[0], np.cumsum(self.ns)[:-1]]).astype(np.int64))
        self.total = int(self.ns.sum())
        self.h = lib().or_mixed_create(mode, sign, len(self.ns), _p(self.ns))

    def exec_f32(self, x, out, first=0, count=None, threads=0):
        count = len(self.ns) - first if count is None else count
        lib().or_mixed_exec_f32(self.h, first, count, _p(self.offsets), _p(x), _p(out), threads)

    def exec_f64(self, x, out, first=0, count=None, threads=0):
        count = len(self.ns) - first if count is None else count
        lib().or_mixed_exec_f64(self.h, first, count, _p(self.offsets), _p(x), _p(out), threads)

    def __del__(self):
        try:
            lib().or_mixed_destroy(self.h)
        except Exception:
            pass
