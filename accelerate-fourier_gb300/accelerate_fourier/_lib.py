"""ctypes binding of libaf (include/af.h).

This is the Python-side equivalent of the `foreign import ccall` stubs a
Haskell caller writes: every function here forwards plain device pointers and
sizes to the C ABI.  There is no fallback: if libaf.so cannot be loaded, every
transform raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

I64 = ctypes.c_int64
PTR = ctypes.c_void_p
INT = ctypes.c_int

AF_OK, AF_ERR_INVALID, AF_ERR_UNSUPPORTED, AF_ERR_CUDA, AF_ERR_ALLOC, AF_ERR_TIMEOUT = range(6)
INTERLEAVED, PLANAR = 0, 1

# af_algo values
ALGO = {
    "auto": 0, "decompose": 1, "chirp2": 2, "chirp235": 3,
    "prep_dit2": 4, "prep_dif2": 5, "prep_splitradix": 6,
    "adhoc_auto": 7, "adhoc_dit2": 8, "adhoc_splitradix": 9, "adhoc_dit235": 10,
    "adhoc_chirp2": 11, "adhoc_chirp235": 12,
}

# name -> (argtypes, restype); every symbol include/af.h declares
SIGNATURES = {
    "af_version": ([], ctypes.c_char_p),
    "af_last_error": ([], ctypes.c_char_p),
    "af_plan_create": ([ctypes.POINTER(PTR), I64, INT, INT], INT),
    "af_plan_destroy": ([PTR], INT),
    "af_plan_describe": ([PTR, ctypes.c_char_p, ctypes.c_size_t], INT),
    "af_plan_tree": ([I64, INT, ctypes.c_char_p, ctypes.c_size_t], INT),
    "af_plan_launches": ([PTR, I64, ctypes.POINTER(I64)], INT),
    "af_exec_c2c": ([PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_plan_create_f64": ([ctypes.POINTER(PTR), I64, INT, INT], INT),
    "af_exec_c2c_f64": ([PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_vjp_c2c_f64": ([PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_exec_c2c_2d_f64": ([PTR, PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_exec_c2c_3d_f64": ([PTR, PTR, PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_exec_c2c_axis_f64": ([PTR, INT, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_scale_down_f64": ([INT, PTR, PTR, I64, I64, PTR], INT),
    "af_cyclic_reverse_f64": ([INT, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_cyclic_reverse_2d_f64": ([INT, PTR, PTR, PTR, PTR, I64, I64, I64, PTR], INT),
    "af_to_spectrum_f64": ([PTR, PTR, INT, INT, PTR, PTR, I64, PTR], INT),
    "af_from_spectrum_f64": ([PTR, INT, PTR, PTR, PTR, I64, PTR], INT),
    "af_vjp_to_spectrum_f64": ([PTR, INT, PTR, PTR, PTR, I64, PTR], INT),
    "af_untangle_spectra_f64": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_untangle_spectra_2d_f64": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, I64, PTR], INT),
    "af_entangle_spectra_f64": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_two_to_spectrum_f64": ([PTR, PTR, PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_two_to_spectrum_2d_f64": ([PTR, PTR, PTR, PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_two_from_spectrum_f64": ([PTR, INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_two_from_spectrum_2d_f64": ([PTR, PTR, INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_convolve_cyclic_f64": ([PTR, INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_vjp_c2c": ([PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_scale_down": ([INT, PTR, PTR, I64, I64, PTR], INT),
    "af_cyclic_reverse": ([INT, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_batch_create": ([ctypes.POINTER(PTR), PTR, I64, INT], INT),
    "af_batch_destroy": ([PTR], INT),
    "af_batch_launches": ([PTR, ctypes.POINTER(I64)], INT),
    "af_batch_exec": ([PTR, PTR, PTR, PTR], INT),
    "af_batch_vjp": ([PTR, PTR, PTR, PTR], INT),
    "af_batch_forward_cotangent": ([PTR, PTR, PTR, PTR, PTR, PTR], INT),
    "af_batch_status": ([PTR, PTR], INT),
    "af_batch_create_tuned": ([ctypes.POINTER(PTR), PTR, I64, INT, ctypes.c_char_p, PTR], INT),
    "af_batch_describe": ([PTR, ctypes.c_char_p, ctypes.c_size_t], INT),
    "af_exec_c2c_noalloc": ([I64, INT, PTR, PTR, I64, PTR], INT),
    "af_cyclic_reverse_2d": ([INT, PTR, PTR, PTR, PTR, I64, I64, I64, PTR], INT),
    "af_exec_c2c_axis": ([PTR, INT, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_exec_c2c_2d": ([PTR, PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_exec_c2c_3d": ([PTR, PTR, PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_to_spectrum": ([PTR, PTR, INT, INT, PTR, PTR, I64, PTR], INT),
    "af_from_spectrum": ([PTR, INT, PTR, PTR, PTR, I64, PTR], INT),
    "af_vjp_to_spectrum": ([PTR, INT, PTR, PTR, PTR, I64, PTR], INT),
    "af_two_to_spectrum": ([PTR, PTR, PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_two_to_spectrum_2d": ([PTR, PTR, PTR, PTR, INT, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_two_from_spectrum": ([PTR, INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_two_from_spectrum_2d": ([PTR, PTR, INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_untangle_spectra": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_untangle_spectra_2d": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, I64, PTR], INT),
    "af_entangle_spectra": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_convolve_cyclic": ([PTR, INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, PTR], INT),
    "af_karatsuba_i64": ([PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_karatsuba_i32_i64": ([PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_karatsuba_f32": ([PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_karatsuba_f64": ([PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_conv_cyclic_fold_i64": ([PTR, PTR, I64, I64, PTR], INT),
    "af_conv_cyclic_fold_f32": ([PTR, PTR, I64, I64, PTR], INT),
    "af_conv_cyclic_fold_f64": ([PTR, PTR, I64, I64, PTR], INT),
    "af_conv_complex_i64": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_conv_complex_f32": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
    "af_conv_complex_f64": ([INT, PTR, PTR, PTR, PTR, PTR, PTR, I64, I64, PTR], INT),
}

FULL, HALF = 0, 1  # af_spectrum


class AfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libaf error {code}: {msg}")
        self.code = code


_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libaf.so (building it first when it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise AfError(AF_ERR_UNSUPPORTED, f"{path} missing; run the build")
            _build.build()
        L = ctypes.CDLL(path)
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
        return L


def check(code: int):
    if code != AF_OK:
        msg = load().af_last_error().decode(errors="replace")
        raise AfError(code, msg)


def plan_tree(n: int, algo: str = "auto") -> str:
    buf = ctypes.create_string_buffer(1 << 16)
    check(load().af_plan_tree(n, ALGO[algo], buf, len(buf)))
    return buf.value.decode()


class Plan:
    """An af_plan: a reference plan tree with its device tables, over
    Complex Float, or Complex Double when `double` is set."""

    def __init__(self, n: int, sign: int, algo: str = "auto", double: bool = False):
        self._h = PTR()
        self.n = int(n)
        self.sign = int(sign)
        self.algo = algo
        self.double = bool(double)
        create = load().af_plan_create_f64 if self.double else load().af_plan_create
        check(create(ctypes.byref(self._h), self.n, self.sign, ALGO[algo]))

    @property
    def handle(self):
        return self._h

    def describe(self) -> str:
        buf = ctypes.create_string_buffer(1 << 16)
        check(load().af_plan_describe(self._h, buf, len(buf)))
        return buf.value.decode()

    def launches(self, batch: int) -> int:
        out = I64()
        check(load().af_plan_launches(self._h, batch, ctypes.byref(out)))
        return out.value

    def exec_ptr(self, src_re, src_im, dst_re, dst_im, batch, stream=0, layout=INTERLEAVED, vjp=False):
        lib = load()
        if self.double:
            f = lib.af_vjp_c2c_f64 if vjp else lib.af_exec_c2c_f64
        else:
            f = lib.af_vjp_c2c if vjp else lib.af_exec_c2c
        check(f(self._h, layout, src_re, src_im, dst_re, dst_im, batch, stream))

    def __del__(self):
        try:
            if self._h:
                load().af_plan_destroy(self._h)
                self._h = PTR()
        except Exception:
            pass


class Batch:
    """An af_batch: many transforms of mixed lengths stored back to back."""

    def __init__(self, lengths, sign: int = -1, tune_cache=None, tune: bool = False, stream=0):
        """tune (or a tune_cache path): the planner choices are timed on the
        device (af_batch_create_tuned) and kept in tune_cache when given."""
        import numpy as np
        self.lengths = np.ascontiguousarray(np.asarray(lengths, dtype=np.int64))
        self.sign = int(sign)
        self.total = int(self.lengths.sum())
        self._h = PTR()
        if tune or tune_cache:
            path = str(tune_cache).encode() if tune_cache else None
            check(load().af_batch_create_tuned(ctypes.byref(self._h), self.lengths.ctypes.data, len(self.lengths),
                                               self.sign, path, stream))
        else:
            check(load().af_batch_create(ctypes.byref(self._h), self.lengths.ctypes.data, len(self.lengths),
                                         self.sign))

    def describe(self) -> dict:
        import json
        buf = ctypes.create_string_buffer(1 << 16)
        check(load().af_batch_describe(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def launches(self) -> int:
        out = I64()
        check(load().af_batch_launches(self._h, ctypes.byref(out)))
        return out.value

    def exec_ptr(self, src, dst, stream=0):
        check(load().af_batch_exec(self._h, src, dst, stream))

    def vjp_ptr(self, src, dst, stream=0):
        check(load().af_batch_vjp(self._h, src, dst, stream))

    def forward_cotangent_ptr(self, x, w, cot, loss, stream=0):
        check(load().af_batch_forward_cotangent(self._h, x, w, cot, loss, stream))

    def status(self, stream=0):
        """Waits for the last call on `stream`; raises AfError (AF_ERR_TIMEOUT)
        when a work item of its persistent launch gave up waiting."""
        check(load().af_batch_status(self._h, stream))

    def __del__(self):
        try:
            if self._h:
                load().af_batch_destroy(self._h)
                self._h = PTR()
        except Exception:
            pass
