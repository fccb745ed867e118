"""Convolution.Adhoc / Convolution.Preprocessed
(src/Data/Array/Accelerate/Convolution/{Adhoc,Preprocessed}.hs).

`karatsuba(x, y)` is the linear convolution of equal-length rows (length
2L-1 out); `cyclic(conv)` and `complex(conv)` are the reference's
combinators.  int64 (exact, wrap-around like Haskell Int), int32 (widened to
int64 results), float32 and float64 CUDA tensors.  The combinators accept the
convolutions of this module (the C ABI runs the whole composition).
"""
from __future__ import annotations

import torch

from . import _lib, _tensor

_KARA = {torch.int64: "af_karatsuba_i64", torch.int32: "af_karatsuba_i32_i64",
         torch.float32: "af_karatsuba_f32", torch.float64: "af_karatsuba_f64"}
_OUT = {torch.int64: torch.int64, torch.int32: torch.int64, torch.float32: torch.float32,
        torch.float64: torch.float64}
_FOLD = {torch.int64: "af_conv_cyclic_fold_i64", torch.float32: "af_conv_cyclic_fold_f32",
         torch.float64: "af_conv_cyclic_fold_f64"}
_COMPLEX = {torch.int64: "af_conv_complex_i64", torch.float32: "af_conv_complex_f32",
            torch.float64: "af_conv_complex_f64"}


def _rows2(x, y):
    if x.shape != y.shape or x.dtype != y.dtype:
        raise ValueError("both arrays must have the same size and type")
    _tensor.require_cuda(x)
    if x.dtype not in _KARA:
        raise TypeError(f"unsupported element type {x.dtype}")
    x, y = x.contiguous(), y.contiguous()
    L, batch = _tensor.rows(x)
    return x, y, L, batch


def _karatsuba(x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
    x, y, L, batch = _rows2(x, y)
    z = torch.empty(*x.shape[:-1], max(0, 2 * L - 1), dtype=_OUT[x.dtype], device=x.device)
    if z.numel():
        _lib.check(getattr(_lib.load(), _KARA[x.dtype])(x.data_ptr(), y.data_ptr(), z.data_ptr(), L, batch,
                                                        _tensor.stream_ptr()))
    return z


class _Conv:
    """A convolution function of two arrays, tagged with its composition."""

    def __init__(self, kind: str, fn):
        self.kind = kind
        self.fn = fn

    def __call__(self, x, y):
        return self.fn(x, y)


karatsuba = _Conv("karatsuba", _karatsuba)
karatsuba.__doc__ = "Convolution.Adhoc.karatsuba (Convolution/Adhoc.hs:36-63)."


def karatsuba_preprocessed(length: int):
    """Convolution.Preprocessed.karatsuba len (Convolution/Preprocessed.hs:29-56):
    the recursive form; its arithmetic equals the loop form's."""
    def conv(x, y):
        if x.shape[-1] != length:
            raise ValueError("length mismatch")
        return _karatsuba(x, y)
    return _Conv("karatsuba", conv)


def _fold(z: torch.Tensor, L: int) -> torch.Tensor:
    if z.dtype not in _FOLD:
        raise TypeError(f"unsupported element type {z.dtype}")
    batch = z.numel() // max(2 * L - 1, 1) if L else 0
    out = torch.empty(*z.shape[:-1], L, dtype=z.dtype, device=z.device)
    if out.numel():
        _lib.check(getattr(_lib.load(), _FOLD[z.dtype])(z.data_ptr(), out.data_ptr(), L, batch,
                                                        _tensor.stream_ptr()))
    return out


def cyclic(conv: _Conv) -> _Conv:
    """Convolution.Adhoc.cyclic (Convolution/Adhoc.hs:104-111): wrap a linear
    convolution to the input length."""
    if not isinstance(conv, _Conv) or conv.kind != "karatsuba":
        raise TypeError("cyclic takes a karatsuba convolution of this module")

    def fn(x, y):
        z = conv(x, y)
        return _fold(z.contiguous(), int(x.shape[-1]))
    return _Conv("cyclic", fn)


def complex(conv: _Conv):
    """Convolution.Adhoc.complex (Convolution/Adhoc.hs:117-128): a complex
    convolution from three real ones.  Arguments are (re, im) pairs; returns
    a pair."""
    if not isinstance(conv, _Conv) or conv.kind not in ("karatsuba", "cyclic"):
        raise TypeError("complex takes karatsuba or cyclic(karatsuba) of this module")
    cyc = 1 if conv.kind == "cyclic" else 0

    def fn(x, y):
        xr, xi = x
        yr, yi = y
        xr, yr, L, batch = _rows2(xr, yr)
        xi, yi, _, _ = _rows2(xi, yi)
        if xr.dtype == torch.int32:
            xr, xi, yr, yi = (t.to(torch.int64) for t in (xr, xi, yr, yi))
        ol = L if cyc else max(0, 2 * L - 1)
        zr = torch.empty(*xr.shape[:-1], ol, dtype=xr.dtype, device=xr.device)
        zi = torch.empty_like(zr)
        if zr.numel():
            _lib.check(getattr(_lib.load(), _COMPLEX[xr.dtype])(cyc, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(),
                                                                yi.data_ptr(), zr.data_ptr(), zi.data_ptr(), L,
                                                                batch, _tensor.stream_ptr()))
        return zr, zi
    return fn
