"""Fourier.Real (src/Data/Array/Accelerate/Fourier/Real.hs).

Real transforms through complex transforms.  `subTrans` arguments are
Transform objects (planned.transform & co.), like the reference's
`Transform (sh:.Int) (Complex a)` arguments: toSpectrum/fromSpectrum take
the transform of half the real length, the two-signal functions take a
transform of the full length (or a 2-D transform for the *2d forms).
Complex results are complex64 CUDA tensors; pairs of real arrays are tuples
of float32 tensors (Accelerate's `Array sh (a, a)`).  float64 / complex128
arguments run in Complex Double (the reference functions are polymorphic over
`A.RealFloat a`) and give float64 / complex128 results.
"""
from __future__ import annotations

import torch

from . import _lib, _tensor


def _real_rows(x: torch.Tensor):
    _tensor.require_cuda(x)
    double = x.dtype == torch.float64
    x = x.contiguous().to(_tensor.rdtype(double))
    n, batch = _tensor.rows(x)
    return x, n, batch, double


def _complex_rows(s):
    double = _tensor.is_double(s)
    if isinstance(s, tuple):
        re, im = (t.contiguous().to(_tensor.rdtype(double)) for t in s)
        _tensor.require_cuda(re)
        n, batch = _tensor.rows(re)
        return (re, im), n, batch, _lib.PLANAR, double
    s = _tensor.as_complex(s, double)
    n, batch = _tensor.rows(s)
    return s, n, batch, _lib.INTERLEAVED, double


def _ptrs(s, layout):
    if layout == _lib.PLANAR:
        return s[0].data_ptr(), s[1].data_ptr()
    return s.data_ptr(), None


def toSpectrum(subTrans, x: torch.Tensor, half: bool = False) -> torch.Tensor:
    """Real.toSpectrum (Real.hs:49-70): N reals -> N complex bins (the full
    spectrum); half=True keeps bins 0..N/2 only."""
    x, n, batch, double = _real_rows(x)
    if n % 2:
        raise ValueError("toSpectrum needs an even length")
    if n // 2 != subTrans.length:
        raise ValueError(f"sub-transform length {subTrans.length} is not half of {n}")
    nout = n // 2 + 1 if half else n
    out = torch.empty(*x.shape[:-1], nout, dtype=_tensor.cdtype(double), device=x.device)
    if x.numel():
        _lib.check(_tensor.fn("af_to_spectrum", double)(subTrans.plan_of(double).handle, x.data_ptr(),
                                                         _lib.HALF if half else _lib.FULL, _lib.INTERLEAVED,
                                                         out.data_ptr(), None, batch, _tensor.stream_ptr()))
    return out


def _from(name, subTrans, spec):
    s, n, batch, layout, double = _complex_rows(spec)
    if n % 2 or n // 2 != subTrans.length:
        raise ValueError(f"sub-transform length {subTrans.length} is not half of {n}")
    ref = s[0] if layout == _lib.PLANAR else s
    out = torch.empty(*ref.shape[:-1], n, dtype=_tensor.rdtype(double), device=ref.device)
    if out.numel():
        re, im = _ptrs(s, layout)
        _lib.check(_tensor.fn(name, double)(subTrans.plan_of(double).handle, layout, re, im, out.data_ptr(), batch,
                                            _tensor.stream_ptr()))
    return out


def fromSpectrum(subTrans, spec) -> torch.Tensor:
    """Real.fromSpectrum (Real.hs:92-108): a self-adjoint spectrum of N bins
    -> N reals (unscaled)."""
    return _from("af_from_spectrum", subTrans, spec)


def toSpectrum_vjp(subTrans, cotangent) -> torch.Tensor:
    """Adjoint of toSpectrum (forward subTrans): Re(DFT^H cot) as N reals."""
    return _from("af_vjp_to_spectrum", subTrans, cotangent)


def _pair(fg):
    double = fg[0].dtype == torch.float64
    f, g = (t.contiguous().to(_tensor.rdtype(double)) for t in fg)
    _tensor.require_cuda(f)
    if f.shape != g.shape:
        raise ValueError("the two real arrays must have one shape")
    return f, g, double


def twoToSpectrum(subTrans, fg):
    """Real.twoToSpectrum (Real.hs:129-137): two real arrays through one
    complex transform; returns their two spectra."""
    f, g, double = _pair(fg)
    n, batch = _tensor.rows(f)
    if n != subTrans.length:
        raise ValueError("length mismatch")
    a = torch.empty(f.shape, dtype=_tensor.cdtype(double), device=f.device)
    b = torch.empty_like(a)
    if f.numel():
        _lib.check(_tensor.fn("af_two_to_spectrum", double)(subTrans.plan_of(double).handle, f.data_ptr(),
                                                             g.data_ptr(), _lib.INTERLEAVED, a.data_ptr(), None,
                                                             b.data_ptr(), None, batch, _tensor.stream_ptr()))
    return a, b


def twoToSpectrum2d(subTrans2d, fg):
    """Real.twoToSpectrum2d (Real.hs:139-145); subTrans2d is a Transform2d."""
    f, g, double = _pair(fg)
    p0, p1, batch = subTrans2d.shape_check(f.shape, double)
    a = torch.empty(f.shape, dtype=_tensor.cdtype(double), device=f.device)
    b = torch.empty_like(a)
    if f.numel():
        _lib.check(_tensor.fn("af_two_to_spectrum_2d", double)(p0.handle, p1.handle, f.data_ptr(), g.data_ptr(),
                                                                _lib.INTERLEAVED, a.data_ptr(), None, b.data_ptr(),
                                                                None, batch, _tensor.stream_ptr()))
    return a, b


def untangleSpectra(spec):
    """Real.untangleSpectra (Real.hs:168-172)."""
    double = _tensor.is_double(spec)
    s = _tensor.as_complex(spec, double)
    n, batch = _tensor.rows(s)
    a, b = torch.empty_like(s), torch.empty_like(s)
    if s.numel():
        _lib.check(_tensor.fn("af_untangle_spectra", double)(_lib.INTERLEAVED, s.data_ptr(), None, a.data_ptr(),
                                                              None, b.data_ptr(), None, n, batch,
                                                              _tensor.stream_ptr()))
    return a, b


def untangleSpectra2d(spec):
    """Real.untangleSpectra2d (Real.hs:174-179)."""
    double = _tensor.is_double(spec)
    s = _tensor.as_complex(spec, double)
    h, w = int(s.shape[-2]), int(s.shape[-1])
    batch = s.numel() // max(h * w, 1) if h * w else 0
    a, b = torch.empty_like(s), torch.empty_like(s)
    if s.numel():
        _lib.check(_tensor.fn("af_untangle_spectra_2d", double)(_lib.INTERLEAVED, s.data_ptr(), None,
                                                                 a.data_ptr(), None, b.data_ptr(), None, h, w,
                                                                 batch, _tensor.stream_ptr()))
    return a, b


def entangleSpectra(cd):
    """Real.entangleSpectra (Real.hs:207-211): c + i d."""
    double = _tensor.is_double(cd[0])
    c, d = (_tensor.as_complex(t, double) for t in cd)
    if c.shape != d.shape:
        raise ValueError("the two spectra must have one shape")
    n, batch = _tensor.rows(c)
    out = torch.empty_like(c)
    if c.numel():
        _lib.check(_tensor.fn("af_entangle_spectra", double)(_lib.INTERLEAVED, c.data_ptr(), None, d.data_ptr(),
                                                              None, out.data_ptr(), None, n, batch,
                                                              _tensor.stream_ptr()))
    return out


entangleSpectra2d = entangleSpectra  # element-wise (Real.hs:213-217)


def twoFromSpectrum(subTrans, ab):
    """Real.twoFromSpectrum (Real.hs:189-195): entangle, transform, split."""
    double = _tensor.is_double(ab[0])
    a, b = (_tensor.as_complex(t, double) for t in ab)
    n, batch = _tensor.rows(a)
    if n != subTrans.length:
        raise ValueError("length mismatch")
    f = torch.empty(a.shape, dtype=_tensor.rdtype(double), device=a.device)
    g = torch.empty_like(f)
    if a.numel():
        _lib.check(_tensor.fn("af_two_from_spectrum", double)(subTrans.plan_of(double).handle, _lib.INTERLEAVED,
                                                               a.data_ptr(), None, b.data_ptr(), None, f.data_ptr(),
                                                               g.data_ptr(), batch, _tensor.stream_ptr()))
    return f, g


def twoFromSpectrum2d(subTrans2d, ab):
    """Real.twoFromSpectrum2d (Real.hs:197-203)."""
    double = _tensor.is_double(ab[0])
    a, b = (_tensor.as_complex(t, double) for t in ab)
    p0, p1, batch = subTrans2d.shape_check(a.shape, double)
    f = torch.empty(a.shape, dtype=_tensor.rdtype(double), device=a.device)
    g = torch.empty_like(f)
    if a.numel():
        _lib.check(_tensor.fn("af_two_from_spectrum_2d", double)(p0.handle, p1.handle, _lib.INTERLEAVED,
                                                                  a.data_ptr(), None, b.data_ptr(), None,
                                                                  f.data_ptr(), g.data_ptr(), batch,
                                                                  _tensor.stream_ptr()))
    return f, g


def untangleCoefficient(a: complex, b: complex):
    """Real.untangleCoefficient (Real.hs:181-186) on scalars."""
    bc = b.conjugate()
    return (a + bc) / 2, (a - bc) * (-1j / 2)


def entangleCoefficient(c: complex, d: complex):
    """Real.entangleCoefficient (Real.hs:231-236) on scalars."""
    di = d * 1j
    return c + di, (c - di).conjugate()
