"""Fourier.Utility (src/Data/Array/Accelerate/Fourier/Utility.hs:17-26)."""
from __future__ import annotations

from . import _lib, _tensor


def scaleDown(x):
    """Multiply by 1/length along the last axis; returns a new array.
    complex128 (or float64 planes) runs in Complex Double."""
    double = _tensor.is_double(x)
    f = _tensor.fn("af_scale_down", double)
    if isinstance(x, tuple):
        re, im = (t.contiguous().to(_tensor.rdtype(double)).clone() for t in x)
        _tensor.require_cuda(re)
        n, batch = _tensor.rows(re)
        if re.numel():
            _lib.check(f(_lib.PLANAR, re.data_ptr(), im.data_ptr(), n, batch, _tensor.stream_ptr()))
        return re, im
    y = _tensor.as_complex(x, double).clone()
    n, batch = _tensor.rows(y)
    if y.numel():
        _lib.check(f(_lib.INTERLEAVED, y.data_ptr(), None, n, batch, _tensor.stream_ptr()))
    return y
