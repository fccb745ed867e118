"""Fourier.Utility (src/Data/Array/Accelerate/Fourier/Utility.hs:17-26)."""
from __future__ import annotations

from . import _lib, _tensor


def scaleDown(x):
    """Multiply by 1/length along the last axis; returns a new array."""
    if isinstance(x, tuple):
        re, im = (t.contiguous().clone() for t in x)
        _tensor.require_cuda(re)
        n, batch = _tensor.rows(re)
        _lib.check(_lib.load().af_scale_down(_lib.PLANAR, re.data_ptr(), im.data_ptr(), n, batch,
                                             _tensor.stream_ptr()))
        return re, im
    y = _tensor.as_c64(x).clone()
    n, batch = _tensor.rows(y)
    if y.numel():
        _lib.check(_lib.load().af_scale_down(_lib.INTERLEAVED, y.data_ptr(), None, n, batch,
                                             _tensor.stream_ptr()))
    return y
