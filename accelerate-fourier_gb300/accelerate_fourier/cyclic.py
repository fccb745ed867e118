"""Cyclic (src/Data/Array/Accelerate/Cyclic.hs:20-39).

complex64 arrays run in Complex Float, complex128 arrays in Complex Double."""
from __future__ import annotations

import torch

from . import _lib, _tensor


def reverse(x):
    """Cyclic.reverse: out[k] = x[(-k) mod n] along the last axis."""
    double = _tensor.is_double(x)
    x = _tensor.as_complex(x, double)
    n, batch = _tensor.rows(x)
    y = torch.empty_like(x)
    if x.numel():
        _lib.check(_tensor.fn("af_cyclic_reverse", double)(_lib.INTERLEAVED, x.data_ptr(), None, y.data_ptr(),
                                                            None, n, batch, _tensor.stream_ptr()))
    return y


def reverse2d(x):
    """Cyclic.reverse2d: out[y, x] = in[-y mod h, -x mod w] over the last two axes."""
    double = _tensor.is_double(x)
    x = _tensor.as_complex(x, double)
    if x.dim() < 2:
        raise ValueError("reverse2d needs at least two axes")
    h, w = int(x.shape[-2]), int(x.shape[-1])
    batch = x.numel() // max(h * w, 1) if h * w else 0
    y = torch.empty_like(x)
    if x.numel():
        _lib.check(_tensor.fn("af_cyclic_reverse_2d", double)(_lib.INTERLEAVED, x.data_ptr(), None, y.data_ptr(),
                                                               None, h, w, batch, _tensor.stream_ptr()))
    return y
