"""Cyclic (src/Data/Array/Accelerate/Cyclic.hs:20-39)."""
from __future__ import annotations

from . import _lib, _tensor


def reverse(x):
    """out[k] = x[(-k) mod n] along the last axis."""
    x = _tensor.as_c64(x)
    n, batch = _tensor.rows(x)
    y = torch_empty_like(x)
    if x.numel():
        _lib.check(_lib.load().af_cyclic_reverse(_lib.INTERLEAVED, x.data_ptr(), None, y.data_ptr(), None,
                                                 n, batch, _tensor.stream_ptr()))
    return y


def torch_empty_like(x):
    import torch
    return torch.empty_like(x)
