"""Fourier.Adhoc (src/Data/Array/Accelerate/Fourier/Adhoc.hs).

The reference builds these transforms without knowing the length on the
host; here the length is read from the array when the function is applied
and the plan is cached per length."""
from __future__ import annotations

from . import _lib
from .planned import Transform
from .sign import check, forward, inverse  # noqa: F401


def _apply(algo: str, sign: int, x):
    n = (x[0] if isinstance(x, tuple) else x).shape[-1]
    return Transform(check(sign), n, algo)(x)


def transform(sign: int, x):
    """Adhoc.transform (Adhoc.hs:74-84): split-radix / dit235 / chirp235 by size."""
    return _apply("adhoc_auto", sign, x)


def ditSplitRadix(sign: int, x):
    """Adhoc.ditSplitRadix (Adhoc.hs:101-108)."""
    return _apply("adhoc_splitradix", sign, x)


def dit2(sign: int, x):
    """Adhoc.dit2 (Adhoc.hs:138-153)."""
    return _apply("adhoc_dit2", sign, x)


def dit235(sign: int, x):
    """Adhoc.dit235 (Adhoc.hs:171-204)."""
    return _apply("adhoc_dit235", sign, x)


def transformChirp2(sign: int, x):
    """Adhoc.transformChirp2 (Adhoc.hs:342-350)."""
    return _apply("adhoc_chirp2", sign, x)


def transformChirp235(sign: int, x):
    """Adhoc.transformChirp235 (Adhoc.hs:355-362)."""
    return _apply("adhoc_chirp235", sign, x)


def plan_tree(n: int, algo: str = "adhoc_auto") -> str:
    return _lib.plan_tree(n, algo)


def _shape_of(x):
    return (x[0] if isinstance(x, tuple) else x).shape


def transform2d(sign: int, x, algo: str = "adhoc_auto"):
    """Adhoc.transform2d (Adhoc.hs:365-371) with SubTransform = Adhoc.transform
    sign: the same algorithm over both axes, lengths read from the array."""
    from .planned import TransformND
    s = _shape_of(x)
    return TransformND(Transform(check(sign), s[-1], algo), Transform(sign, s[-2], algo))(x)


def transform3d(sign: int, x, algo: str = "adhoc_auto"):
    """Adhoc.transform3d (Adhoc.hs:373-380)."""
    from .planned import TransformND
    s = _shape_of(x)
    return TransformND(Transform(check(sign), s[-1], algo), Transform(sign, s[-2], algo),
                       Transform(sign, s[-3], algo))(x)
