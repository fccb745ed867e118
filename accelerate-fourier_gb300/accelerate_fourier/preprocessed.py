"""Fourier.Preprocessed (src/Data/Array/Accelerate/Fourier/Preprocessed.hs).

The size is known on the host; the transform object is built once and
shared between calls (`let transform = dit2 1024 in transform x ...`)."""
from __future__ import annotations

from .planned import Transform
from .sign import forward, inverse  # noqa: F401


def ditSplitRadix(sign: int, length: int) -> Transform:
    """Preprocessed.ditSplitRadix (Preprocessed.hs:53-93); length a power of two."""
    return Transform(sign, length, "prep_splitradix")


def dit2(sign: int, length: int) -> Transform:
    """Preprocessed.dit2 (Preprocessed.hs:99-111); length a power of two."""
    return Transform(sign, length, "prep_dit2")


def dif2(sign: int, length: int) -> Transform:
    """Preprocessed.dif2 (Preprocessed.hs:117-135); length a power of two."""
    return Transform(sign, length, "prep_dif2")


def transform2d(transform0: Transform, transform1: Transform):
    """Preprocessed.transform2d (Preprocessed.hs:142-148): transform0 along the
    last axis, transform1 along the second-to-last."""
    from .planned import TransformND
    return TransformND(transform0, transform1)


def transform3d(transform0: Transform, transform1: Transform, transform2: Transform):
    """Preprocessed.transform3d (Preprocessed.hs:154-160)."""
    from .planned import TransformND
    return TransformND(transform0, transform1, transform2)
