"""Fourier.Preprocessed (src/Data/Array/Accelerate/Fourier/Preprocessed.hs).

The size is known on the host; the transform object is built once and
shared between calls (`let transform = dit2 1024 in transform x ...`)."""
from __future__ import annotations

from .planned import Transform
from .sign import forward, inverse  # noqa: F401


def ditSplitRadix(sign: int, length: int) -> Transform:
    """Preprocessed.ditSplitRadix (Preprocessed.hs:433-444); length a power of two."""
    return Transform(sign, length, "prep_splitradix")


def dit2(sign: int, length: int) -> Transform:
    """Preprocessed.dit2 (Preprocessed.hs:479-491); length a power of two."""
    return Transform(sign, length, "prep_dit2")


def dif2(sign: int, length: int) -> Transform:
    """Preprocessed.dif2 (Preprocessed.hs:497-515); length a power of two."""
    return Transform(sign, length, "prep_dif2")
