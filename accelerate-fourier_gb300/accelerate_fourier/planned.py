"""Fourier.Planned (src/Data/Array/Accelerate/Fourier/Planned.hs).

`transform(sign, length)` returns a Transform: a callable applying the
reference's planned algorithm (split-radix / Cooley-Tukey / Good-Thomas /
Rader / Bluestein, chosen by the reference planner) to the last axis of a
CUDA array.  Like the reference, the length must equal the last extent of
every array the transform is applied to, and results are unscaled.
"""
from __future__ import annotations

import functools

from . import _lib, _tensor
from .sign import check, forward, inverse  # noqa: F401


class Transform:
    """`Transform sh a = Acc (Array sh a) -> Acc (Array sh a)` (Private.hs:29)."""

    def __init__(self, sign: int, length: int, algo: str = "auto"):
        self.sign = check(sign)
        self.length = int(length)
        self.algo = algo
        self.plan = _plan(self.sign, self.length, algo)

    def __call__(self, x, out=None):
        return _tensor.run_plan(self.plan, x, out=out)

    def vjp(self, cotangent, out=None):
        """Adjoint: DFT^H applied to the cotangent (unscaled opposite-sign transform)."""
        return _tensor.run_plan(self.plan, cotangent, vjp=True, out=out)

    def describe(self) -> str:
        return self.plan.describe()


@functools.lru_cache(maxsize=256)
def _plan(sign: int, length: int, algo: str) -> _lib.Plan:
    return _lib.Plan(length, sign, algo)


def transform(sign: int, length: int) -> Transform:
    """Planned.transform (Planned.hs:103-106)."""
    return Transform(sign, length, "auto")


def transformDecompose(sign: int, length: int) -> Transform:
    """Planned.transformDecompose (Planned.hs:114-119): no Bluestein."""
    return Transform(sign, length, "decompose")


def transformChirp2(sign: int, length: int) -> Transform:
    """Planned.transformChirp2 (Planned.hs:704-708): Bluestein, power-of-two pad."""
    return Transform(sign, length, "chirp2")


def transformChirp235(sign: int, length: int) -> Transform:
    """Planned.transformChirp235 (Planned.hs:716-720): Bluestein, 5-smooth pad."""
    return Transform(sign, length, "chirp235")


def plan(length: int) -> str:
    """Planned.plan (Planned.hs:201-203) as the plan tree text."""
    return _lib.plan_tree(length, "auto")


def planDecompose(length: int) -> str:
    return _lib.plan_tree(length, "decompose")
