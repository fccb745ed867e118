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
    """`Transform sh a = Acc (Array sh a) -> Acc (Array sh a)` (Private.hs:29).

    Like the reference's transforms (polymorphic over `A.RealFloat a`), one
    Transform applies to Complex Float and Complex Double arrays: complex128
    data (or float64 planes) runs on a Complex Double plan of the same tree,
    made on first use."""

    def __init__(self, sign: int, length: int, algo: str = "auto"):
        self.sign = check(sign)
        self.length = int(length)
        self.algo = algo
        self.plan = _plan(self.sign, self.length, algo)

    def plan_for(self, x) -> _lib.Plan:
        return self.plan_of(_tensor.is_double(x))

    def plan_of(self, double: bool) -> _lib.Plan:
        """The plan of this transform over Complex Double (double) or Complex Float."""
        return _plan(self.sign, self.length, self.algo, True) if double else self.plan

    def __call__(self, x, out=None):
        return _tensor.run_plan(self.plan_for(x), x, out=out)

    def vjp(self, cotangent, out=None):
        """Adjoint: DFT^H applied to the cotangent (unscaled opposite-sign transform)."""
        return _tensor.run_plan(self.plan_for(cotangent), cotangent, vjp=True, out=out)

    def describe(self) -> str:
        return self.plan.describe()


@functools.lru_cache(maxsize=256)
def _plan(sign: int, length: int, algo: str, double: bool = False) -> _lib.Plan:
    return _lib.Plan(length, sign, algo, double)


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


class TransformND:
    """A 2-D or 3-D transform over the last axes: transforms[0] runs along
    the last (least significant) axis, as in the reference's
    SubTransformPair/SubTransformTriple (Preprocessed.hs:136-160); each
    transform keeps its own sign.  libaf addresses the strided axes directly
    instead of transposing (Adhoc.hs:365-380)."""

    def __init__(self, *transforms: Transform):
        if len(transforms) not in (2, 3):
            raise ValueError("TransformND takes two or three transforms")
        self.transforms = transforms

    def shape_check(self, shape, double: bool = False):
        d = len(self.transforms)
        if len(shape) < d:
            raise ValueError(f"array needs at least {d} axes")
        for k, t in enumerate(self.transforms):
            if int(shape[-1 - k]) != t.length:
                raise ValueError(f"axis {-1 - k} has length {shape[-1 - k]}, transform length {t.length}")
        img = 1
        for t in self.transforms:
            img *= t.length
        batch = 1
        for s in shape[:-d]:
            batch *= int(s)
        return (*[t.plan_of(double) for t in self.transforms], batch)

    def __call__(self, x, out=None):
        import torch
        lib = _lib.load()
        d = len(self.transforms)
        double = _tensor.is_double(x)
        if isinstance(x, tuple):
            re, im = (t.contiguous().to(torch.float64 if double else torch.float32) for t in x)
            _tensor.require_cuda(re)
            *_, batch = self.shape_check(re.shape)
            ore = torch.empty_like(re) if out is None else out[0]
            oim = torch.empty_like(im) if out is None else out[1]
            args = (_lib.PLANAR, re.data_ptr(), im.data_ptr(), ore.data_ptr(), oim.data_ptr(), batch,
                    _tensor.stream_ptr())
            res = (ore, oim)
            n = re.numel()
        else:
            _tensor.require_cuda(x)
            x = x.contiguous() if double else _tensor.as_c64(x)
            *_, batch = self.shape_check(x.shape)
            y = torch.empty_like(x) if out is None else out
            args = (_lib.INTERLEAVED, x.data_ptr(), None, y.data_ptr(), None, batch, _tensor.stream_ptr())
            res = y
            n = x.numel()
        if n:
            handles = [t.plan_for(x).handle for t in self.transforms]
            if double:
                f = lib.af_exec_c2c_2d_f64 if d == 2 else lib.af_exec_c2c_3d_f64
            else:
                f = lib.af_exec_c2c_2d if d == 2 else lib.af_exec_c2c_3d
            _lib.check(f(*handles, *args))
        return res


def convolveCyclic(length: int):
    """Planned.convolveCyclic (Planned.hs:779-790): a function of two complex
    arrays of the given length, F(G(x)/n * G(y)) with the planned transforms.
    complex128 (or float64 planes) runs in Complex Double."""
    t = Transform(forward, length, "auto")

    def conv(x, y):
        import torch
        if isinstance(x, tuple) != isinstance(y, tuple):
            raise ValueError("x and y must have one layout")
        double = _tensor.is_double(x)
        f = _tensor.fn("af_convolve_cyclic", double)
        h = t.plan_of(double).handle
        if isinstance(x, tuple):
            xr, xi, yr, yi = (a.contiguous().to(_tensor.rdtype(double)) for a in (*x, *y))
            _tensor.require_cuda(xr)
            if xr.shape != yr.shape:
                raise ValueError("signals must have equal size")
            n, batch = _tensor.rows(xr)
            if n != length:
                raise ValueError("length mismatch")
            ore, oim = torch.empty_like(xr), torch.empty_like(xi)
            if xr.numel():
                _lib.check(f(h, _lib.PLANAR, xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(),
                             ore.data_ptr(), oim.data_ptr(), batch, _tensor.stream_ptr()))
            return ore, oim
        x, y = _tensor.as_complex(x, double), _tensor.as_complex(y, double)
        if x.shape != y.shape:
            raise ValueError("signals must have equal size")
        n, batch = _tensor.rows(x)
        if n != length:
            raise ValueError("length mismatch")
        out = torch.empty_like(x)
        if x.numel():
            _lib.check(f(h, _lib.INTERLEAVED, x.data_ptr(), None, y.data_ptr(), None, out.data_ptr(), None, batch,
                         _tensor.stream_ptr()))
        return out

    return conv
