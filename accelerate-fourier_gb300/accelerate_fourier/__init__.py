"""accelerate_fourier -- GB300 (sm_103a) implementation of accelerate-fourier's
transform hot path behind the reference's module structure.

Modules mirror the reference's Haskell modules:
  planned       Data.Array.Accelerate.Fourier.Planned
  preprocessed  Data.Array.Accelerate.Fourier.Preprocessed
  adhoc         Data.Array.Accelerate.Fourier.Adhoc
  real          Data.Array.Accelerate.Fourier.Real
  utility       Data.Array.Accelerate.Fourier.Utility
  convolution   Data.Array.Accelerate.Convolution.{Adhoc,Preprocessed}
  cyclic        Data.Array.Accelerate.Cyclic
All compute runs in libaf.so (CUDA); there is no CPU fallback.
"""
from . import _lib  # noqa: F401
from .sign import forward, inverse  # noqa: F401


def build(force: bool = False) -> str:
    from . import _build
    return _build.build(force=force)
