"""Tensor plumbing between torch CUDA tensors and the libaf C ABI.

Arrays follow the reference's convention: the transform runs over the last
axis, every leading axis is batch.  Complex data is a complex64 tensor
(interleaved) or a pair (re, im) of float32 tensors (planar, Accelerate's own
layout of `Array sh (Complex Float)`); the planned transforms also take
Complex Double (complex128, or a pair of float64 tensors).
"""
from __future__ import annotations

import torch

from . import _lib


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def require_cuda(t: torch.Tensor, what: str = "array"):
    if not t.is_cuda:
        raise ValueError(f"{what} must be a CUDA tensor (libaf has no CPU path)")


def as_c64(x: torch.Tensor) -> torch.Tensor:
    require_cuda(x)
    if x.dtype != torch.complex64:
        x = x.to(torch.complex64)
    return x.contiguous()


def rows(x: torch.Tensor):
    n = x.shape[-1] if x.dim() else 0
    batch = 1
    for s in x.shape[:-1]:
        batch *= int(s)
    return int(n), int(batch)


def is_double(x) -> bool:
    """Complex Double data: a complex128 tensor or a pair of float64 tensors."""
    if isinstance(x, tuple):
        return x[0].dtype == torch.float64
    return x.dtype == torch.complex128


def cdtype(double: bool):
    return torch.complex128 if double else torch.complex64


def rdtype(double: bool):
    return torch.float64 if double else torch.float32


def as_complex(x: torch.Tensor, double: bool) -> torch.Tensor:
    """x as a contiguous complex64 (or complex128) CUDA tensor."""
    require_cuda(x)
    return x.to(cdtype(double)).contiguous()


def fn(name: str, double: bool):
    """The C entry point `name`, or its Complex Double form `name_f64`."""
    return getattr(_lib.load(), name + ("_f64" if double else ""))


def run_plan(plan: "_lib.Plan", x, vjp: bool = False, out=None):
    """Apply an af_plan to the last axis of x (complex64 tensor or (re, im);
    complex128 or float64 pairs for a Complex Double plan)."""
    if isinstance(x, tuple):
        re, im = (t.contiguous().to(torch.float64 if plan.double else torch.float32) for t in x)
        require_cuda(re)
        n, batch = rows(re)
        if n != plan.n:
            raise ValueError(f"length {n} does not match plan length {plan.n}")
        ore = torch.empty_like(re) if out is None else out[0]
        oim = torch.empty_like(im) if out is None else out[1]
        if re.numel():
            plan.exec_ptr(re.data_ptr(), im.data_ptr(), ore.data_ptr(), oim.data_ptr(), batch,
                          stream_ptr(), _lib.PLANAR, vjp)
        return ore, oim
    if plan.double:
        require_cuda(x)
        x = x.to(torch.complex128).contiguous()
    else:
        x = as_c64(x)
    n, batch = rows(x)
    if n != plan.n:
        raise ValueError(f"length {n} does not match plan length {plan.n}")
    y = torch.empty_like(x) if out is None else out
    if x.numel():
        plan.exec_ptr(x.data_ptr(), None, y.data_ptr(), None, batch, stream_ptr(), _lib.INTERLEAVED, vjp)
    return y
