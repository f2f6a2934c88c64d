"""Buffer plumbing between Python arrays and the C ABI.

Accepted tensors are numpy arrays (host memory) and torch tensors (CPU or CUDA), complex128 and C-contiguous, the
storage layout of NSL::Tensor<NSL::complex<double>>. Results are returned in the kind of the input: numpy in,
numpy out; a CUDA tensor in, a CUDA tensor out (ordered after the caller's current torch stream).
"""
from __future__ import annotations

import contextlib

import numpy as np

try:  # torch is optional for host-only use
    import torch
except Exception:  # pragma: no cover
    torch = None


def is_torch(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor)


def is_cuda(x) -> bool:
    return is_torch(x) and x.is_cuda


def as_c128(x):
    """Contiguous complex128 view/copy of x (numpy or torch), keeping its kind and device."""
    if is_torch(x):
        if x.dtype != torch.complex128:
            x = x.to(torch.complex128)
        return x.contiguous()
    x = np.asarray(x)
    if x.dtype != np.complex128:
        x = x.astype(np.complex128)
    return np.ascontiguousarray(x)


def ptr(x) -> int:
    return int(x.data_ptr()) if is_torch(x) else int(x.ctypes.data)


def empty_like(x, shape=None):
    shape = tuple(x.shape) if shape is None else tuple(shape)
    if is_torch(x):
        return torch.empty(shape, dtype=torch.complex128, device=x.device)
    return np.empty(shape, dtype=np.complex128)


def numel(shape) -> int:
    n = 1
    for s in shape:
        n *= int(s)
    return n


@contextlib.contextmanager
def stream_order(ctx, *tensors):
    """Orders the library's stream after the caller's torch stream (and back) when CUDA tensors are involved."""
    if not any(is_cuda(t) for t in tensors):
        yield
        return
    dev = next(t.device for t in tensors if is_cuda(t))
    cur = torch.cuda.current_stream(dev)
    ext = ctx.torch_stream(dev)
    ext.wait_stream(cur)
    try:
        yield
    finally:
        cur.wait_stream(ext)
