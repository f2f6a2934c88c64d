"""Device context: one CUDA device and the stream the library orders its work on.

Replaces the NSL::Device selection of the reference (src/NSL/device.tpp:22-143) for the hot path.
"""
from __future__ import annotations

import ctypes as C
import sys
import threading

from . import _lib


class Context:
    def __init__(self, device: int = 0, stream: int | None = None):
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.nslg_ctx_create(int(device), C.c_void_p(stream) if stream else None, C.byref(h)))
        self.handle = h
        self.device = int(device)
        self._ext = None

    @property
    def stream(self) -> int:
        return int(_lib.load().nslg_ctx_stream(self.handle) or 0)

    def torch_stream(self, dev=None):
        import torch

        if self._ext is None:
            self._ext = torch.cuda.ExternalStream(self.stream, device=dev or torch.device("cuda", self.device))
        return self._ext

    def synchronize(self):
        _lib.check(_lib.load().nslg_ctx_synchronize(self.handle))

    def __del__(self):
        if sys.is_finalizing():  # the CUDA runtime may already be torn down; the OS reclaims everything
            return
        try:
            if getattr(self, "handle", None):
                _lib.load().nslg_ctx_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


_default = None
_dlock = threading.Lock()


def default_context() -> Context:
    global _default
    with _dlock:
        if _default is None:
            _default = Context(0)
    return _default
