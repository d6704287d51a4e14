"""Device, stream and workspace plumbing around the C-ABI library.

torch supplies device memory and the current CUDA stream; every compute call
goes through ``oopao_gb300._native``.  A missing GPU or library raises
``OopaoError`` (no CPU fallback).
"""
import torch

from .tools import OopaoError


_linalg_loaded = False


def _preload_torch_linalg():
    """Load torch's CUDA linear-algebra library by absolute path.

    torch opens it lazily by file name at the first ``torch.linalg`` call on a
    GPU tensor; under some launchers (profilers that rewrite the loader
    environment) that lookup fails.  Loading it once here makes the later
    lookup resolve to the already-loaded library."""
    global _linalg_loaded
    if _linalg_loaded:
        return
    _linalg_loaded = True
    import ctypes
    import os
    p = os.path.join(os.path.dirname(torch.__file__), 'lib', 'libtorch_cuda_linalg.so')
    if os.path.exists(p):
        try:
            ctypes.CDLL(p, mode=ctypes.RTLD_GLOBAL)
        except OSError:
            pass


def device():
    if not torch.cuda.is_available():
        raise OopaoError('oopao_gb300 needs a CUDA device (GB300); none is visible')
    _preload_torch_linalg()
    return torch.device('cuda', torch.cuda.current_device())


class Workspace:
    """Grow-only device scratch buffer (reused across calls on one stream)."""

    def __init__(self):
        self._buf = None

    def get(self, nbytes):
        if self._buf is None or self._buf.numel() < nbytes:
            self._buf = None
            self._buf = torch.empty(int(nbytes), dtype=torch.uint8, device=device())
        return self._buf

    def release(self):
        self._buf = None
