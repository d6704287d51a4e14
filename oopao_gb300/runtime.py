"""Device, stream and workspace plumbing around the C-ABI library.

torch supplies device memory and the current CUDA stream; every compute call
goes through ``oopao_gb300._native``.  A missing GPU or library raises
``OopaoError`` (no CPU fallback).
"""
import torch

from .tools import OopaoError


def device():
    if not torch.cuda.is_available():
        raise OopaoError('oopao_gb300 needs a CUDA device (GB300); none is visible')
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
