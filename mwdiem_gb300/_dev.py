"""Device-memory plumbing for the Python entry points (torch is used only for allocation, copies
and streams)."""
from __future__ import annotations

import numpy as np
import torch

_NP2T = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
         np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64, np.dtype(np.uint32): torch.int32}


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("mwdiem_gb300 needs a CUDA device; none is visible")


def stream_handle(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


class Arg:
    """One array argument: a device tensor, plus the numpy array to copy back into (in-place
    semantics of pycuda's ``cuda.InOut``) when the caller passed host memory."""

    def __init__(self, x, dtype, name, out=False, device=None):
        self.name = name
        self.host = None
        npdt = np.dtype(dtype)
        tdt = _NP2T[npdt]
        if isinstance(x, torch.Tensor):
            if not x.is_cuda:
                x = x.numpy()
            else:
                if out and (x.dtype != tdt or not x.is_contiguous()):
                    raise TypeError(f"{name}: in/out device tensor must be contiguous {tdt}")
                self.t = x if (x.dtype == tdt and x.is_contiguous()) else x.to(tdt).contiguous()
                return
        a = np.asarray(x)
        if out:
            if a.dtype != npdt or not a.flags.c_contiguous or not a.flags.writeable:
                # the reference would also hand back a new array in that case (MWDiem.py:917 rebinds)
                a = np.ascontiguousarray(a, dtype=npdt)
            self.host = a
        else:
            a = np.ascontiguousarray(a, dtype=npdt)
        self.t = torch.from_numpy(a).to(device or "cuda", non_blocking=False)

    @property
    def ptr(self) -> int:
        return self.t.data_ptr()

    def result(self):
        if self.host is not None:
            self.host[...] = self.t.cpu().numpy().reshape(self.host.shape)
            return self.host
        return self.t


def is_device(x) -> bool:
    return isinstance(x, torch.Tensor) and x.is_cuda
