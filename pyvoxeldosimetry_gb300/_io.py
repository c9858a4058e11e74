"""Host <-> device marshalling for the Python API.

Inputs may be numpy arrays (copied to the device), CPU torch tensors (pinned
ones are copied asynchronously on the current stream) or CUDA torch tensors
(used in place, zero copy).  Results come back in the caller's kind.
"""
from __future__ import annotations

import numpy as np
import torch

NUMPY, CPU_TENSOR, CUDA_TENSOR = "numpy", "cpu", "cuda"


def kind_of(x) -> str:
    if isinstance(x, torch.Tensor):
        return CUDA_TENSOR if x.device.type == "cuda" else CPU_TENSOR
    return NUMPY


def to_device(x, device: torch.device, name: str = "array") -> torch.Tensor:
    """A contiguous float32 CUDA tensor holding ``x`` (no copy if it already is one)."""
    if isinstance(x, torch.Tensor):
        if x.device.type == "cuda":
            if x.device != device:
                x = x.to(device)
            if x.dtype != torch.float32:
                x = x.float()
            return x.contiguous()
        t = x if x.dtype == torch.float32 else x.float()
        return t.contiguous().to(device, non_blocking=t.is_pinned())
    a = np.ascontiguousarray(x, dtype=np.float32)
    if a.ndim == 0:
        raise ValueError(f"{name} must be an array")
    return torch.from_numpy(a).to(device)


def from_device(t: torch.Tensor, kind: str, out=None):
    """Return ``t`` in the caller's kind; CPU results are copied back (pinned
    staging for CPU tensors) and the current stream is synchronised."""
    if kind == CUDA_TENSOR:
        if out is not None:
            out.copy_(t)
            return out
        return t
    if kind == CPU_TENSOR:
        dst = out if out is not None else torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        dst.copy_(t, non_blocking=True)
        torch.cuda.current_stream(t.device).synchronize()
        return dst
    res = t.cpu().numpy()
    if out is not None:
        np.copyto(out, res)
        return out
    return res
