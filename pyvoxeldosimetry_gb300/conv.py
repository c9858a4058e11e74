"""Device-side convolution plan: a thin owner of a ``pvd_plan*`` from the C ABI.

Torch supplies device memory and the current CUDA stream; every computation
happens in ``libpvd_gb300.so``.  There is no CPU path: without a CUDA device
or without the library, construction raises.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np
import torch

from . import _native as N


def _require_cuda(device) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("pyvoxeldosimetry_gb300 needs a CUDA device (sm_103a); no CPU fallback exists")
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.type != "cuda":
        raise ValueError(f"device must be a CUDA device, got {dev}")
    return dev


def _stream_handle(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


class ConvPlan:
    """FFT dose-point-kernel convolution plan for one volume shape.

    Parameters
    ----------
    shape : (n0, n1, n2) volume dims, C order (n2 contiguous).
    kmax : largest kernel dims (LINEAR mode: sets the zero padding).
    n_kernels : kernel slots (nuclides) sharing one forward transform.
    mode : "linear" (zero-padded, cropped "same" convolution) or
        "reference_circular" (exactly the reference's unpadded circular
        operator, kernel_convolution.py:71-74).
    pad : optional explicit FFT lengths.
    tma : stage the column passes' tiles with TMA bulk tensor loads (persistent,
        double-buffered).  Off by default: measured on GB300 it is 1-7 % slower than
        loading the tiles straight into registers (the passes are barrier/issue
        bound, and the two stages cost an occupancy step).
    """

    def __init__(self, shape: Sequence[int], kmax: Sequence[int] = (1, 1, 1), n_kernels: int = 1,
                 mode: str = "linear", pad: Sequence[int] | None = None, device=None, tma: bool = False):
        self.device = _require_cuda(device)
        self._lib = N.load()
        if mode not in ("linear", "reference_circular"):
            raise ValueError(f"mode must be 'linear' or 'reference_circular', got {mode!r}")
        self.shape = tuple(int(s) for s in shape)
        if len(self.shape) != 3:
            raise ValueError("shape must have 3 dims")
        self.mode = mode
        self.n_kernels = int(n_kernels)
        d = N.ConvDesc()
        for i in range(3):
            d.n[i] = self.shape[i]
            d.kmax[i] = int(kmax[i])
            d.pad[i] = int(pad[i]) if pad is not None else 0
        d.mode = N.PVD_MODE_LINEAR if mode == "linear" else N.PVD_MODE_CIRCULAR
        d.n_kernels = self.n_kernels
        d.flags = N.PVD_PLAN_TMA if tma else 0
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check(self._lib.pvd_plan_create(C.byref(d), C.byref(h)))
        self._h = h
        info = N.PlanInfo()
        N.check(self._lib.pvd_plan_get_info(self._h, C.byref(info)))
        self.fft_shape = tuple(info.p)
        self.workspace_bytes = int(info.workspace_bytes)
        self.h = int(info.h)
        self.hs = int(info.hs)
        self._kernel_set = [False] * self.n_kernels

    # -- kernels --------------------------------------------------------------
    def set_kernel(self, slot: int, kernel: np.ndarray, scale: float = 1.0, normalize: bool = False) -> None:
        """Load a kernel (host array, any float dtype) into ``slot``.

        ``normalize`` divides by the kernel's sum, computed in FP64 on the GPU;
        ``scale`` multiplies the (normalised) kernel.
        """
        k = np.ascontiguousarray(kernel, dtype=np.float64)
        if k.ndim != 3:
            raise ValueError("kernel must be 3-D")
        flags = N.PVD_KERNEL_NORMALIZE if normalize else 0
        with torch.cuda.device(self.device):
            N.check(self._lib.pvd_plan_set_kernel(self._h, int(slot), k.ctypes.data_as(C.c_void_p), k.shape[0],
                                                  k.shape[1], k.shape[2], float(scale), flags))
        self._kernel_set[slot] = True

    # -- execution ------------------------------------------------------------
    def _check_vol(self, t: torch.Tensor, what: str) -> torch.Tensor:
        if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
            raise TypeError(f"{what} must be a CUDA torch tensor")
        if tuple(t.shape) != self.shape:
            raise ValueError(f"{what} has shape {tuple(t.shape)}, plan expects {self.shape}")
        if t.dtype != torch.float32 or not t.is_contiguous():
            raise TypeError(f"{what} must be a contiguous float32 tensor")
        if t.device != self.device:
            raise ValueError(f"{what} is on {t.device}, plan on {self.device}")
        return t

    def execute(self, activity, density: torch.Tensor | None = None, out: torch.Tensor | None = None,
                out_scale: float = 1.0, weights: Sequence[float] | None = None, stream=None) -> torch.Tensor:
        """Dose for every kernel slot: ``out[s] = out_scale * (A (*) K_s) / rho``.

        ``activity`` is one CUDA float32 volume, or a sequence of volumes
        combined as ``sum_t weights[t] * activity[t]`` inside the first pass.
        Returns ``out`` of shape (n_kernels, *shape); enqueued on ``stream``
        (default: torch's current stream).
        """
        if out is None:
            out = torch.empty((self.n_kernels, *self.shape), dtype=torch.float32, device=self.device)
        elif tuple(out.shape) != (self.n_kernels, *self.shape) or out.dtype != torch.float32 \
                or not out.is_contiguous() or out.device != self.device:
            raise ValueError("out must be a contiguous float32 CUDA tensor of shape (n_kernels, *shape)")
        rho = self._check_vol(density, "density").data_ptr() if density is not None else None
        sh = _stream_handle(stream)
        if isinstance(activity, torch.Tensor):
            a = self._check_vol(activity, "activity")
            if weights is not None:
                raise ValueError("weights apply to a sequence of activity volumes")
            st = self._lib.pvd_conv_execute(self._h, a.data_ptr(), rho, out.data_ptr(), float(out_scale), sh)
        else:
            acts = [self._check_vol(a, "activity[t]") for a in activity]
            if weights is None or len(weights) != len(acts):
                raise ValueError("weights must give one value per activity volume")
            ptrs = (C.c_void_p * len(acts))(*[a.data_ptr() for a in acts])
            w = (C.c_float * len(acts))(*[float(x) for x in weights])
            st = self._lib.pvd_conv_execute_weighted(self._h, ptrs, w, len(acts), rho, out.data_ptr(),
                                                     float(out_scale), sh)
        N.check(st)
        return out

    def execute_host(self, activity, density=None, out=None, out_scale: float = 1.0, stream=None):
        """Dose from HOST arrays (numpy or CPU tensors) through the plan's pipelined
        host path (pvd_conv_execute_host): uploads, passes and downloads overlap.

        Returns ``out`` (a CPU float32 tensor of shape (n_kernels, *shape), page-locked
        when allocated here) after the copies back have completed.
        """
        keep = []

        def host_ptr(x, what):
            if isinstance(x, torch.Tensor):
                if x.device.type != "cpu" or x.dtype != torch.float32 or not x.is_contiguous():
                    raise TypeError(f"{what} must be a contiguous float32 CPU tensor")
                if tuple(x.shape) != self.shape:
                    raise ValueError(f"{what} has shape {tuple(x.shape)}, plan expects {self.shape}")
                keep.append(x)
                return x.data_ptr()
            a = np.ascontiguousarray(x, dtype=np.float32)
            if a.shape != self.shape:
                raise ValueError(f"{what} has shape {a.shape}, plan expects {self.shape}")
            keep.append(a)
            return a.ctypes.data

        ap = host_ptr(activity, "activity")
        rp = host_ptr(density, "density") if density is not None else None
        if out is None:
            out = torch.empty((self.n_kernels, *self.shape), dtype=torch.float32, pin_memory=True)
        elif not (isinstance(out, torch.Tensor) and out.device.type == "cpu" and out.dtype == torch.float32
                  and out.is_contiguous() and tuple(out.shape) == (self.n_kernels, *self.shape)):
            raise ValueError("out must be a contiguous float32 CPU tensor of shape (n_kernels, *shape)")
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device):
            N.check(self._lib.pvd_conv_execute_host(self._h, ap, rp, out.data_ptr(), float(out_scale),
                                                    int(stream.cuda_stream)))
            stream.synchronize()
        return out

    def status(self) -> None:
        """Raise if a pass reported a device-side error (a TMA load that timed out)."""
        N.check(self._lib.pvd_plan_status(self._h))

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.pvd_plan_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
