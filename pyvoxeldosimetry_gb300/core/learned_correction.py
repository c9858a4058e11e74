"""Learned heterogeneity correction of the kernel-convolution dose.

No counterpart in the reference: its correction for tissue heterogeneity is the
``tissue_densities`` argument that ``DoseCalculator.calculate_dose`` accepts and
never uses (pyvoxeldosimetry/core/dose_calculator.py:90), and its Monte Carlo
(core/monte_carlo.py:10-172) cannot be constructed (:38-40).

Here a small 3-D U-Net predicts, per voxel, mu = log(D_MC / D_conv) and s = the
log of mu's squared error, from the activity, the density and the
density-scaled convolution dose.  Corrected dose = D_conv * exp(mu); voxels whose
predicted error sqrt(exp(s)) exceeds a threshold keep the plain convolution
dose (the fallback).  The network is trained only on pairs this package
produces itself: ``generate_training_pairs`` runs the GPU Monte Carlo and the
GPU convolution on seeded CT-like phantoms.

Every layer runs in ``libpvd_gb300.so`` (``pvd_unet_*``): 3x3x3 convolutions,
their data and weight gradients as implicit GEMMs on the tcgen05 tensor cores
(BF16 operands, FP32 accumulation in tensor memory), pooling, upsampling, the
head, the loss, Adam.  Torch only allocates device memory and supplies the
stream.

Network: 4 levels with 16, 32, 64, 128 channels; two 3x3x3 convolutions with
LeakyReLU(0.01) per level and decoder stage; 2x2x2 average pooling;
nearest-neighbour upsampling; skip connections by channel concatenation
([upsampled, skip], free in the plane layout: adjacent planes of one buffer);
a 1x1x1 head 16 -> 2.  Crop dimensions must be multiples of 8; whole volumes
are covered by crops that may overhang the volume (zero input there).
"""
from __future__ import annotations

import ctypes as C
import itertools
import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from .. import _native as N
from ..conv import _require_cuda, _stream_handle

SLOPE = 0.01
EPS = 1e-4
LAYERS: List[Tuple[str, int, int]] = [
    ("e0a", 16, 16), ("e0b", 16, 16), ("e1a", 16, 32), ("e1b", 32, 32),
    ("e2a", 32, 64), ("e2b", 64, 64), ("e3a", 64, 128), ("e3b", 128, 128),
    ("d2a", 192, 64), ("d2b", 64, 64), ("d1a", 96, 32), ("d1b", 32, 32),
    ("d0a", 48, 16), ("d0b", 16, 16),
]
LEVEL = {"e0a": 0, "e0b": 0, "e1a": 1, "e1b": 1, "e2a": 2, "e2b": 2, "e3a": 3, "e3b": 3,
         "d2a": 2, "d2b": 2, "d1a": 1, "d1b": 1, "d0a": 0, "d0b": 0}
CHANNELS = {name: (ci, co) for name, ci, co in LAYERS}
HEAD_SIZE = 34
# input channels: activity / max (sqrt), density (linear), conv dose / max (sqrt)
INPUT_MODES = (1, 0, 1)


def geometry(dims) -> N.UnetGeom:
    g = N.UnetGeom()
    N.check(N.load().pvd_unet_geometry(int(dims[0]), int(dims[1]), int(dims[2]), C.byref(g)))
    return g


def conv_flops(dims) -> float:
    """Dense FLOPs of one forward pass (2 x 27 x cin x cout per voxel per conv, plus the head)."""
    v0 = float(dims[0] * dims[1] * dims[2])
    f = sum(2.0 * 27 * ci * co * v0 / 8 ** LEVEL[name] for name, ci, co in LAYERS)
    return f + 2.0 * 32 * v0


class _Tensor:
    """A plane-layout BF16 tensor (or a channel range of one)."""

    __slots__ = ("buf", "ptr", "channels", "geom", "rows")

    def __init__(self, buf, ptr, channels, geom):
        self.buf, self.ptr, self.channels, self.geom = buf, ptr, channels, geom
        self.rows = geom.rows

    @staticmethod
    def zeros(channels, geom, device):
        buf = torch.zeros(channels // 8 * geom.rows * 8, dtype=torch.bfloat16, device=device)
        return _Tensor(buf, buf.data_ptr(), channels, geom)

    def planes(self, first, count_channels):
        return _Tensor(self.buf, self.ptr + first // 8 * self.rows * 16, count_channels, self.geom)

    def to_dense(self) -> torch.Tensor:
        """[C, D, H, W] float32 copy of the interior (for tests and inspection)."""
        g = self.geom
        d, h, w = g.dims[0], g.dims[1], g.dims[2]
        off = (self.ptr - self.buf.data_ptr()) // 2
        v = self.buf[off:off + self.channels // 8 * self.rows * 8].view(self.channels // 8, self.rows, 8)
        v = v[:, g.margin:g.margin + g.padded].reshape(self.channels // 8, d + 2, h + 2, w + 2, 8)
        v = v[:, 1:d + 1, 1:h + 1, 1:w + 1, :].permute(0, 4, 1, 2, 3).reshape(self.channels, d, h, w)
        return v.float()

    def load_dense(self, x: torch.Tensor) -> None:
        """Write a [C, D, H, W] tensor into the interior (tests)."""
        g = self.geom
        d, h, w = g.dims[0], g.dims[1], g.dims[2]
        off = (self.ptr - self.buf.data_ptr()) // 2
        v = self.buf[off:off + self.channels // 8 * self.rows * 8].view(self.channels // 8, self.rows, 8)
        pad = torch.zeros(self.channels // 8, d + 2, h + 2, w + 2, 8, dtype=torch.bfloat16, device=self.buf.device)
        pad[:, 1:d + 1, 1:h + 1, 1:w + 1, :] = x.reshape(self.channels // 8, 8, d, h, w).permute(0, 2, 3, 4, 1).to(
            torch.bfloat16)
        v[:, g.margin:g.margin + g.padded] = pad.reshape(self.channels // 8, -1, 8)


class _Workspace:
    """Activation, gradient and scratch buffers for one crop shape."""

    def __init__(self, dims, device, train: bool):
        if any(int(d) % 8 for d in dims):
            raise ValueError(f"U-Net crop dims must be multiples of 8, got {tuple(dims)}")
        self.dims = tuple(int(d) for d in dims)
        self.geo = [geometry([d >> l for d in self.dims]) for l in range(4)]
        g = self.geo
        Z = lambda c, l: _Tensor.zeros(c, g[l], device)  # noqa: E731
        self.t = t = {}
        t["x0"], t["e0a"], t["cat0"] = Z(16, 0), Z(16, 0), Z(48, 0)
        t["p1"], t["e1a"], t["cat1"] = Z(16, 1), Z(32, 1), Z(96, 1)
        t["p2"], t["e2a"], t["cat2"] = Z(32, 2), Z(64, 2), Z(192, 2)
        t["p3"], t["e3a"], t["e3b"] = Z(64, 3), Z(128, 3), Z(128, 3)
        t["d2a"], t["d2b"] = Z(64, 2), Z(64, 2)
        t["d1a"], t["d1b"] = Z(32, 1), Z(32, 1)
        t["d0a"], t["d0b"] = Z(16, 0), Z(16, 0)
        t["e0b"] = t["cat0"].planes(32, 16)
        t["e1b"] = t["cat1"].planes(64, 32)
        t["e2b"] = t["cat2"].planes(128, 64)
        n0 = self.dims[0] * self.dims[1] * self.dims[2]
        self.pred = torch.zeros(2 * n0, dtype=torch.float32, device=device)
        lib = N.load()
        ws = 0
        sz = C.c_size_t()
        N.check(lib.pvd_unet_head_loss_workspace(C.byref(g[0]), C.byref(sz)))
        ws = max(ws, sz.value)
        self.gr = gr = {}
        if train:
            for name, ci, co in LAYERS:
                N.check(lib.pvd_unet_wgrad_workspace(C.byref(g[LEVEL[name]]), ci, co, C.byref(sz)))
                ws = max(ws, sz.value)
                N.check(lib.pvd_unet_bias_grad_workspace(C.byref(g[LEVEL[name]]), co, C.byref(sz)))
                ws = max(ws, sz.value)
            gr["d0b"], gr["d0a"], gr["cat0"] = Z(16, 0), Z(16, 0), Z(48, 0)
            gr["d1b"], gr["d1a"], gr["cat1"] = Z(32, 1), Z(32, 1), Z(96, 1)
            gr["d2b"], gr["d2a"], gr["cat2"] = Z(64, 2), Z(64, 2), Z(192, 2)
            gr["e3b"], gr["e3a"], gr["p3"] = Z(128, 3), Z(128, 3), Z(64, 3)
            gr["e2a"], gr["p2"], gr["e1a"], gr["p1"], gr["e0a"] = Z(64, 2), Z(32, 2), Z(32, 1), Z(16, 1), Z(16, 0)
            gr["e0b"] = gr["cat0"].planes(32, 16)
            gr["e1b"] = gr["cat1"].planes(64, 32)
            gr["e2b"] = gr["cat2"].planes(128, 64)
        self.scratch = torch.empty(max(ws, 256), dtype=torch.uint8, device=device)


@dataclass
class TrainStats:
    steps: int = 0
    seconds: float = 0.0
    loss_mu: List[float] = field(default_factory=list)
    loss_s: List[float] = field(default_factory=list)
    grad_norm: List[float] = field(default_factory=list)  # before clipping
    skipped: int = 0                                      # steps cut by the running-mean limit


class UNet3D:
    """The correction network: FP32 master parameters, BF16 packed weights,
    forward / backward / Adam through the C ABI."""

    def __init__(self, seed: int = 0, device=None):
        self.device = _require_cuda(device)
        self._lib = N.load()
        self.offsets: Dict[str, Tuple[int, int, int]] = {}  # name -> (w offset, b offset, packed offset)
        o = po = 0
        for name, ci, co in LAYERS:
            self.offsets[name] = (o, o + co * ci * 27, po)
            o += co * ci * 27 + co
            po += co * ci * 27
        self.head_offset = o
        self.n_params = o + HEAD_SIZE
        rng = np.random.default_rng(seed)
        p = np.zeros(self.n_params, np.float32)
        for name, ci, co in LAYERS:
            wo, _, _ = self.offsets[name]
            p[wo:wo + co * ci * 27] = rng.normal(0.0, math.sqrt(2.0 / (27 * ci)), co * ci * 27)
        p[o:o + 32] = rng.normal(0.0, 0.01, 32)
        p[o + 33] = math.log(0.01)
        self.params = torch.from_numpy(p).to(self.device)
        self.grads = torch.zeros(self.n_params + 2, dtype=torch.float32, device=self.device)
        self.m = torch.zeros(self.n_params, dtype=torch.float32, device=self.device)
        self.v = torch.zeros(self.n_params, dtype=torch.float32, device=self.device)
        self.packed_fwd = torch.zeros(po, dtype=torch.bfloat16, device=self.device)
        self.packed_bwd = torch.zeros(po, dtype=torch.bfloat16, device=self.device)
        self.clip_work = torch.zeros(1028, dtype=torch.float32, device=self.device)
        self.step = 0
        self._ws: Dict[Tuple[Tuple[int, int, int], bool, int], _Workspace] = {}
        self._sym: Dict[Tuple[int, int, int], torch.Tensor] = {}
        self._side: List[torch.cuda.Stream] = []
        self._packed_for = -1

    # --- parameters -------------------------------------------------------
    def load_flat(self, flat) -> None:
        flat = torch.as_tensor(np.asarray(flat, np.float32))
        if flat.numel() != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {flat.numel()}")
        self.params.copy_(flat.to(self.device))
        self._packed_for = -1

    def state_dict(self) -> dict:
        return {"params": self.params.cpu().numpy(), "step": self.step}

    def load_state_dict(self, sd: dict) -> None:
        self.load_flat(sd["params"])
        self.step = int(sd.get("step", 0))

    def _ptr(self, t: torch.Tensor, off_elems: int) -> int:
        return t.data_ptr() + off_elems * t.element_size()

    def _pack(self, stream) -> None:
        if self._packed_for == self.step:
            return
        for name, ci, co in LAYERS:
            wo, _, po = self.offsets[name]
            N.check(self._lib.pvd_unet_pack_weights(self._ptr(self.params, wo), ci, co,
                                                    self._ptr(self.packed_fwd, po), self._ptr(self.packed_bwd, po),
                                                    stream))
        self._packed_for = self.step

    def _sym_buffer(self, crop) -> torch.Tensor:
        """[2 * crop voxels] FP32: the symmetry-averaged prediction (mu then s) of a crop."""
        buf = self._sym.get(crop)
        if buf is None:
            buf = self._sym[crop] = torch.empty(2 * int(np.prod(crop)), dtype=torch.float32, device=self.device)
        return buf

    def workspace(self, dims, train: bool, slot: int = 0) -> _Workspace:
        """The activations of one crop shape (slot: one per stream that runs passes
        concurrently)."""
        key = (tuple(int(d) for d in dims), bool(train), int(slot))
        ws = self._ws.get(key)
        if ws is None:
            ws = self._ws[key] = _Workspace(dims, self.device, train)
        return ws

    def side_streams(self, n: int) -> List[torch.cuda.Stream]:
        while len(self._side) < n:
            self._side.append(torch.cuda.Stream(self.device))
        return self._side[:n]

    # --- layers -----------------------------------------------------------
    def _conv(self, name, x: _Tensor, y: _Tensor, stream) -> None:
        ci, co = CHANNELS[name]
        wo, bo, po = self.offsets[name]
        N.check(self._lib.pvd_unet_conv3d(C.byref(x.geom), x.ptr, ci, self._ptr(self.packed_fwd, po),
                                          self._ptr(self.params, bo), y.ptr, co, None, N.PVD_UNET_ACT_LEAKY,
                                          SLOPE, stream))

    def _dgrad(self, name, gy: _Tensor, dx: _Tensor, mask: Optional[_Tensor], stream) -> None:
        ci, co = CHANNELS[name]
        _, _, po = self.offsets[name]
        N.check(self._lib.pvd_unet_conv3d(C.byref(gy.geom), gy.ptr, co, self._ptr(self.packed_bwd, po), None,
                                          dx.ptr, ci, mask.ptr if mask is not None else None, 0, SLOPE, stream))

    def _wgrad(self, name, x: _Tensor, gy: _Tensor, ws: _Workspace, stream) -> None:
        ci, co = CHANNELS[name]
        wo, bo, _ = self.offsets[name]
        N.check(self._lib.pvd_unet_conv3d_wgrad(C.byref(x.geom), x.ptr, ci, gy.ptr, co, self._ptr(self.grads, wo), 0,
                                                ws.scratch.data_ptr(), ws.scratch.numel(), stream))
        N.check(self._lib.pvd_unet_bias_grad(C.byref(gy.geom), gy.ptr, co, self._ptr(self.grads, bo),
                                             ws.scratch.data_ptr(), ws.scratch.numel(), stream))

    def _pool(self, x: _Tensor, y: _Tensor, stream):
        N.check(self._lib.pvd_unet_pool(C.byref(x.geom), x.ptr, C.byref(y.geom), y.ptr, x.channels, stream))

    def _up(self, x: _Tensor, y: _Tensor, stream):
        N.check(self._lib.pvd_unet_upsample(C.byref(x.geom), x.ptr, C.byref(y.geom), y.ptr, x.channels, stream))

    # --- passes -----------------------------------------------------------
    def pack_input(self, ws: _Workspace, volumes: Sequence[torch.Tensor], scales, origin, stream, sym: int = 0) -> None:
        """scales: host floats, or a device float32 tensor of len(volumes) scales.  ``sym``
        packs the volumes transformed by that grid symmetry (``symmetry``); origin and the
        workspace's crop are then in the transformed frame."""
        vd = volumes[0].shape
        n = len(volumes)
        vp = (C.c_void_p * n)(*[v.data_ptr() for v in volumes])
        if isinstance(scales, torch.Tensor):
            sc, sc_d = None, scales.data_ptr()
        else:
            sc, sc_d = (C.c_float * n)(*[float(s) for s in scales]), None
        md = (C.c_int * n)(*INPUT_MODES[:n])
        dims = (C.c_int * 3)(*[int(d) for d in vd])
        org = (C.c_int * 3)(*[int(o) for o in origin])
        N.check(self._lib.pvd_unet_pack_input_sym(C.byref(ws.geo[0]), vp, sc, sc_d, md, n, dims, org, int(sym),
                                                  ws.t["x0"].ptr, stream))

    def forward(self, ws: _Workspace, stream) -> torch.Tensor:
        """Run the network on ws.t['x0']; returns pred [2 * D*H*W] (mu then s)."""
        self._pack(stream)
        t = ws.t
        self._conv("e0a", t["x0"], t["e0a"], stream)
        self._conv("e0b", t["e0a"], t["e0b"], stream)
        self._pool(t["e0b"], t["p1"], stream)
        self._conv("e1a", t["p1"], t["e1a"], stream)
        self._conv("e1b", t["e1a"], t["e1b"], stream)
        self._pool(t["e1b"], t["p2"], stream)
        self._conv("e2a", t["p2"], t["e2a"], stream)
        self._conv("e2b", t["e2a"], t["e2b"], stream)
        self._pool(t["e2b"], t["p3"], stream)
        self._conv("e3a", t["p3"], t["e3a"], stream)
        self._conv("e3b", t["e3a"], t["e3b"], stream)
        self._up(t["e3b"], t["cat2"].planes(0, 128), stream)
        self._conv("d2a", t["cat2"], t["d2a"], stream)
        self._conv("d2b", t["d2a"], t["d2b"], stream)
        self._up(t["d2b"], t["cat1"].planes(0, 64), stream)
        self._conv("d1a", t["cat1"], t["d1a"], stream)
        self._conv("d1b", t["d1a"], t["d1b"], stream)
        self._up(t["d1b"], t["cat0"].planes(0, 32), stream)
        self._conv("d0a", t["cat0"], t["d0a"], stream)
        self._conv("d0b", t["d0a"], t["d0b"], stream)
        N.check(self._lib.pvd_unet_head(C.byref(ws.geo[0]), t["d0b"].ptr, self._ptr(self.params, self.head_offset),
                                        ws.pred.data_ptr(), stream))
        return ws.pred

    def backward(self, ws: _Workspace, target: torch.Tensor, weight: torch.Tensor, origin, stream) -> None:
        """Loss on the crop at `origin` of the target / weight volumes, and every
        parameter gradient into self.grads (the two loss values after them)."""
        self.head_loss(ws, target, weight, origin, stream)
        self.backward_layers(ws, stream)

    def head_loss(self, ws: _Workspace, target: torch.Tensor, weight: torch.Tensor, origin, stream,
                  sym: int = 0) -> None:
        """The loss, the head's gradients and the gradient into the last layer (``sym``:
        the crop is of the volumes transformed by that grid symmetry, as packed)."""
        if not ws.gr:
            raise RuntimeError("workspace was created for inference only")
        t, gr, lib = ws.t, ws.gr, self._lib
        vd = (C.c_int * 3)(*[int(d) for d in target.shape])
        org = (C.c_int * 3)(*[int(o) for o in origin])
        N.check(lib.pvd_unet_head_loss_sym(C.byref(ws.geo[0]), t["d0b"].ptr, self._ptr(self.params, self.head_offset),
                                           ws.pred.data_ptr(), target.data_ptr(), weight.data_ptr(), vd, org, int(sym),
                                           EPS, SLOPE, gr["d0b"].ptr, self._ptr(self.grads, self.head_offset),
                                           ws.scratch.data_ptr(), ws.scratch.numel(), stream))

    def backward_layers(self, ws: _Workspace, stream) -> None:
        """Every layer's parameter gradients, from the gradient head_loss left in the
        last layer (no per-crop arguments: the same launches every step)."""
        if not ws.gr:
            raise RuntimeError("workspace was created for inference only")
        t, gr, lib = ws.t, ws.gr, self._lib
        g0, g1, g2, g3 = (C.byref(x) for x in ws.geo)
        self._wgrad("d0b", t["d0a"], gr["d0b"], ws, stream)
        self._dgrad("d0b", gr["d0b"], gr["d0a"], t["d0a"], stream)
        self._wgrad("d0a", t["cat0"], gr["d0a"], ws, stream)
        self._dgrad("d0a", gr["d0a"], gr["cat0"], None, stream)
        N.check(lib.pvd_unet_upsample_backward(g0, gr["cat0"].ptr, g1, gr["d1b"].ptr, t["d1b"].ptr, 32, SLOPE, stream))
        self._wgrad("d1b", t["d1a"], gr["d1b"], ws, stream)
        self._dgrad("d1b", gr["d1b"], gr["d1a"], t["d1a"], stream)
        self._wgrad("d1a", t["cat1"], gr["d1a"], ws, stream)
        self._dgrad("d1a", gr["d1a"], gr["cat1"], None, stream)
        N.check(lib.pvd_unet_upsample_backward(g1, gr["cat1"].ptr, g2, gr["d2b"].ptr, t["d2b"].ptr, 64, SLOPE, stream))
        self._wgrad("d2b", t["d2a"], gr["d2b"], ws, stream)
        self._dgrad("d2b", gr["d2b"], gr["d2a"], t["d2a"], stream)
        self._wgrad("d2a", t["cat2"], gr["d2a"], ws, stream)
        self._dgrad("d2a", gr["d2a"], gr["cat2"], None, stream)
        N.check(lib.pvd_unet_upsample_backward(g2, gr["cat2"].ptr, g3, gr["e3b"].ptr, t["e3b"].ptr, 128, SLOPE,
                                               stream))
        self._wgrad("e3b", t["e3a"], gr["e3b"], ws, stream)
        self._dgrad("e3b", gr["e3b"], gr["e3a"], t["e3a"], stream)
        self._wgrad("e3a", t["p3"], gr["e3a"], ws, stream)
        self._dgrad("e3a", gr["e3a"], gr["p3"], None, stream)
        N.check(lib.pvd_unet_pool_backward(g3, gr["p3"].ptr, g2, gr["e2b"].ptr, t["e2b"].ptr, 64, 1, SLOPE, stream))
        self._wgrad("e2b", t["e2a"], gr["e2b"], ws, stream)
        self._dgrad("e2b", gr["e2b"], gr["e2a"], t["e2a"], stream)
        self._wgrad("e2a", t["p2"], gr["e2a"], ws, stream)
        self._dgrad("e2a", gr["e2a"], gr["p2"], None, stream)
        N.check(lib.pvd_unet_pool_backward(g2, gr["p2"].ptr, g1, gr["e1b"].ptr, t["e1b"].ptr, 32, 1, SLOPE, stream))
        self._wgrad("e1b", t["e1a"], gr["e1b"], ws, stream)
        self._dgrad("e1b", gr["e1b"], gr["e1a"], t["e1a"], stream)
        self._wgrad("e1a", t["p1"], gr["e1a"], ws, stream)
        self._dgrad("e1a", gr["e1a"], gr["p1"], None, stream)
        N.check(lib.pvd_unet_pool_backward(g1, gr["p1"].ptr, g0, gr["e0b"].ptr, t["e0b"].ptr, 16, 1, SLOPE, stream))
        self._wgrad("e0b", t["e0a"], gr["e0b"], ws, stream)
        self._dgrad("e0b", gr["e0b"], gr["e0a"], t["e0a"], stream)
        self._wgrad("e0a", t["x0"], gr["e0a"], ws, stream)

    def clip_gradients(self, max_norm: float, spike_factor: float = 0.0, stream=None) -> None:
        """Scale the parameter gradients to a global L2 norm of at most max_norm and, with
        spike_factor > 0, of at most spike_factor times the running mean of earlier norms
        (on the device; the norm before clipping is left in clip_work[1024], the count of
        steps the running-mean limit cut in clip_work[1027])."""
        N.check(self._lib.pvd_grad_clip(self.grads.data_ptr(), self.n_params, float(max_norm), float(spike_factor),
                                        self.clip_work.data_ptr(), _stream_handle(stream)))

    def skipped_steps(self) -> int:
        return int(self.clip_work[1027].item())

    def adam(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
             weight_decay: float = 0.0, stream=None) -> None:
        self.step += 1
        N.check(self._lib.pvd_adam_step(self.params.data_ptr(), self.grads.data_ptr(), self.m.data_ptr(),
                                        self.v.data_ptr(), self.n_params, lr, beta1, beta2, eps, weight_decay,
                                        self.step, _stream_handle(stream)))

    def losses(self) -> Tuple[float, float]:
        lv = self.grads[self.n_params:self.n_params + 2].cpu()
        return float(lv[0]), float(lv[1])

    def status(self) -> None:
        code = C.c_int()
        N.check(self._lib.pvd_unet_status(C.byref(code), 1))


# ---------------------------------------------------------------------------
# training data and training
# ---------------------------------------------------------------------------
@dataclass
class TrainingPair:
    """One phantom: device float32 volumes of one grid."""
    activity: torch.Tensor
    density: torch.Tensor
    dose_conv: torch.Tensor
    dose_mc: torch.Tensor
    target: torch.Tensor  # log(D_MC / D_conv), 0 where undefined
    weight: torch.Tensor  # 1 where D_conv > rel_threshold * max and both doses > 0
    scales: Tuple[float, float, float]


def input_scales(activity_max: float, dose_max: float) -> Tuple[float, float, float]:
    return (1.0 / activity_max if activity_max > 0 else 0.0, 1.0, 1.0 / dose_max if dose_max > 0 else 0.0)


TISSUE_DENSITY = 0.2  # g/cc: lung and denser; dose to air is not a target


def _input_scales_device(activity: torch.Tensor, density: torch.Tensor, dose: torch.Tensor) -> torch.Tensor:
    """The input scales of ``input_scales`` computed on the device (no host round
    trip): a float32 tensor [1/max activity, 1, 1/max dose over tissue]."""
    mx = torch.empty(5, dtype=torch.float32, device=activity.device)
    N.check(N.load().pvd_unet_input_maxima(activity.data_ptr(), density.data_ptr(), dose.data_ptr(), activity.numel(),
                                           TISSUE_DENSITY, mx.data_ptr(), _stream_handle(None)))
    return mx[2:5]


def log_ratio_target(dose_conv: np.ndarray, dose_mc: np.ndarray, density: np.ndarray,
                     rel_threshold: float = 0.1) -> Tuple[np.ndarray, np.ndarray, float]:
    """Training target and weight of one phantom (host arithmetic: data preparation,
    not the dose path).  Weighted voxels: tissue (density >= TISSUE_DENSITY) whose
    convolution dose exceeds rel_threshold x its maximum over tissue, or whose Monte
    Carlo dose exceeds rel_threshold x the Monte Carlo's maximum over tissue, with both
    doses positive; target log(D_MC / D_conv) clipped to [-3, 3] there, 0 elsewhere.
    The Monte Carlo test matters in lung: a beta's range there is about three times its
    range in water, the Monte Carlo dose reaches ten times the convolution's, and a
    selection on the convolution dose alone leaves about a third of the lung voxels
    above 10 % of the Monte Carlo maximum out of the loss (Y-90, 3 mm phantoms).  Air
    is excluded because dose to local mass there is dominated by the 1000x smaller
    mass, in both methods.  Returns (target float32, weight float32, tissue maximum of
    the convolution dose)."""
    dc = np.asarray(dose_conv, np.float64)
    dm = np.asarray(dose_mc, np.float64)
    tissue = np.asarray(density) >= TISSUE_DENSITY
    dmax = float(dc[tissue].max()) if tissue.any() else float(dc.max())
    mmax = float(dm[tissue].max()) if tissue.any() else float(dm.max())
    ok = tissue & ((dc > rel_threshold * dmax) | (dm > rel_threshold * mmax)) & (dm > 0) & (dc > 0)
    tgt = np.zeros(dc.shape, np.float32)
    tgt[ok] = np.clip(np.log(dm[ok] / dc[ok]), -3.0, 3.0)
    return tgt, ok.astype(np.float32), dmax


def make_pair(activity: np.ndarray, density: np.ndarray, dose_conv: np.ndarray, dose_mc: np.ndarray,
              rel_threshold: float = 0.1, device=None) -> TrainingPair:
    """One phantom's volumes on the device, with its target and weight (``log_ratio_target``)."""
    tgt, w, dmax = log_ratio_target(dose_conv, dose_mc, density, rel_threshold)
    dev = _require_cuda(device)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)  # noqa: E731
    return TrainingPair(T(activity), T(density), T(dose_conv), T(dose_mc), T(tgt), T(w),
                        input_scales(float(np.max(activity)), dmax))


def mc_consistent_config(radionuclide: str) -> dict:
    """Convolution options under which the plain dose and the Monte Carlo emit the same
    energy per decay: the analytic kernel is normalised to the mean energy of the beta
    spectrum the Monte Carlo samples (the piecewise-linear density through the decay
    data's spectrum points: 1.135 MeV for Y-90, 0.234 for Lu-177, 0.349 for I-131,
    where the data files state means of 0.934, 0.149 and 0.182 MeV).  Without this the
    ratio D_MC / D_conv carries that constant factor besides the heterogeneity the
    network is meant to learn."""
    from ..data.mc_physics import spectrum_mean
    return {"energy_per_decay_mev": spectrum_mean(radionuclide)}


def generate_training_pairs(n: int, shape=(64, 64, 64), voxel_mm: float = 4.0, radionuclide: str = "Y90",
                            histories: int = 20_000_000, seed: int = 100, rel_threshold: float = 0.1,
                            device=None) -> List[TrainingPair]:
    """Seeded CT-like phantoms -> (activity, density, density-scaled convolution
    dose, Monte Carlo dose) on the GPU.  Both doses are dose rates (Gy/s), the
    convolution's normalised to the Monte Carlo's energy per decay
    (``mc_consistent_config``)."""
    from ..phantoms import ct_phantom
    from .kernel_convolution import KernelConvolutionCalculator
    from .monte_carlo import MonteCarloCalculator

    dev = _require_cuda(device)
    conv = KernelConvolutionCalculator(radionuclide, config=mc_consistent_config(radionuclide))
    mc = MonteCarloCalculator(radionuclide, n_particles=histories)
    vox = (voxel_mm,) * 3
    pairs = []
    try:
        for i in range(n):
            act, rho = ct_phantom(shape, voxel_mm, seed=seed + i)
            a_t = torch.from_numpy(act).to(dev)
            r_t = torch.from_numpy(rho).to(dev)
            dc = conv.calculate_dose_rate(a_t, vox, density=r_t)
            dm = mc.calculate_dose_rate(a_t, vox, density=r_t, seed=seed + i)
            pairs.append(make_pair(act, rho, dc.cpu().numpy(), dm.cpu().numpy(), rel_threshold, dev))
    finally:
        conv.close()
        mc.close()
    return pairs


def crop_origin(rng: np.random.Generator, vd, crop, hot: Optional[np.ndarray] = None, flips=()) -> List[int]:
    """Origin of a training crop of a volume of dims vd: inside the volume where the
    crop fits, else covering it (origin in [vd - crop, 0]).  With ``hot`` (flat indices
    of weighted voxels) the crop holds one of them, drawn uniformly, at a uniformly
    random place within the crop, clamped to the same range (which keeps it inside).
    ``flips``: the crop is of the volume flipped along those axes (the origin is in
    the flipped frame; the weighted voxel is mapped into it)."""
    lo = [min(0, vd[k] - c) for k, c in enumerate(crop)]
    hi = [max(0, vd[k] - c) for k, c in enumerate(crop)]
    if hot is not None and hot.size:
        v = [int(x) for x in np.unravel_index(int(hot[int(rng.integers(hot.size))]), vd)]
        for k in flips:
            v[k] = vd[k] - 1 - v[k]
        return [min(max(v[k] - int(rng.integers(c)), lo[k]), hi[k]) for k, c in enumerate(crop)]
    return [int(rng.integers(lo[k], hi[k] + 1)) for k in range(3)]


def train(net: UNet3D, pairs: Sequence[TrainingPair], steps: int, crop=(32, 32, 32), lr: float = 2e-3,
          seed: int = 0, log_every: int = 0, clip: float = 1.0, warmup: float = 0.05,
          spike_factor: float = 10.0, focus: bool = True, graphs: bool = True,
          augment: bool = True) -> TrainStats:
    """Adam on random crops of random pairs; a crop lies inside its volume when it
    fits, else covers it from a random offset.  With ``focus`` every crop holds a
    weighted voxel drawn uniformly from the pair's weighted voxels, at a uniformly
    random place in the crop: the loss lives on a few tenths of a percent of the
    voxels (tissue near the activity), and a crop without any gives a zero gradient
    that Adam's momentum still steps on.  With ``augment`` each crop is taken from the
    volumes flipped along a random set of axes (one of the 8 flips; the inputs, target
    and weight alike, pvd_unet_pack_input_sym / pvd_unet_head_loss_sym): the dose
    physics is flip-invariant, and the network learns it that way instead of from the
    phantoms' orientation.  The learning rate rises linearly over
    the first ``warmup`` fraction of the steps, then decays on a cosine; gradients are
    clipped to a global norm of ``clip`` (0: no clipping) and to ``spike_factor`` times
    the running mean of the earlier norms: one outlying crop would otherwise throw
    Adam's second moments off course.  The direction of a clipped gradient is kept:
    dropping such steps instead lets the momentum carry a diverging network further.
    With ``graphs`` the launches that take no per-crop argument -- weight packing and
    the forward pass; every layer's backward -- are recorded once as two CUDA graphs
    and replayed, leaving four library calls per step on the host (input packing,
    loss head, clipping, Adam) instead of about ninety."""
    rng = np.random.default_rng(seed)
    ws = net.workspace(crop, train=True)
    stream = _stream_handle(None)
    stats = TrainStats()
    hot = [np.flatnonzero(p.weight.cpu().numpy().ravel()) if focus else None for p in pairs]
    torch.cuda.synchronize(net.device)
    t0 = time.perf_counter()
    g_fwd = g_bwd = None
    for it in range(steps):
        ip = int(rng.integers(len(pairs)))
        p = pairs[ip]
        sym = int(rng.integers(8)) if augment else 0
        origin = crop_origin(rng, tuple(p.activity.shape), crop, hot[ip], symmetry(sym)[1])
        net.pack_input(ws, (p.activity, p.density, p.dose_conv), p.scales, origin, stream, sym=sym)
        if g_fwd is not None:
            g_fwd.replay()
            net.head_loss(ws, p.target, p.weight, origin, stream, sym=sym)
            g_bwd.replay()
        else:
            net.forward(ws, stream)
            net.head_loss(ws, p.target, p.weight, origin, stream, sym=sym)
            net.backward_layers(ws, stream)
        nw = max(1, int(warmup * steps))
        lr_t = lr * (it + 1) / nw if it < nw else lr * 0.5 * (1 + math.cos(math.pi * (it - nw) / max(1, steps - nw)))
        if clip > 0:
            net.clip_gradients(clip, spike_factor if it >= nw else 0.0)
        net.adam(lr=lr_t)
        if graphs and it == 0 and steps > 1:
            # recorded after one eager step (every launch configuration is set up by then)
            g_fwd, g_bwd = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
            net._packed_for = -1
            with torch.cuda.graph(g_fwd):
                net.forward(ws, _stream_handle(None))
            with torch.cuda.graph(g_bwd):
                net.backward_layers(ws, _stream_handle(None))
        if log_every and (it % log_every == 0 or it == steps - 1):
            lm, ls = net.losses()
            stats.loss_mu.append(lm)
            stats.loss_s.append(ls)
            stats.grad_norm.append(float(net.clip_work[1024]))
    torch.cuda.synchronize(net.device)
    stats.seconds = time.perf_counter() - t0
    net._packed_for = -1  # the graph's packing does not track the step count
    stats.steps = steps
    stats.skipped = net.skipped_steps()
    net.status()
    return stats


SYMMETRY_SETS = (1, 8, 48)  # identity; the 8 flips; flips and the 6 axis permutations


def symmetry(code: int) -> Tuple[Tuple[int, int, int], Tuple[int, ...]]:
    """(axis permutation, flipped axes) of grid symmetry ``code`` in [0, 48), as the
    library numbers them: permutation code // 8 of (0, 1, 2) in lexicographic order,
    then the axes k of the permuted volume with bit k of code % 8 set flipped.  The
    transformed volume is ``np.flip(np.transpose(v, perm), flips)``."""
    if not 0 <= code < N.PVD_UNET_SYMMETRIES:
        raise ValueError("symmetry code must be in [0, 48)")
    perm = list(itertools.permutations((0, 1, 2)))[code // 8]
    return perm, tuple(k for k in range(3) if (code % 8) >> k & 1)


def _round8(shape) -> tuple:
    return tuple(-(-int(s) // 8) * 8 for s in shape)


INFERENCE_BYTES_PER_VOXEL = 300  # activations of every level (BF16) + the FP32 prediction, per crop voxel


def flip_streams(symmetries: int, crop, device) -> int:
    """How many symmetry passes run concurrently: up to 4, each with its own
    workspace, within a quarter of the device's free memory."""
    free, _ = torch.cuda.mem_get_info(device)
    per = INFERENCE_BYTES_PER_VOXEL * int(np.prod(crop))
    return max(1, min(4, symmetries, int(0.25 * free) // max(per, 1)))


def predict(net: UNet3D, activity: torch.Tensor, density: torch.Tensor, dose_conv: torch.Tensor,
            scales=None, sigma_max: float = 0.5, mu_clamp: float = 3.0, out: Optional[torch.Tensor] = None,
            return_fallback: bool = False, symmetries: int = 1, streams: Optional[int] = None):
    """Corrected dose for a whole volume (device float32 tensors of one shape).
    The network runs on one crop covering the volume, its dims rounded up to
    multiples of 8 (the overhang reads as zero input).  ``symmetries`` (1, 8 or 48)
    averages the prediction (mu and s) over that many grid symmetries: the network
    runs on each transformed volume and its output is mapped back and summed
    (pvd_unet_symmetry_accumulate).  The 8 flips hold for any voxel size; the 48
    include axis permutations and hold only for isotropic voxels.  The passes run on
    ``streams`` side streams at once (default ``flip_streams``: the deep, small layers
    of one pass leave most SMs idle), and are summed on the current stream in
    symmetry order, so the result does not depend on the stream count.  Everything
    is enqueued without a host round trip; the current stream waits for all of it.
    ``net.status()`` reads the tensor-core pipeline's status word afterwards."""
    if symmetries not in SYMMETRY_SETS:
        raise ValueError(f"symmetries must be one of {SYMMETRY_SETS}")
    dev = net.device
    shape = tuple(activity.shape)
    if scales is None:
        scales = _input_scales_device(activity, density, dose_conv)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=dev)
    fb = torch.empty(shape, dtype=torch.uint8, device=dev) if return_fallback else None
    stream = _stream_handle(None)
    crop = _round8(shape)
    geo0 = geometry(crop)
    vols = (activity, density, dose_conv)
    vd = (C.c_int * 3)(*shape)
    if symmetries == 1:
        ws = net.workspace(crop, train=False)
        net.pack_input(ws, vols, scales, (0, 0, 0), stream)
        pred = net.forward(ws, stream)
    else:
        pred = net._sym_buffer(crop)
        main = torch.cuda.current_stream(dev)
        net._pack(stream)  # weights packed once, before the passes fork
        nst = streams if streams is not None else flip_streams(symmetries, crop, dev)
        side = net.side_streams(max(1, min(int(nst), symmetries)))
        ready = torch.cuda.Event()
        ready.record(main)
        reusable = [ready] * len(side)  # when a side stream's workspace may be written again
        for k in range(symmetries):
            i = k % len(side)
            st = side[i]
            st.wait_event(reusable[i])
            perm, _ = symmetry(k)
            ws_k = net.workspace(_round8(shape[a] for a in perm), train=False, slot=i + 1)
            sh = int(st.cuda_stream)
            net.pack_input(ws_k, vols, scales, (0, 0, 0), sh, sym=k)
            pk = net.forward(ws_k, sh)
            done = torch.cuda.Event()
            done.record(st)
            main.wait_event(done)
            N.check(net._lib.pvd_unet_symmetry_accumulate(C.byref(ws_k.geo[0]), pk.data_ptr(), C.byref(geo0),
                                                          vd, k, 1.0 / symmetries, int(k > 0), pred.data_ptr(),
                                                          stream))
            reusable[i] = torch.cuda.Event()
            reusable[i].record(main)
    org = (C.c_int * 3)(0, 0, 0)
    N.check(net._lib.pvd_unet_apply_correction(C.byref(geo0), pred.data_ptr(), dose_conv.data_ptr(), vd, org,
                                               sigma_max, mu_clamp, out.data_ptr(),
                                               fb.data_ptr() if fb is not None else None, stream))
    return (out, fb) if return_fallback else out


def dose_errors(dose: np.ndarray, reference: np.ndarray, rel_threshold: float = 0.1,
                density: Optional[np.ndarray] = None) -> Dict[str, float]:
    """Relative errors |D - D_ref| / D_ref over voxels with D_ref > rel_threshold
    x max (max and voxels restricted to tissue when a density map is given)."""
    d = np.asarray(dose, np.float64)
    r = np.asarray(reference, np.float64)
    sel = np.ones(r.shape, bool) if density is None else np.asarray(density) >= TISSUE_DENSITY
    m = sel & (r > rel_threshold * r[sel].max())
    e = np.abs(d[m] - r[m]) / r[m]
    return {"mean": float(e.mean()), "median": float(np.median(e)), "p95": float(np.percentile(e, 95)),
            "max": float(e.max()), "within_3pct": float((e <= 0.03).mean()), "voxels": int(m.sum())}


def save_model(net: UNet3D, path: str) -> None:
    """FP32 parameters and the optimiser step count, as an .npz file."""
    np.savez(path, params=net.params.cpu().numpy(), step=np.int64(net.step), layers=np.array(repr(LAYERS)))


def load_model(path: str, device=None) -> UNet3D:
    z = np.load(path)
    if str(z["layers"]) != repr(LAYERS):
        raise ValueError(f"{path}: saved for a different layer table")
    net = UNet3D(device=device)
    net.load_state_dict({"params": z["params"], "step": int(z["step"])})
    return net


from .dosimetry_base import DosimetryCalculator  # noqa: E402


class NNCorrectedDoseCalculator(DosimetryCalculator):
    """Plain density-scaled kernel convolution plus the learned heterogeneity
    correction, behind the reference's calculator interface
    (core/dosimetry_base.py:8-70).  config: ``model`` (a UNet3D) or
    ``model_path`` (.npz from save_model), ``sigma_max`` (fallback threshold on
    the predicted error of log(D_MC/D_conv), default 0.5), ``symmetries`` (the
    prediction averaged over the 8 grid flips by default; 48 adds the axis
    permutations and needs isotropic voxels; 1 runs the network once), plus the
    convolution calculator's own options.  The convolution runs under
    ``mc_consistent_config`` (the energy per decay of the Monte Carlo the network
    was trained against) unless the config says otherwise.  Without a density map
    the plain convolution is returned: the correction is a correction for
    heterogeneity."""

    def __init__(self, radionuclide: str, tissue_composition=None, config: Optional[dict] = None):
        super().__init__(radionuclide, tissue_composition, config)
        if not isinstance(radionuclide, str):
            raise TypeError("NNCorrectedDoseCalculator takes one radionuclide")
        from .kernel_convolution import KernelConvolutionCalculator
        conv_cfg = {**mc_consistent_config(radionuclide), **self.config}
        self.conv = KernelConvolutionCalculator(radionuclide, self.config.get("tissue_name", "water"),
                                                self.config.get("kernel_resolution", 1.0), conv_cfg)
        model = self.config.get("model")
        if model is None and self.config.get("model_path"):
            model = load_model(self.config["model_path"], self.config.get("device"))
        if model is None:
            raise ValueError("NNCorrectedDoseCalculator needs config['model'] or config['model_path']")
        self.model: UNet3D = model
        self.sigma_max = float(self.config.get("sigma_max", 0.5))
        self.symmetries = int(self.config.get("symmetries", 8))
        if self.symmetries not in SYMMETRY_SETS:
            raise ValueError(f"symmetries must be one of {SYMMETRY_SETS}")
        self._fb = None

    def calculate_dose_rate(self, activity_map, voxel_size: Tuple[float, float, float], density=None):
        from .. import _io
        if len(voxel_size) != 3:
            raise ValueError("voxel_size must be a tuple of length 3.")
        kind = _io.kind_of(activity_map)
        dev = self.model.device
        a = _io.to_device(activity_map, dev, "activity")
        if density is None:
            return _io.from_device(self.conv.calculate_dose_rate(a, voxel_size), kind)
        if self.symmetries == 48 and len({float(v) for v in voxel_size}) != 1:
            raise ValueError("48 symmetries (axis permutations) need isotropic voxels; use 8")
        rho = _io.to_device(density, dev, "density")
        dc = self.conv.calculate_dose_rate(a, voxel_size, density=rho)
        out, self._fb = predict(self.model, a, rho, dc, sigma_max=self.sigma_max, return_fallback=True,
                                symmetries=self.symmetries)
        self.model.status()
        return _io.from_device(out, kind)

    def fallback_fraction(self) -> float:
        """Fraction of voxels of the last call that kept the plain convolution dose."""
        return 0.0 if self._fb is None else float(self._fb.float().mean())

    def calculate_absorbed_dose(self, activity_maps, time_points: List[float], voxel_size, density=None):
        from .kernel_convolution import trapezoid_weights
        from .activity_sampler import weighted_sum
        if len(activity_maps) != len(time_points):
            raise ValueError("Number of activity maps must match number of time points")
        rates = [self.calculate_dose_rate(a, voxel_size, density=density) for a in activity_maps]
        return weighted_sum(rates, trapezoid_weights(time_points, 3600.0))

    def calculate_absorbed_dose_from_accumulated(self, accumulated_activity, voxel_size, density=None,
                                                 seconds_per_unit: float = 3600.0):
        return self.calculate_dose_rate(accumulated_activity, voxel_size, density=density) * seconds_per_unit

    def close(self):
        self.conv.close()
