"""ORACLE — test infrastructure only, never the product path.

Float64 torch-CPU restatement of the learned heterogeneity correction network
(no counterpart in the reference: its density hook ``tissue_densities``,
pyvoxeldosimetry/core/dose_calculator.py:90, is unused and its Monte Carlo,
core/monte_carlo.py:38-40, cannot run).  Only ``tests/`` import this module; the
CUDA layers (``pvd_unet_*``) are checked against it.

Network: a 4-level 3-D U-Net, 16 -> 128 channels, 3x3x3 convolutions with
zero padding 1 and LeakyReLU(0.01), 2x2x2 average pooling, nearest-neighbour
upsampling, skip connections by channel concatenation [upsampled, skip], and a
1x1x1 head with two outputs: mu = predicted log(D_MC / D_conv) and s =
predicted log of mu's squared error.  Loss over the n voxels of a crop with
e = mu - t and l = log(e^2 + eps) (l a constant):
    loss_mu = sum w e^2 / n,   loss_s = sum w (s - l)^2 / n.
The s head reads the last features without passing its gradient back into the
network (only loss_mu trains the convolutions).

``forward`` / ``backward`` restate the GPU computation step by step.  With
``bf16=True`` every tensor the GPU stores in BF16 (activations, pooled and
upsampled tensors, gradients between layers) is rounded to BF16 here at the
same point, and weights are rounded to BF16 where the GPU packs them, so the
remaining difference is FP32-vs-FP64 accumulation.  ``autograd_grads`` is the
same network differentiated by torch autograd without any rounding: it checks
the hand-written backward.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

SLOPE = 0.01
EPS = 1e-4
# (name, input channels, output channels); inputs of d2a/d1a/d0a are [upsampled, skip]
LAYERS = [
    ("e0a", 16, 16), ("e0b", 16, 16), ("e1a", 16, 32), ("e1b", 32, 32),
    ("e2a", 32, 64), ("e2b", 64, 64), ("e3a", 64, 128), ("e3b", 128, 128),
    ("d2a", 192, 64), ("d2b", 64, 64), ("d1a", 96, 32), ("d1b", 32, 32),
    ("d0a", 48, 16), ("d0b", 16, 16),
]
HEAD_SIZE = 34  # w_mu (16), w_s (16), b_mu, b_s


def n_params() -> int:
    return sum(co * ci * 27 + co for _, ci, co in LAYERS) + HEAD_SIZE


def unpack(flat) -> dict:
    """Flat parameter vector -> {name: (W [co, ci, 3, 3, 3], b [co])} + 'head'."""
    flat = torch.as_tensor(np.asarray(flat, dtype=np.float64))
    out, o = {}, 0
    for name, ci, co in LAYERS:
        w = flat[o:o + co * ci * 27].reshape(co, ci, 3, 3, 3)
        o += co * ci * 27
        b = flat[o:o + co]
        o += co
        out[name] = (w, b)
    out["head"] = flat[o:o + HEAD_SIZE]
    return out


def _bf(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.bfloat16).to(torch.float64)


def _lrelu(x):
    return torch.where(x > 0, x, x * SLOPE)


def _lrelu_grad(m):
    return torch.where(m > 0, torch.ones_like(m), torch.full_like(m, SLOPE))


def _pool(x):
    return F.avg_pool3d(x, 2)


def _up(x):
    return x.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)


def _up_bwd(g):
    n, c, d, h, w = g.shape
    return g.reshape(n, c, d // 2, 2, h // 2, 2, w // 2, 2).sum((3, 5, 7))


def forward(params: dict, x0: torch.Tensor, bf16: bool = True) -> dict:
    """x0: [1, 16, D, H, W] float64 network input.  Returns every stored tensor."""
    r = _bf if bf16 else (lambda t: t)

    def conv(x, name):
        w, b = params[name]
        w = _bf(w) if bf16 else w
        return r(_lrelu(F.conv3d(x, w, b, padding=1)))

    a = {"x0": r(x0)}
    a["e0a"] = conv(a["x0"], "e0a")
    a["e0b"] = conv(a["e0a"], "e0b")
    a["p1"] = r(_pool(a["e0b"]))
    a["e1a"] = conv(a["p1"], "e1a")
    a["e1b"] = conv(a["e1a"], "e1b")
    a["p2"] = r(_pool(a["e1b"]))
    a["e2a"] = conv(a["p2"], "e2a")
    a["e2b"] = conv(a["e2a"], "e2b")
    a["p3"] = r(_pool(a["e2b"]))
    a["e3a"] = conv(a["p3"], "e3a")
    a["e3b"] = conv(a["e3a"], "e3b")
    a["cat2"] = torch.cat([_up(a["e3b"]), a["e2b"]], 1)
    a["d2a"] = conv(a["cat2"], "d2a")
    a["d2b"] = conv(a["d2a"], "d2b")
    a["cat1"] = torch.cat([_up(a["d2b"]), a["e1b"]], 1)
    a["d1a"] = conv(a["cat1"], "d1a")
    a["d1b"] = conv(a["d1a"], "d1b")
    a["cat0"] = torch.cat([_up(a["d1b"]), a["e0b"]], 1)
    a["d0a"] = conv(a["cat0"], "d0a")
    a["d0b"] = conv(a["d0a"], "d0b")
    h = params["head"]
    f = a["d0b"][0]  # [16, D, H, W]
    mu = torch.einsum("c,cdhw->dhw", h[0:16], f) + h[32]
    s = torch.einsum("c,cdhw->dhw", h[16:32], f) + h[33]
    a["pred"] = torch.stack([mu, s])
    a["s_detached"] = torch.einsum("c,cdhw->dhw", h[16:32], f.detach()) + h[33]
    return a


def backward(params: dict, acts: dict, target: torch.Tensor, weight: torch.Tensor, bf16: bool = True):
    """Hand-written backward in the GPU's order.  target, weight: [D, H, W].
    Returns (grads {name: (dW, db)} + 'head' (34), loss_mu, loss_s)."""
    r = _bf if bf16 else (lambda t: t)
    h = params["head"]
    mu, s = acts["pred"][0], acts["pred"][1]
    n = mu.numel()
    e = mu - target
    l = torch.log(e * e + EPS)
    gm = 2 * weight * e / n
    gs = 2 * weight * (s - l) / n
    f = acts["d0b"][0]
    head_g = torch.cat([(gm * f).sum((1, 2, 3)), (gs * f).sum((1, 2, 3)), gm.sum()[None], gs.sum()[None]])
    loss_mu = float((weight * e * e).sum() / n)
    loss_s = float((weight * (s - l) ** 2).sum() / n)
    g = {"head": head_g}

    def wb(name):
        w, _ = params[name]
        return _bf(w) if bf16 else w

    def layer(name, x, gy):
        """Weight and bias gradients of a conv given its input x and pre-activation gradient gy."""
        w, _ = params[name]
        dw = torch.nn.grad.conv3d_weight(x, w.shape, gy, padding=1)
        g[name] = (dw, gy.sum((0, 2, 3, 4)))

    def dgrad(name, x_shape, gy, mask=None):
        dx = torch.nn.grad.conv3d_input(x_shape, wb(name), gy, padding=1)
        if mask is not None:
            dx = dx * _lrelu_grad(mask)
        return r(dx)

    A = acts
    g_d0b = r((h[0:16, None, None, None] * gm)[None] * _lrelu_grad(A["d0b"]))
    layer("d0b", A["d0a"], g_d0b)
    g_d0a = dgrad("d0b", A["d0a"].shape, g_d0b, A["d0a"])
    layer("d0a", A["cat0"], g_d0a)
    g_cat0 = dgrad("d0a", A["cat0"].shape, g_d0a)
    c_up0 = A["d1b"].shape[1]
    g_d1b = r(_up_bwd(g_cat0[:, :c_up0]) * _lrelu_grad(A["d1b"]))
    layer("d1b", A["d1a"], g_d1b)
    g_d1a = dgrad("d1b", A["d1a"].shape, g_d1b, A["d1a"])
    layer("d1a", A["cat1"], g_d1a)
    g_cat1 = dgrad("d1a", A["cat1"].shape, g_d1a)
    c_up1 = A["d2b"].shape[1]
    g_d2b = r(_up_bwd(g_cat1[:, :c_up1]) * _lrelu_grad(A["d2b"]))
    layer("d2b", A["d2a"], g_d2b)
    g_d2a = dgrad("d2b", A["d2a"].shape, g_d2b, A["d2a"])
    layer("d2a", A["cat2"], g_d2a)
    g_cat2 = dgrad("d2a", A["cat2"].shape, g_d2a)
    c_up2 = A["e3b"].shape[1]
    g_e3b = r(_up_bwd(g_cat2[:, :c_up2]) * _lrelu_grad(A["e3b"]))
    layer("e3b", A["e3a"], g_e3b)
    g_e3a = dgrad("e3b", A["e3a"].shape, g_e3b, A["e3a"])
    layer("e3a", A["p3"], g_e3a)
    g_p3 = dgrad("e3a", A["p3"].shape, g_e3a)
    g_e2b = r((g_cat2[:, c_up2:] + _up(g_p3) / 8) * _lrelu_grad(A["e2b"]))
    layer("e2b", A["e2a"], g_e2b)
    g_e2a = dgrad("e2b", A["e2a"].shape, g_e2b, A["e2a"])
    layer("e2a", A["p2"], g_e2a)
    g_p2 = dgrad("e2a", A["p2"].shape, g_e2a)
    g_e1b = r((g_cat1[:, c_up1:] + _up(g_p2) / 8) * _lrelu_grad(A["e1b"]))
    layer("e1b", A["e1a"], g_e1b)
    g_e1a = dgrad("e1b", A["e1a"].shape, g_e1b, A["e1a"])
    layer("e1a", A["p1"], g_e1a)
    g_p1 = dgrad("e1a", A["p1"].shape, g_e1a)
    g_e0b = r((g_cat0[:, c_up0:] + _up(g_p1) / 8) * _lrelu_grad(A["e0b"]))
    layer("e0b", A["e0a"], g_e0b)
    g_e0a = dgrad("e0b", A["e0a"].shape, g_e0b, A["e0a"])
    layer("e0a", A["x0"], g_e0a)
    return g, loss_mu, loss_s


def autograd_grads(params: dict, x0: torch.Tensor, target: torch.Tensor, weight: torch.Tensor):
    """The same network and loss differentiated by torch autograd (float64, no rounding).
    The log-error target l of the s-loss and the features the s head reads are
    detached, as in the hand-written backward."""
    leaves = {}
    p2 = {}
    for name, _, _ in LAYERS:
        w, b = params[name]
        w = w.clone().requires_grad_(True)
        b = b.clone().requires_grad_(True)
        leaves[name] = (w, b)
        p2[name] = (w, b)
    hd = params["head"].clone().requires_grad_(True)
    p2["head"] = hd
    a = forward(p2, x0, bf16=False)
    mu, s = a["pred"][0], a["s_detached"]
    n = mu.numel()
    e = mu - target
    l = torch.log(e.detach() ** 2 + EPS)
    loss = (weight * e * e).sum() / n + (weight * (s - l) ** 2).sum() / n
    loss.backward()
    g = {name: (w.grad, b.grad) for name, (w, b) in leaves.items()}
    g["head"] = hd.grad
    return g


def flat_grads(g: dict) -> np.ndarray:
    """{name: (dW, db)} + head -> flat vector in the parameter order of ``unpack``."""
    parts = []
    for name, _, _ in LAYERS:
        dw, db = g[name]
        parts += [dw.reshape(-1).numpy(), db.reshape(-1).numpy()]
    parts.append(g["head"].reshape(-1).numpy())
    return np.concatenate(parts)


def input_features(volumes, scales, modes) -> torch.Tensor:
    """The 16-channel network input: channel c = transform(volume_c * scale_c),
    transform 0 linear, 1 sqrt, 2 log1p (negative values clipped to 0 first for
    1 and 2), computed in FP32 like the GPU, other channels zero."""
    d, h, w = volumes[0].shape
    x = torch.zeros(1, 16, d, h, w, dtype=torch.float64)
    for c, (v, sc, m) in enumerate(zip(volumes, scales, modes)):
        t = torch.as_tensor(np.asarray(v, dtype=np.float32)) * np.float32(sc)
        if m == 1:
            t = torch.sqrt(torch.clamp(t, min=0))
        elif m == 2:
            t = torch.log1p(torch.clamp(t, min=0))
        x[0, c] = t.to(torch.float64)
    return x
