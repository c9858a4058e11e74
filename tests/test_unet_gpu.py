"""Learned-correction network on the GPU against the float64 CPU oracle.

Per layer (convolution forward, data gradient with mask and accumulation,
weight gradient, bias gradient, pooling, upsampling, head, loss): GPU result vs
torch float64 on the same BF16-rounded inputs.  Tolerances: BF16 outputs within
4e-3 normwise and 1e-2 of max (one BF16 rounding, 2^-9 relative); FP32 outputs
(weight / bias gradients, head, loss) within 1e-4 normwise.
Whole network: loss and every parameter gradient vs the oracle's hand-written
backward with BF16 rounding at the GPU's storage points (2e-2 normwise per
layer), and vs unrounded autograd (0.1 normwise).
"""
import ctypes as C

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from oracle import unet as ou

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from pyvoxeldosimetry_gb300 import _native as N
    from pyvoxeldosimetry_gb300.core import learned_correction as lc
    lib = N.load()
    code = C.c_int()
    lib.pvd_unet_status(C.byref(code), 1)
    return N, lc, lib, torch.device("cuda", 0)


def _bf(x):
    return x.to(torch.bfloat16).to(torch.float64)


def _nrm(a, b):
    a = torch.as_tensor(a, dtype=torch.float64).cpu()
    b = torch.as_tensor(b, dtype=torch.float64).cpu()
    return float((a - b).norm() / b.norm().clamp_min(1e-300))


def _check_bf16(out, ref, what):
    ref = ref.cpu().double()
    out = out.cpu().double()
    e = _nrm(out, ref)
    m = float((out - ref).abs().max() / ref.abs().max().clamp_min(1e-300))
    assert e <= 4e-3 and m <= 1e-2, f"{what}: normwise {e:.2e}, max {m:.2e}"


def _halo_zero(t, lc):
    """Every row of the tensor's planes outside the interior voxels is zero."""
    g = t.geom
    d, h, w = g.dims[0], g.dims[1], g.dims[2]
    off = (t.ptr - t.buf.data_ptr()) // 2
    v = t.buf[off:off + t.channels // 8 * t.rows * 8].view(t.channels // 8, t.rows, 8).float()
    mask = torch.ones(t.rows, dtype=torch.bool, device=v.device)
    inner = torch.zeros(d + 2, h + 2, w + 2, dtype=torch.bool, device=v.device)
    inner[1:d + 1, 1:h + 1, 1:w + 1] = True
    mask[g.margin:g.margin + g.padded] = ~inner.reshape(-1)
    return float(v[:, mask].abs().max()) == 0.0


DIMS = (11, 13, 17)  # padded 13 x 15 x 19: 29 row tiles, the last one partial


def _dense(c, dims, gen, scale=1.0):
    return (torch.randn((c,) + dims, generator=gen, dtype=torch.float64) * scale).to(torch.bfloat16).double()


@pytest.mark.parametrize("cin,cout", [(16, 16), (48, 16), (16, 32), (64, 64), (128, 128), (192, 64)])
def test_conv_forward(env, cin, cout):
    N, lc, lib, dev = env
    gen = torch.Generator().manual_seed(cin * 1000 + cout)
    g = lc.geometry(DIMS)
    X = _dense(cin, DIMS, gen)
    W = torch.randn(cout, cin, 27, generator=gen, dtype=torch.float64) * np.sqrt(2.0 / (27 * cin))
    b = torch.randn(cout, generator=gen, dtype=torch.float64) * 0.1
    x = lc._Tensor.zeros(cin, g, dev)
    x.load_dense(X.float().to(dev))
    y = lc._Tensor.zeros(cout, g, dev)
    w32 = W.float().to(dev)
    packed = torch.zeros(27 * cin * cout, dtype=torch.bfloat16, device=dev)
    N.check(lib.pvd_unet_pack_weights(w32.data_ptr(), cin, cout, packed.data_ptr(), None, None))
    b32 = b.float().to(dev)
    N.check(lib.pvd_unet_conv3d(C.byref(g), x.ptr, cin, packed.data_ptr(), b32.data_ptr(), y.ptr, cout, None,
                                N.PVD_UNET_ACT_LEAKY, 0.01, None))
    code = C.c_int()
    N.check(lib.pvd_unet_status(C.byref(code), 1))
    ref = F.leaky_relu(F.conv3d(X[None], _bf(W).reshape(cout, cin, 3, 3, 3), b.float().double(), padding=1), 0.01)[0]
    _check_bf16(y.to_dense(), ref, f"conv {cin}->{cout}")
    assert _halo_zero(y, lc)


@pytest.mark.parametrize("cin,cout,mode", [(16, 16, "fwd"), (32, 32, "fwd"), (96, 32, "fwd"), (128, 128, "fwd"),
                                            (192, 64, "fwd"), (96, 32, "dgrad"), (64, 192, "dgrad")])
def test_conv_persistent_many_tiles(env, cin, cout, mode):
    """About 1170 row tiles: more than one tile per persistent CTA, all three kernel
    forms (dx taps stacked along N for 16/32 output channels, all taps resident, a
    ring of tap slots for the large layers)."""
    N, lc, lib, dev = env
    dims = (46, 50, 58)
    gen = torch.Generator().manual_seed(3 * cin + cout)
    g = lc.geometry(dims)
    X = _dense(cin, dims, gen)
    W = torch.randn(cout, cin, 27, generator=gen, dtype=torch.float64) * np.sqrt(2.0 / (27 * cin))
    x = lc._Tensor.zeros(cin, g, dev)
    x.load_dense(X.float().to(dev))
    y = lc._Tensor.zeros(cout, g, dev)
    packed = torch.zeros(27 * cin * cout, dtype=torch.bfloat16, device=dev)
    if mode == "fwd":
        N.check(lib.pvd_unet_pack_weights(W.float().to(dev).data_ptr(), cin, cout, packed.data_ptr(), None, None))
        N.check(lib.pvd_unet_conv3d(C.byref(g), x.ptr, cin, packed.data_ptr(), None, y.ptr, cout, None,
                                    N.PVD_UNET_ACT_LEAKY, 0.01, None))
        ref = F.leaky_relu(F.conv3d(X[None], _bf(W).reshape(cout, cin, 3, 3, 3), padding=1), 0.01)[0]
    else:  # the data gradient of a cout -> cin convolution: run cin -> cout on the mirrored packing
        Wt = torch.randn(cin, cout, 27, generator=gen, dtype=torch.float64) * 0.05
        N.check(lib.pvd_unet_pack_weights(Wt.float().to(dev).data_ptr(), cout, cin, None, packed.data_ptr(), None))
        N.check(lib.pvd_unet_conv3d(C.byref(g), x.ptr, cin, packed.data_ptr(), None, y.ptr, cout, None, 0, 0.01,
                                    None))
        ref = torch.nn.grad.conv3d_input((1, cout) + dims, _bf(Wt).reshape(cin, cout, 3, 3, 3), X[None],
                                         padding=1)[0]
    code = C.c_int()
    N.check(lib.pvd_unet_status(C.byref(code), 1))
    _check_bf16(y.to_dense(), ref, f"{mode} {cin}->{cout} many tiles")
    assert _halo_zero(y, lc)


@pytest.mark.parametrize("cin,cout", [(16, 16), (32, 64), (48, 16), (96, 32), (192, 64), (128, 128)])
def test_conv_data_gradient(env, cin, cout):
    """Input gradient of a cin -> cout conv: the kernel run cout -> cin on the
    mirrored packing, times leaky'(mask), then with accumulation."""
    N, lc, lib, dev = env
    gen = torch.Generator().manual_seed(7 + cin + 3 * cout)
    g = lc.geometry(DIMS)
    G = _dense(cout, DIMS, gen)
    M = _dense(cin, DIMS, gen)
    W = torch.randn(cout, cin, 27, generator=gen, dtype=torch.float64) * 0.05
    gt = lc._Tensor.zeros(cout, g, dev)
    gt.load_dense(G.float().to(dev))
    mt = lc._Tensor.zeros(cin, g, dev)
    mt.load_dense(M.float().to(dev))
    dx = lc._Tensor.zeros(cin, g, dev)
    w32 = W.float().to(dev)
    bwd = torch.zeros(27 * cin * cout, dtype=torch.bfloat16, device=dev)
    N.check(lib.pvd_unet_pack_weights(w32.data_ptr(), cin, cout, None, bwd.data_ptr(), None))
    N.check(lib.pvd_unet_conv3d(C.byref(g), gt.ptr, cout, bwd.data_ptr(), None, dx.ptr, cin, mt.ptr, 0, 0.01, None))
    ref = torch.nn.grad.conv3d_input((1, cin) + DIMS, _bf(W).reshape(cout, cin, 3, 3, 3), G[None], padding=1)[0]
    ref = ref * torch.where(M > 0, 1.0, 0.01)
    first = dx.to_dense()
    _check_bf16(first, ref, f"dgrad {cout}->{cin}")
    assert _halo_zero(dx, lc)
    # accumulate: dx += the same gradient without a mask
    N.check(lib.pvd_unet_conv3d(C.byref(g), gt.ptr, cout, bwd.data_ptr(), None, dx.ptr, cin, None,
                                N.PVD_UNET_ACCUMULATE, 0.01, None))
    ref2 = first.double().cpu() + torch.nn.grad.conv3d_input((1, cin) + DIMS, _bf(W).reshape(cout, cin, 3, 3, 3),
                                                              G[None], padding=1)[0]
    _check_bf16(dx.to_dense(), ref2, f"dgrad accumulate {cout}->{cin}")
    code = C.c_int()
    N.check(lib.pvd_unet_status(C.byref(code), 1))


@pytest.mark.parametrize("cin,cout", [(16, 16), (48, 16), (16, 32), (192, 64), (128, 128), (64, 192)])
def test_weight_and_bias_gradient(env, cin, cout):
    N, lc, lib, dev = env
    gen = torch.Generator().manual_seed(11 * cin + cout)
    g = lc.geometry(DIMS)
    X = _dense(cin, DIMS, gen)
    G = _dense(cout, DIMS, gen)
    x = lc._Tensor.zeros(cin, g, dev)
    x.load_dense(X.float().to(dev))
    gt = lc._Tensor.zeros(cout, g, dev)
    gt.load_dense(G.float().to(dev))
    sz = C.c_size_t()
    N.check(lib.pvd_unet_wgrad_workspace(C.byref(g), cin, cout, C.byref(sz)))
    ws = torch.empty(sz.value, dtype=torch.uint8, device=dev)
    dw = torch.full((cout, cin, 27), 7.0, dtype=torch.float32, device=dev)
    N.check(lib.pvd_unet_conv3d_wgrad(C.byref(g), x.ptr, cin, gt.ptr, cout, dw.data_ptr(), 0, ws.data_ptr(),
                                      ws.numel(), None))
    ref = torch.nn.grad.conv3d_weight(X[None], (cout, cin, 3, 3, 3), G[None], padding=1).reshape(cout, cin, 27)
    e = _nrm(dw.double(), ref)
    assert e <= 1e-4, f"wgrad {cin}x{cout}: normwise {e:.2e}"
    # accumulate adds a second copy; deterministic: same bits twice
    dw2 = dw.clone()
    N.check(lib.pvd_unet_conv3d_wgrad(C.byref(g), x.ptr, cin, gt.ptr, cout, dw2.data_ptr(), 1, ws.data_ptr(),
                                      ws.numel(), None))
    assert torch.equal(dw2, dw + dw)
    N.check(lib.pvd_unet_bias_grad_workspace(C.byref(g), cout, C.byref(sz)))
    wsb = torch.empty(sz.value, dtype=torch.uint8, device=dev)
    db = torch.empty(cout, dtype=torch.float32, device=dev)
    N.check(lib.pvd_unet_bias_grad(C.byref(g), gt.ptr, cout, db.data_ptr(), wsb.data_ptr(), wsb.numel(), None))
    assert _nrm(db.double(), G.sum((1, 2, 3))) <= 1e-5
    code = C.c_int()
    N.check(lib.pvd_unet_status(C.byref(code), 1))


def test_pool_upsample_head_loss(env):
    N, lc, lib, dev = env
    gen = torch.Generator().manual_seed(5)
    fd, cd = (8, 12, 16), (4, 6, 8)
    gf, gc = lc.geometry(fd), lc.geometry(cd)
    X = _dense(32, fd, gen)
    x = lc._Tensor.zeros(32, gf, dev)
    x.load_dense(X.float().to(dev))
    y = lc._Tensor.zeros(32, gc, dev)
    N.check(lib.pvd_unet_pool(C.byref(gf), x.ptr, C.byref(gc), y.ptr, 32, None))
    _check_bf16(y.to_dense(), F.avg_pool3d(X[None], 2)[0], "pool")
    u = lc._Tensor.zeros(32, gf, dev)
    N.check(lib.pvd_unet_upsample(C.byref(gc), y.ptr, C.byref(gf), u.ptr, 32, None))
    assert torch.equal(u.to_dense(), ou._up(y.to_dense()[None].double())[0].float())
    assert _halo_zero(y, lc) and _halo_zero(u, lc)
    # backward of both, with mask and accumulation
    Gc = _dense(32, cd, gen)
    Mf = _dense(32, fd, gen)
    gct = lc._Tensor.zeros(32, gc, dev)
    gct.load_dense(Gc.float().to(dev))
    mf = lc._Tensor.zeros(32, gf, dev)
    mf.load_dense(Mf.float().to(dev))
    dxf = lc._Tensor.zeros(32, gf, dev)
    dxf.load_dense(X.float().to(dev))
    N.check(lib.pvd_unet_pool_backward(C.byref(gc), gct.ptr, C.byref(gf), dxf.ptr, mf.ptr, 32, 1, 0.01, None))
    ref = (X + ou._up(Gc[None])[0] / 8) * torch.where(Mf > 0, 1.0, 0.01)
    _check_bf16(dxf.to_dense(), ref, "pool backward")
    Mc = _dense(32, cd, gen)
    mc = lc._Tensor.zeros(32, gc, dev)
    mc.load_dense(Mc.float().to(dev))
    dxc = lc._Tensor.zeros(32, gc, dev)
    N.check(lib.pvd_unet_upsample_backward(C.byref(gf), x.ptr, C.byref(gc), dxc.ptr, mc.ptr, 32, 0.01, None))
    _check_bf16(dxc.to_dense(), ou._up_bwd(X[None])[0] * torch.where(Mc > 0, 1.0, 0.01), "upsample backward")
    # head + loss on a crop overhanging the volume
    H = _dense(16, fd, gen)
    h = lc._Tensor.zeros(16, gf, dev)
    h.load_dense(H.float().to(dev))
    wh = torch.randn(34, generator=gen, dtype=torch.float64) * 0.3
    whd = wh.float().to(dev)
    n = int(np.prod(fd))
    pred = torch.empty(2 * n, dtype=torch.float32, device=dev)
    N.check(lib.pvd_unet_head(C.byref(gf), h.ptr, whd.data_ptr(), pred.data_ptr(), None))
    mu = torch.einsum("c,cdhw->dhw", wh[:16].float().double(), H) + float(np.float32(wh[32]))
    s = torch.einsum("c,cdhw->dhw", wh[16:32].float().double(), H) + float(np.float32(wh[33]))
    p = pred.cpu().double().reshape(2, *fd)
    assert _nrm(p[0], mu) <= 1e-5 and _nrm(p[1], s) <= 1e-5
    vol = (10, 14, 20)
    origin = (3, -2, 5)
    T = torch.randn(vol, generator=gen, dtype=torch.float64) * 0.3
    Wt = (torch.rand(vol, generator=gen) > 0.4).double()
    Td, Wd = T.float().to(dev), Wt.float().to(dev)
    N.check(lib.pvd_unet_head_loss_workspace(C.byref(gf), C.byref(sz := C.c_size_t())))
    ws = torch.empty(sz.value, dtype=torch.uint8, device=dev)
    gx = lc._Tensor.zeros(16, gf, dev)
    out = torch.empty(36, dtype=torch.float32, device=dev)
    vd = (C.c_int * 3)(*vol)
    org = (C.c_int * 3)(*origin)
    N.check(lib.pvd_unet_head_loss(C.byref(gf), h.ptr, whd.data_ptr(), pred.data_ptr(), Td.data_ptr(), Wd.data_ptr(),
                                   vd, org, ou.EPS, 0.01, gx.ptr, out.data_ptr(), ws.data_ptr(), ws.numel(), None))
    tc = torch.zeros(fd, dtype=torch.float64)
    wc = torch.zeros(fd, dtype=torch.float64)
    sl = [slice(max(0, -o), min(f, v - o)) for o, f, v in zip(origin, fd, vol)]
    sv = [slice(s_.start + o, s_.stop + o) for s_, o in zip(sl, origin)]
    tc[sl[0], sl[1], sl[2]] = T.float().double()[sv[0], sv[1], sv[2]]
    wc[sl[0], sl[1], sl[2]] = Wt[sv[0], sv[1], sv[2]]
    hw = wh.float().double()
    # the oracle's head-loss formulas on the crop (the GPU's own pred as mu, s)
    e_ = p[0] - tc
    l_ = torch.log(e_ * e_ + ou.EPS)
    gm = 2 * wc * e_ / n
    gs = 2 * wc * (p[1] - l_) / n
    ref_g = torch.cat([(gm * H).sum((1, 2, 3)), (gs * H).sum((1, 2, 3)), gm.sum()[None], gs.sum()[None]])
    o = out.cpu().double()
    assert _nrm(o[:34], ref_g) <= 1e-4
    assert abs(o[34] - float((wc * e_ * e_).sum() / n)) <= 1e-5 * abs(float(o[34])) + 1e-12
    assert abs(o[35] - float((wc * (p[1] - l_) ** 2).sum() / n)) <= 1e-5 * abs(float(o[35])) + 1e-12
    gref = hw[0:16, None, None, None] * gm * torch.where(H > 0, 1.0, 0.01)
    _check_bf16(gx.to_dense(), gref, "head gradient")
    code = C.c_int()
    N.check(lib.pvd_unet_status(C.byref(code), 1))


def _network_problem(dims, seed):
    rng = np.random.default_rng(seed)
    flat = np.zeros(ou.n_params(), np.float32)
    o = 0
    for _, ci, co in ou.LAYERS:
        flat[o:o + co * ci * 27] = rng.normal(0, np.sqrt(2.0 / (27 * ci)), co * ci * 27)
        o += co * ci * 27
        flat[o:o + co] = rng.normal(0, 0.05, co)
        o += co
    flat[o:o + 34] = rng.normal(0, 0.3, 34)
    vols = [rng.random(dims).astype(np.float32) for _ in range(3)]
    target = rng.normal(0, 0.3, dims).astype(np.float32)
    weight = (rng.random(dims) > 0.3).astype(np.float32)
    return flat, vols, target, weight


@pytest.mark.parametrize("dims", [(16, 16, 16), (24, 16, 32)])
def test_network_gradients_match_oracle(env, dims):
    N, lc, lib, dev = env
    flat, vols, target, weight = _network_problem(dims, 3)
    net = lc.UNet3D(device=dev)
    net.load_flat(flat)
    ws = net.workspace(dims, train=True)
    vt = [torch.from_numpy(v).to(dev) for v in vols]
    td, wd = torch.from_numpy(target).to(dev), torch.from_numpy(weight).to(dev)
    s = torch.cuda.current_stream().cuda_stream
    net.pack_input(ws, vt, (1.0, 1.0, 1.0), (0, 0, 0), s)
    net.forward(ws, s)
    net.backward(ws, td, wd, (0, 0, 0), s)
    net.status()
    g_gpu = net.grads[:net.n_params].cpu().double().numpy()
    lm, ls = net.losses()

    params = ou.unpack(flat.astype(np.float64))
    x0 = ou.input_features(vols, [1.0, 1.0, 1.0], [1, 0, 1])
    T, Wt = torch.from_numpy(target).double(), torch.from_numpy(weight).double()
    acts = ou.forward(params, x0, bf16=True)
    g_or, lm_o, ls_o = ou.backward(params, acts, T, Wt, bf16=True)
    g_ref = ou.flat_grads(g_or)
    pred = net.workspace(dims, train=True).pred.cpu().double().reshape(2, *dims)
    ga = ou.flat_grads(ou.autograd_grads(params, x0, T, Wt))
    errs = {"pred": _nrm(pred, acts["pred"]), "loss_mu": abs(lm - lm_o) / lm_o, "loss_s": abs(ls - ls_o) / ls_o,
            "all": _nrm(g_gpu, g_ref), "all_autograd": _nrm(g_gpu, ga), "layers": {}}
    o = 0
    for name, ci, co in ou.LAYERS:
        n = co * ci * 27 + co
        errs["layers"][name] = (_nrm(g_gpu[o:o + n], g_ref[o:o + n]), _nrm(g_gpu[o:o + n], ga[o:o + n]))
        o += n
    errs["head"] = _nrm(g_gpu[o:], g_ref[o:])
    print(f"network {dims}: {errs}")
    # BF16 storage between 14 layers: the tensor core's FP32 accumulation order
    # flips some BF16 roundings relative to FP64, and the flips compound
    assert errs["pred"] <= 1e-2 and errs["loss_mu"] <= 1e-2 and errs["loss_s"] <= 1e-2, errs
    assert errs["all"] <= 3e-2 and errs["all_autograd"] <= 1e-1, errs
    for name, (e, ea) in errs["layers"].items():
        assert e <= 1e-1 and ea <= 2.5e-1, (name, errs)
    assert errs["head"] <= 1e-2, errs


def test_adam_step(env):
    N, lc, lib, dev = env
    rng = np.random.default_rng(9)
    p = rng.normal(size=1000).astype(np.float32)
    g = rng.normal(size=1000).astype(np.float32)
    pd, gd = torch.from_numpy(p).to(dev), torch.from_numpy(g).to(dev)
    m, v = torch.zeros_like(pd), torch.zeros_like(pd)
    for step in (1, 2):
        N.check(lib.pvd_adam_step(pd.data_ptr(), gd.data_ptr(), m.data_ptr(), v.data_ptr(), 1000, 1e-2, 0.9, 0.999,
                                  1e-8, 0.01, step, None))
    ref = torch.from_numpy(p).double().requires_grad_(True)
    opt = torch.optim.AdamW([ref], lr=1e-2, betas=(0.9, 0.999), eps=1e-8, weight_decay=0.01)
    for _ in range(2):
        opt.zero_grad()
        ref.grad = torch.from_numpy(g).double()
        opt.step()
    # AdamW applies the decay as p *= (1 - lr wd) before the update; the kernel as lr wd p in the update
    assert _nrm(pd.cpu().double(), ref.detach()) <= 1e-5


def test_gradient_clip_and_running_mean_limit():
    """pvd_grad_clip: the global norm (FP64 partial sums) scales the gradients down to
    max_norm, and to spike_factor x the running mean of the earlier (limited) norms; a
    non-finite norm zeroes them (counted in work[1027], like the limited steps)."""
    from pyvoxeldosimetry_gb300 import _native as N
    lib = N.load()
    dev = torch.device("cuda", 0)
    g = torch.randn(100_003, generator=torch.Generator().manual_seed(1)).to(dev)
    work = torch.zeros(1028, device=dev)
    nrm = float(g.double().norm())
    g1 = g.clone()
    N.check(lib.pvd_grad_clip(g1.data_ptr(), g1.numel(), 1.0, 10.0, work.data_ptr(), None))
    torch.cuda.synchronize()
    assert abs(float(work[1024]) - nrm) <= 1e-5 * nrm
    assert torch.allclose(g1, g / nrm, rtol=1e-5, atol=1e-9)
    assert abs(float(work[1026]) - 1.0) <= 1e-6          # running mean of the limited norms
    g2 = g * (0.5 / nrm)                                  # below both limits: untouched
    ref2 = g2.clone()
    N.check(lib.pvd_grad_clip(g2.data_ptr(), g2.numel(), 100.0, 10.0, work.data_ptr(), None))
    assert torch.equal(g2, ref2)
    mean = float(work[1026])
    g3 = g * (1000.0 / nrm)                               # a spike: cut to 10 x the running mean, direction kept
    N.check(lib.pvd_grad_clip(g3.data_ptr(), g3.numel(), 1e6, 10.0, work.data_ptr(), None))
    torch.cuda.synchronize()
    assert abs(float(g3.double().norm()) - 10.0 * mean) <= 1e-4 * 10.0 * mean and float(work[1027]) == 1.0
    assert torch.allclose(g3 / g3.norm(), g / g.norm(), rtol=1e-4, atol=1e-7)
    g4 = g.clone()
    g4[7] = float("nan")                                  # non-finite: zeroed, NaN not propagated
    N.check(lib.pvd_grad_clip(g4.data_ptr(), g4.numel(), 1.0, 0.0, work.data_ptr(), None))
    torch.cuda.synchronize()
    assert float(g4.abs().max()) == 0.0 and not torch.isnan(g4).any() and float(work[1027]) == 2.0
    assert lib.pvd_grad_clip(g.data_ptr(), g.numel(), 0.0, 1.0, work.data_ptr(), None) == 1


def test_graph_replayed_training_matches_eager(env):
    """train(graphs=True) replays the forward pass and the layer backward as CUDA
    graphs; every reduction in a step has a fixed order, so the parameters after a few
    steps equal those of the eager loop bit for bit (focused crops, a crop that fits)."""
    N, lc, lib, dev = env
    shape = (24, 32, 24)
    rng = np.random.default_rng(8)
    act = rng.random(shape).astype(np.float32)
    rho = (0.3 + rng.random(shape)).astype(np.float32)
    dc = (act * 0.01 + 1e-3).astype(np.float32)
    dm = (dc * np.exp(rng.normal(0.0, 0.1, shape))).astype(np.float32)
    pair = lc.make_pair(act, rho, dc, dm, device=dev)
    nets = []
    for graphs in (False, True):
        net = lc.UNet3D(seed=2, device=dev)
        lc.train(net, [pair], 6, crop=(16, 16, 16), lr=1e-3, seed=1, graphs=graphs)
        net.status()
        nets.append(net)
    assert torch.equal(nets[0].params, nets[1].params)
    assert not torch.equal(nets[0].params, lc.UNet3D(seed=2, device=dev).params)   # the steps did move them
    # inference after graph training packs the final weights
    a, r, d = (torch.from_numpy(x).to(dev) for x in (act, rho, dc))
    assert torch.equal(lc.predict(nets[0], a, r, d, sigma_max=float("inf")),
                       lc.predict(nets[1], a, r, d, sigma_max=float("inf")))
