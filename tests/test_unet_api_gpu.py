"""The NN-corrected dose behind the reference's calculator API: routing through
DoseCalculator(method='nn_corrected'), numpy in / numpy out, the fallback to the
plain convolution, the corrected-dose epilogue against its definition, and the
model file round trip."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from pyvoxeldosimetry_gb300 import phantoms
    from pyvoxeldosimetry_gb300.core import learned_correction as lc
    net = lc.UNet3D(seed=3)
    path = str(tmp_path_factory.mktemp("model") / "unet.npz")
    lc.save_model(net, path)
    act, rho = phantoms.ct_phantom((36, 40, 44), 4.0, seed=21)  # not multiples of 8: the crop overhangs
    return lc, net, path, act, rho


def test_fallback_everywhere_returns_the_plain_convolution(setup):
    lc, net, path, act, rho = setup
    from pyvoxeldosimetry_gb300 import DoseCalculator, KernelConvolutionCalculator
    vox = (4.0, 4.0, 4.0)
    # the corrected calculator convolves at the energy per decay of the Monte Carlo it was trained against
    plain = KernelConvolutionCalculator("Y90", config=lc.mc_consistent_config("Y90")).calculate_dose_rate(
        act, vox, density=rho)
    calc = DoseCalculator("Y90", method="nn_corrected", config={"model_path": path, "sigma_max": 0.0})
    res = calc.calculate_dose(activity_maps=[act], voxel_size=vox, tissue_densities=rho)
    d = res.dose_rate_maps[0]
    assert isinstance(d, np.ndarray) and d.shape == act.shape and d.dtype == np.float32
    assert np.array_equal(d, plain)
    assert calc.calculator.fallback_fraction() == 1.0


def test_corrected_dose_is_conv_times_exp_mu(setup):
    lc, net, path, act, rho = setup
    from pyvoxeldosimetry_gb300.core.kernel_convolution import KernelConvolutionCalculator
    dev = torch.device("cuda", 0)
    a, r = torch.from_numpy(act).to(dev), torch.from_numpy(rho).to(dev)
    dc = KernelConvolutionCalculator("Y90").calculate_dose_rate(a, (4.0, 4.0, 4.0), density=r)
    out, fb = lc.predict(net, a, r, dc, sigma_max=float("inf"), mu_clamp=3.0, return_fallback=True)
    net.status()
    crop = tuple(-(-n // 8) * 8 for n in act.shape)
    pred = net.workspace(crop, train=False).pred.reshape(2, *crop)[:, :act.shape[0], :act.shape[1], :act.shape[2]]
    expect = dc * torch.exp(torch.clamp(pred[0], -3.0, 3.0))
    assert int(fb.sum()) == 0
    assert torch.allclose(out, expect, rtol=1e-6, atol=0.0)
    # a loaded model gives the same dose
    net2 = lc.load_model(path)
    out2 = lc.predict(net2, a, r, dc, sigma_max=float("inf"))
    net2.status()
    assert torch.equal(out, out2)


def test_without_density_the_plain_convolution_is_returned(setup):
    lc, net, path, act, rho = setup
    from pyvoxeldosimetry_gb300 import KernelConvolutionCalculator, NNCorrectedDoseCalculator
    vox = (4.0, 4.0, 4.0)
    calc = NNCorrectedDoseCalculator("Y90", config={"model": net})
    assert np.array_equal(calc.calculate_dose_rate(act, vox),
                          KernelConvolutionCalculator("Y90", config=lc.mc_consistent_config("Y90"))
                          .calculate_dose_rate(act, vox))


def _transform(v, code, lc):
    perm, flips = lc.symmetry(code)
    u = np.transpose(v, perm)
    return np.ascontiguousarray(np.flip(u, flips) if flips else u)


def _untransform(u, code, lc):
    perm, flips = lc.symmetry(code)
    u = np.flip(u, flips) if flips else u
    return np.ascontiguousarray(np.transpose(u, np.argsort(perm)))


def test_pack_input_sym_reads_the_transformed_volume(setup):
    """pvd_unet_pack_input_sym of V equals pvd_unet_pack_input of numpy's transformed
    copy U = flip(transpose(V, perm)), bit for bit, for all 48 codes (uneven dims, a
    crop that overhangs U, a non-zero origin)."""
    lc, net, path, act, rho = setup
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    vols = [rng.random((5, 9, 13)).astype(np.float32) for _ in range(3)]
    vt = [torch.from_numpy(v).to(dev) for v in vols]
    s = torch.cuda.current_stream().cuda_stream
    for code in range(48):
        perm, _ = lc.symmetry(code)
        ushape = tuple(vols[0].shape[a] for a in perm)
        ws = net.workspace((16, 16, 16), train=False)
        origin = (-1, 2, 0)
        net.pack_input(ws, vt, (0.5, 1.0, 2.0), origin, s, sym=code)
        got = ws.t["x0"].to_dense().clone()
        ut = [torch.from_numpy(_transform(v, code, lc)).to(dev) for v in vols]
        assert tuple(ut[0].shape) == ushape
        net.pack_input(ws, ut, (0.5, 1.0, 2.0), origin, s)
        assert torch.equal(got, ws.t["x0"].to_dense()), code
    net.status()


def test_symmetry_accumulate_maps_back_to_the_volume_frame(setup):
    lc, net, path, act, rho = setup
    from pyvoxeldosimetry_gb300 import _native as N
    import ctypes as C
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(6)
    vd = (5, 9, 13)
    acc = torch.full((2, 8, 16, 16), -7.0, device=dev)
    ws0 = net.workspace((8, 16, 16), train=False)
    lib = N.load()
    vdc = (C.c_int * 3)(*vd)
    expect = np.full((2, 8, 16, 16), -7.0, np.float32)
    s = torch.cuda.current_stream().cuda_stream
    for k, code in enumerate((0, 5, 11, 22, 47)):
        perm, _ = lc.symmetry(code)
        crop_u = tuple(-(-vd[a] // 8) * 8 for a in perm)
        ws = net.workspace(crop_u, train=False)
        pred = rng.normal(size=(2, *crop_u)).astype(np.float32)
        pt = torch.from_numpy(pred).to(dev)
        N.check(lib.pvd_unet_symmetry_accumulate(C.byref(ws.geo[0]), pt.data_ptr(), C.byref(ws0.geo[0]), vdc, code,
                                                 0.125, int(k > 0), acc.data_ptr(), s))
        for c in range(2):
            u = pred[c][:crop_u[0], :crop_u[1], :crop_u[2]][tuple(slice(0, vd[a]) for a in perm)]
            back = _untransform(u, code, lc) * np.float32(0.125)   # exact: a power of two
            sub = expect[c, :vd[0], :vd[1], :vd[2]]
            expect[c, :vd[0], :vd[1], :vd[2]] = back if k == 0 else sub + back
    assert np.array_equal(acc.cpu().numpy(), expect)       # voxels outside V untouched (-7)
    with pytest.raises(N.PvdError):                         # a crop smaller than the volume
        N.check(lib.pvd_unet_symmetry_accumulate(C.byref(ws0.geo[0]), acc.data_ptr(), C.byref(ws0.geo[0]),
                                                 (C.c_int * 3)(9, 9, 9), 0, 1.0, 0, acc.data_ptr(), s))


def test_predict_averages_over_flips(setup):
    """predict(symmetries=8) is the mean of mu (and s) over the network run on the 8
    flipped volumes, each flipped back; the average is invariant under the group, so
    the corrected dose of a flipped volume is the flipped corrected dose."""
    lc, net, path, act, rho = setup
    dev = torch.device("cuda", 0)
    a, r = torch.from_numpy(act).to(dev), torch.from_numpy(rho).to(dev)
    dc = torch.from_numpy(np.ascontiguousarray(act * 1e-3 + 1e-4)).to(dev)
    out8 = lc.predict(net, a, r, dc, sigma_max=float("inf"), symmetries=8)
    # the passes on 1 or 3 side streams are summed in the same order: the same dose, bit for bit
    for n in (1, 3):
        assert torch.equal(lc.predict(net, a, r, dc, sigma_max=float("inf"), symmetries=8, streams=n), out8)
    crop = tuple(-(-n // 8) * 8 for n in act.shape)
    mus = []
    for code in range(8):
        _, flips = lc.symmetry(code)
        f = (lambda t: torch.flip(t, flips).contiguous()) if flips else (lambda t: t)
        lc.predict(net, f(a), f(r), f(dc), sigma_max=float("inf"))
        p = net.workspace(crop, train=False).pred.reshape(2, *crop)[0, :act.shape[0], :act.shape[1], :act.shape[2]]
        mus.append(torch.flip(p, flips) if flips else p.clone())
    mu = torch.zeros_like(mus[0])
    for m in mus:
        mu = mu + m * 0.125
    expect = dc * torch.exp(torch.clamp(mu, -3.0, 3.0))
    assert torch.allclose(out8, expect, rtol=2e-6, atol=0.0)
    flipped = lc.predict(net, torch.flip(a, (0, 2)).contiguous(), torch.flip(r, (0, 2)).contiguous(),
                         torch.flip(dc, (0, 2)).contiguous(), sigma_max=float("inf"), symmetries=8)
    assert torch.allclose(torch.flip(flipped, (0, 2)), out8, rtol=1e-5, atol=0.0)
    net.status()
    with pytest.raises(ValueError):
        lc.predict(net, a, r, dc, symmetries=4)


def test_head_loss_sym_reads_targets_in_the_flipped_frame(setup):
    """pvd_unet_head_loss_sym on a crop of the flipped volumes equals
    pvd_unet_head_loss on numpy's flipped copies (inputs, target and weight), bit for
    bit: the loss, the head's gradients and the gradient into the last layer."""
    lc, net, path, act, rho = setup
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(11)
    vd = (12, 18, 20)
    vols = [rng.random(vd).astype(np.float32) for _ in range(3)]
    tgt = rng.normal(0.0, 0.3, vd).astype(np.float32)
    wgt = (rng.random(vd) > 0.4).astype(np.float32)
    s = torch.cuda.current_stream().cuda_stream
    ws = net.workspace((16, 16, 16), train=True)
    origin = (-2, 1, 3)
    for code in (3, 5, 6):
        _, flips = lc.symmetry(code)
        outs = []
        for sym, vv, tt, ww in ((code, vols, tgt, wgt),
                                (0, [np.ascontiguousarray(np.flip(v, flips)) for v in vols],
                                 np.ascontiguousarray(np.flip(tgt, flips)), np.ascontiguousarray(np.flip(wgt, flips)))):
            vt = [torch.from_numpy(v).to(dev) for v in vv]
            net.pack_input(ws, vt, (1.0, 1.0, 1.0), origin, s, sym=sym)
            net.forward(ws, s)
            net.head_loss(ws, torch.from_numpy(tt).to(dev), torch.from_numpy(ww).to(dev), origin, s, sym=sym)
            outs.append((net.grads[net.head_offset:].clone(), ws.gr["d0b"].to_dense().clone()))
        assert torch.equal(outs[0][0], outs[1][0]), code
        assert torch.equal(outs[0][1], outs[1][1]), code
    net.status()
