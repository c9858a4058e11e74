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
