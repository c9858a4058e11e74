"""What the learned correction gains: trained on this package's own Monte Carlo
/ convolution pairs, the network's corrected dose is compared with the plain
density-scaled convolution on held-out phantoms, both judged against a Monte
Carlo run with 5x the training histories (tissue voxels above 10 % of the
tissue maximum)."""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_trained_network_beats_plain_convolution():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from pyvoxeldosimetry_gb300.core import learned_correction as lc

    shape, vox = (48, 48, 48), 4.0
    train_pairs = lc.generate_training_pairs(12, shape, vox, "Y90", histories=20_000_000, seed=100)
    held = lc.generate_training_pairs(2, shape, vox, "Y90", histories=100_000_000, seed=900)
    net = lc.UNet3D(seed=0)
    stats = lc.train(net, train_pairs, steps=1500, crop=(48, 48, 48), lr=1e-3, log_every=100)
    report = {"train_seconds": stats.seconds, "loss_mu": stats.loss_mu, "held_out": []}
    for p in held:
        corrected, fb = lc.predict(net, p.activity, p.density, p.dose_conv, sigma_max=float("inf"),
                                   return_fallback=True)
        net.status()
        mc = p.dose_mc.cpu().numpy()
        rho = p.density.cpu().numpy()
        plain = lc.dose_errors(p.dose_conv.cpu().numpy(), mc, density=rho)
        corr = lc.dose_errors(corrected.cpu().numpy(), mc, density=rho)
        report["held_out"].append({"plain": plain, "corrected": corr})
        assert int(fb.sum()) == 0
        assert corr["mean"] < 0.5 * plain["mean"], report
        assert corr["within_3pct"] > plain["within_3pct"], report
    out = os.environ.get("PVD_REPORT_DIR")
    if out:
        with open(os.path.join(out, "unet_training_report.json"), "w") as f:
            json.dump(report, f, indent=1)
    print(json.dumps(report))
