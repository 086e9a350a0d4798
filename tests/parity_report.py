"""Errors of the CUDA path against the float64 oracle of the same method, for
the record (the parity tests assert the bounds; this prints the values).

    python tests/parity_report.py

Workloads: 16 chains of the 90x90 configuration (ss=2, 41x41 supersampled
PSF, EPL(50)+shear, SersicEllipse lens light and source, the configuration's
parameter distributions) through simulate and the fused likelihood +
gradient; 6 chains of the least-squares configuration (100x100, 45 shapelet
channels) through lstsq_simulate."""
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from gigalens_gb300 import _native as N  # noqa: E402
from gigalens_gb300 import workloads as W  # noqa: E402
from oracle import lens_oracle as O  # noqa: E402
from tests.helpers import ORACLE_MODEL, flat_from_struct  # noqa: E402


def fused_errors(bs=16):
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    phys, cfg = W.physical_model(), W.config1()
    ksub = np.asarray(cfg.kernel_supersampled, np.float64)
    ocfg = O.SimConfig(W.DELTA_PIX, 90, 2, ksub)
    truth = W.draw_params(1, seed=0)
    im_t = O.simulate(ORACLE_MODEL, ocfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in truth])
    obs = (im_t[0].numpy() + np.random.default_rng(0).normal(scale=W.BG_RMS, size=(90, 90))).astype(np.float32)
    pm = ForwardProbModel(W.config_prior(), obs, background_rms=W.BG_RMS, exp_time=W.EXP_TIME)
    sim = LensSimulator(phys, cfg, bs=bs)
    xs = W.draw_params(bs, seed=5)
    img = sim.simulate(xs).double().cpu()
    ref = O.simulate(ORACLE_MODEL, ocfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in xs])
    img = img.reshape(ref.shape)
    m = ref.abs().amax(dim=(-2, -1), keepdim=True)
    img_rel_max = float(((img - ref).abs() / m).max())
    big = ref.abs() > 1e-3 * m
    img_rel_pix = float(((img - ref).abs() / ref.abs())[big].max())
    # the same restatement evaluated in float32 (the reference's precision)
    ref32 = O.simulate(ORACLE_MODEL, ocfg, [[{k: v.float() for k, v in d.items()} for d in g] for g in xs],
                       dtype=torch.float32).double()
    img32_rel_max = float(((ref32 - ref).abs() / m).max())
    img32_rel_pix = float(((ref32 - ref).abs() / ref.abs())[big].max())
    plan = sim.prob_plan(pm)
    x = flat_from_struct(xs).float().cuda().contiguous()
    logL, chi2, grad = torch.empty(bs, device="cuda"), torch.empty(bs, device="cuda"), torch.empty_like(x)
    N.call("gl_forward_grad", plan.handle, N.ptr(x), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad), None,
           N.stream_ptr())
    torch.cuda.synchronize()
    xx = x.double().cpu().requires_grad_(True)
    ll, c2 = O.forward_log_likelihood_flat(ORACLE_MODEL, ocfg, xx, obs.astype(np.float64), W.BG_RMS, W.EXP_TIME)
    (g,) = torch.autograd.grad(ll.sum(), xx)
    ll, c2 = ll.detach(), c2.detach()
    gk = grad.double().cpu()
    floor = 1e-2 * g.pow(2).mean(dim=0, keepdim=True).sqrt()
    grel = (gk - g).abs() / torch.maximum(g.abs(), floor)
    x32 = x.cpu().clone().requires_grad_(True)
    l32, _ = O.forward_log_likelihood_flat(ORACLE_MODEL, ocfg, x32, obs, W.BG_RMS, W.EXP_TIME, dtype=torch.float32)
    (g32,) = torch.autograd.grad(l32.sum(), x32)
    grel32 = (g32.double() - g).abs() / torch.maximum(g.abs(), floor)
    return {
        "image: max |err| / max|image|": img_rel_max,
        "image: max relative error per pixel (pixels above 1e-3 of the max)": img_rel_pix,
        "  float32 restatement, image: max |err| / max|image|": img32_rel_max,
        "  float32 restatement, image: max relative error per pixel": img32_rel_pix,
        "  float32 restatement, gradient: max relative error per component": float(grel32.max()),
        "logL: max relative error": float(((logL.double().cpu() - ll).abs() / ll.abs()).max()),
        "chi^2: max relative error": float(((chi2.double().cpu() - c2).abs() / c2.abs()).max()),
        "gradient: median relative error per component": float(grel.median()),
        "gradient: 99th percentile relative error per component": float(torch.quantile(grel.flatten(), 0.99)),
        "gradient: max relative error per component": float(grel.max()),
    }


def lstsq_errors(bs=6):
    from gigalens_gb300.model import PhysicalModel
    from gigalens_gb300.simulator import SimulatorConfig
    from gigalens_gb300.cuda.profiles.light import shapelets
    from gigalens_gb300.cuda.profiles.mass import epl, shear
    from gigalens_gb300.cuda.simulator import LensSimulator

    n, n_max = 100, 8
    phys = PhysicalModel([epl.EPL(50), shear.Shear()], [], [shapelets.Shapelets(n_max, use_lstsq=True,
                                                                                interpolate=False)])
    omodel = dict(lenses=[("EPL", {"niter": 50}), ("SHEAR", {})], lens_light=[],
                  source_light=[("SHAPELETS", {"n_max": n_max})])
    ksub = W.gaussian_psf(W.FWHM, W.DELTA_PIX / 2, 21)
    cfg = SimulatorConfig(delta_pix=W.DELTA_PIX, num_pix=n, supersample=2, kernel_supersampled=ksub)
    ocfg = O.SimConfig(W.DELTA_PIX, n, 2, ksub.astype(np.float64))
    rng = np.random.default_rng(3)
    obs = (rng.normal(scale=0.1, size=(n, n)) + 0.5).astype(np.float32)
    err = np.sqrt(0.1 ** 2 + np.clip(obs, 0, None) / 200.0).astype(np.float32)
    lens = W.draw_params(bs, seed=4)[0]
    src = {"beta": torch.tensor(rng.uniform(0.05, 0.2, bs), dtype=torch.float32),
           "center_x": torch.tensor(rng.normal(0, 0.05, bs), dtype=torch.float32),
           "center_y": torch.tensor(rng.normal(0, 0.05, bs), dtype=torch.float32)}
    xs = [[lens[0], lens[1]], [src]]
    img = LensSimulator(phys, cfg, bs=bs).lstsq_simulate(xs, obs, err).double().cpu()
    ox = [[{k: v.double() for k, v in d.items()} for d in g] for g in xs]
    ref = O.lstsq_simulate(omodel, ocfg, ox, obs.astype(np.float64), err.astype(np.float64))
    img = img.reshape(ref.shape)
    m = ref.abs().amax(dim=(-2, -1), keepdim=True)
    return {"lstsq image: max |err| / max|image|": float(((img - ref).abs() / m).max())}


def main():
    torch.cuda.set_device(0)
    for name, v in list(fused_errors().items()) + list(lstsq_errors().items()):
        print("%-72s %.3g" % (name, v))


if __name__ == "__main__":
    main()
