"""Parity on the benchmark configurations' own inputs, against the float32
restatement of the reference's path (the reference's own precision) and
against the float64 oracle of the same method.

Inputs: parameters drawn from the configurations' distributions
(``workloads.draw_params``: sources down to R = 0.05" and n up to 4, lens
light n up to 6), observed image = a seeded truth draw with Poisson noise at
1000 s and Gaussian background 0.2.
  * configuration 0 shape: 60x60 px, ss = 2, 21x21 supersampled PSF, 64 chains;
  * configuration 1 shape: 90x90 px, ss = 2, 41x41 supersampled PSF, 32 chains.

Bars (spec: images 1e-5 relative per pixel, logL 1e-4 relative,
gradients 1e-3 relative per component, each against the reference's float32
path):
  * logL / log posterior: 1e-4 relative against the float32 restatement AND
    against float64, every chain, no absolute term.
  * chi^2: 1e-4 relative, the same two comparisons.
  * images, pixels above 1e-3 of their image's maximum, no absolute term:
      - against float32: |cuda - f32| <= 1e-5 |f32| on at least 99.9 % of
        the pixels (the fraction is printed and asserted);
      - against float64, every pixel: |cuda - f64| <= 1e-5 |f64| + 2 band,
        where band = the largest |image with float32 ray shooting - float64
        image| at the input and at eight 1-ulp perturbations of the lens
        parameters (oracle): the reference's own float32 deflection error,
        amplified where a lensed source cusp is steep.  It is the whole of
        the float32 restatement's image error (light, PSF and binning in
        float32 add less than 1e-6); near such cusps a 1-ulp change of the
        lens parameters moves a pixel by up to ~5e-5.  The number of pixels
        that need the band term (at most 0.1 %) and their largest relative
        error (at most 2e-4) are printed and asserted.
  * gradients, per component relative to max(|g|, 1e-2 rms over chains):
      - against float32: within 1e-3 on at least 97 % of the components;
      - against float64: within 1e-3, or within twice the float32 noise band
        of the reference's own arithmetic (the float32 restatement's
        gradient at the input and at 1-ulp perturbations of it); the number
        of components that need the band (at most 2 %) and their largest
        relative error (at most 1e-2) are printed and asserted, and the
        kernel's largest error stays inside twice the band's largest value.
"""
import math

import numpy as np
import pytest
import torch

from gigalens_gb300 import _native as N
from gigalens_gb300 import workloads as W
from oracle import lens_oracle as O
from tests.helpers import ORACLE_MODEL, flat_from_struct

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

CASES = {
    "config0_60px_psf21": dict(n=60, psf_base=11, bs=64, seed=10),
    "config1_90px_psf41": dict(n=90, psf_base=21, bs=32, seed=11),
}
PIX_FRACTION = 1e-3      # images: pixels above this fraction of their image's maximum
_cache = {}


def _case(name):
    if name in _cache:
        return _cache[name]
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    c = CASES[name]
    n, bs = c["n"], c["bs"]
    cfg = W.sim_config(n, c["psf_base"])
    ocfg = O.SimConfig(W.DELTA_PIX, n, 2, np.asarray(cfg.kernel_supersampled, np.float64))
    truth = W.draw_params(1, seed=c["seed"] + 1000)
    im_t = O.simulate(ORACLE_MODEL, ocfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in truth])
    obs = W.observe(im_t.float(), seed=c["seed"])[0].numpy().astype(np.float32)
    prior = W.config_prior()
    pm = ForwardProbModel(prior, obs, background_rms=W.BG_RMS, exp_time=W.EXP_TIME)
    sim = LensSimulator(W.physical_model(), cfg, bs=bs)
    xs = W.draw_params(bs, seed=c["seed"])
    x = flat_from_struct(xs).float().contiguous()
    out = dict(n=n, bs=bs, cfg=cfg, ocfg=ocfg, obs=obs, prior=prior, pm=pm, sim=sim, xs=xs, x=x)
    # CUDA: image, logL, chi^2, gradient
    xd = x.cuda()
    out["img"] = sim.simulate_flat(xd).double().cpu()
    plan = sim.prob_plan(pm)
    logL, chi2, grad = torch.empty(bs, device="cuda"), torch.empty(bs, device="cuda"), torch.empty_like(xd)
    N.call("gl_forward_grad", plan.handle, N.ptr(xd), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad), None,
           N.stream_ptr())
    torch.cuda.synchronize()
    out["logL"], out["chi2"], out["grad"] = logL.double().cpu(), chi2.double().cpu(), grad.double().cpu()
    # oracle: float64, float32 (the reference's precision), float32 ray shooting only
    x64 = x.double()
    p64 = O.unflatten(ORACLE_MODEL, x64)
    out["ref64"] = O.simulate(ORACLE_MODEL, ocfg, p64)
    out["ref32"] = O.simulate(ORACLE_MODEL, ocfg, O.unflatten(ORACLE_MODEL, x), dtype=torch.float32).double()
    # float32 noise band of the image: ray shooting in float32 (the rest in
    # float64) at the input and at eight 1-ulp perturbations of the lens
    # parameters, the largest deviation from float64 per pixel
    r = np.random.default_rng(1)
    n_lens = 8
    rband = torch.zeros_like(out["ref64"])
    for i in range(9):
        xq = x64.clone()
        if i:
            pert = r.choice([-1.0, 0.0, 1.0], size=(bs, n_lens)) * 2.0 ** -23
            xq[:, :n_lens] = (x[:, :n_lens] * (1 + torch.tensor(pert, dtype=torch.float32))).double()
        im = O.simulate(ORACLE_MODEL, ocfg, O.unflatten(ORACLE_MODEL, xq), ray_dtype=torch.float32)
        if i == 0:
            out["refray32"] = im
        rband = torch.maximum(rband, (im - out["ref64"]).abs())
    out["rband"] = rband
    xx = x64.clone().requires_grad_(True)
    ll, c2 = O.forward_log_likelihood_flat(ORACLE_MODEL, ocfg, xx, obs.astype(np.float64), W.BG_RMS, W.EXP_TIME)
    (g64,) = torch.autograd.grad(ll.sum(), xx)
    out["ll64"], out["c264"], out["g64"] = ll.detach(), c2.detach(), g64
    x32 = x.clone().requires_grad_(True)
    l32, c32 = O.forward_log_likelihood_flat(ORACLE_MODEL, ocfg, x32, obs, W.BG_RMS, W.EXP_TIME, dtype=torch.float32)
    (g32,) = torch.autograd.grad(l32.sum(), x32)
    out["ll32"], out["c232"], out["g32"] = l32.detach().double(), c32.detach().double(), g32.double()
    # float32 noise band of the gradient: the restatement at the input and at
    # four 1-ulp perturbations of it
    r = np.random.default_rng(0)
    band = (g32.double() - g64).abs()
    for _ in range(4):
        pert = torch.tensor(r.choice([-1.0, 0.0, 1.0], size=tuple(x.shape)) * 2.0 ** -23, dtype=torch.float32)
        xp = (x * (1 + pert)).detach().requires_grad_(True)
        lp, _ = O.forward_log_likelihood_flat(ORACLE_MODEL, ocfg, xp, obs, W.BG_RMS, W.EXP_TIME, dtype=torch.float32)
        (gp,) = torch.autograd.grad(lp.sum(), xp)
        band = torch.maximum(band, (gp.double() - g64).abs())
    out["gband"] = band
    _cache[name] = out
    return out


def _rel(a, b):
    return (a - b).abs() / b.abs()


@pytest.mark.parametrize("name", list(CASES))
def test_loglik_and_chi2_against_float32_and_float64(name):
    s = _case(name)
    r32, r64 = _rel(s["logL"], s["ll32"]), _rel(s["logL"], s["ll64"])
    c32, c64 = _rel(s["chi2"], s["c232"]), _rel(s["chi2"], s["c264"])
    print("\n[%s] logL max rel: vs float32 %.2e, vs float64 %.2e (float32 restatement vs float64 %.2e); "
          "chi2: %.2e / %.2e" % (name, float(r32.max()), float(r64.max()), float(_rel(s["ll32"], s["ll64"]).max()),
                                 float(c32.max()), float(c64.max())))
    assert float(r32.max()) <= 1e-4 and float(r64.max()) <= 1e-4
    assert float(c32.max()) <= 1e-4 and float(c64.max()) <= 1e-4


@pytest.mark.parametrize("name", list(CASES))
def test_log_prob_against_float32_restatement(name):
    """ForwardProbModel.log_prob (tf/model.py:53-86, prior and bijector
    log-Jacobian included) through the public API, against the float32 and
    float64 restatements on the configuration's prior."""
    s = _case(name)
    pm, prior = s["pm"], s["prior"]
    z = pm.bij.inverse(s["xs"]).float()
    logp, _ = pm.log_prob(s["sim"], z.cuda())
    logp = logp.double().cpu()
    for dt in (torch.float64, torch.float32):
        zc = z.to(dt)
        xs = pm.bij.forward(zc)
        ll, _ = O.forward_log_likelihood_flat(ORACLE_MODEL, s["ocfg"], flat_from_struct(xs),
                                              s["obs"].astype(np.float64) if dt == torch.float64 else s["obs"],
                                              W.BG_RMS, W.EXP_TIME, dtype=dt)
        lp = (ll + prior.log_prob(xs) + pm.unconstraining_bij.forward_log_det_jacobian(pm.pack_bij.forward(zc))).double()
        rel = _rel(logp, lp)
        print("\n[%s] log_prob max rel vs %s: %.2e" % (name, str(dt)[6:], float(rel.max())))
        assert float(rel.max()) <= 1e-4


@pytest.mark.parametrize("name", list(CASES))
def test_images_against_float32_and_float64(name):
    s = _case(name)
    img, r32, r64, rray, band = s["img"], s["ref32"], s["ref64"], s["refray32"], s["rband"]
    m = r64.abs().amax(dim=(-2, -1), keepdim=True)
    sel = r64.abs() > PIX_FRACTION * m
    # against the float32 restatement (the literal bar)
    rel32 = _rel(img, r32)[sel]
    ok32 = float((rel32 <= 1e-5).double().mean())
    # against float64, with the band of the reference's own float32 ray shooting
    err64 = (img - r64).abs()
    lit64 = err64 <= 1e-5 * r64.abs()
    ok64 = err64 <= 1e-5 * r64.abs() + 2.0 * band
    need = sel & ~lit64
    rel64 = (err64 / r64.abs())[sel]
    ref_rel = _rel(r32, r64)[sel]
    print("\n[%s] image pixels above %.0e of max: %d; vs float32: %.4f %% within 1e-5 (max rel %.2e); "
          "vs float64: max rel %.2e (float32 restatement %.2e, its ray shooting alone %.2e); "
          "%d pixels (%.4f %%) need the float32 ray-shooting band, max rel among them %.2e"
          % (name, PIX_FRACTION, int(sel.sum()), 100 * ok32, float(rel32.max()), float(rel64.max()),
             float(ref_rel.max()), float(_rel(rray, r64)[sel].max()), int(need.sum()),
             100.0 * float(need.sum()) / float(sel.sum()), float((err64 / r64.abs())[need].max()) if need.any() else 0.0))
    print("[%s] float32 ray-shooting band: largest relative value %.2e" % (
        name, float((band / r64.abs())[sel].max())))
    assert ok32 >= 0.999
    assert bool(ok64[sel].all())
    assert float(need.sum()) <= 1e-3 * float(sel.sum())
    assert float(rel64.max()) <= 2e-4


@pytest.mark.parametrize("name", list(CASES))
def test_gradients_against_float32_and_float64(name):
    s = _case(name)
    g, g32, g64, band = s["grad"], s["g32"], s["g64"], s["gband"]
    floor = 1e-2 * g64.pow(2).mean(dim=0, keepdim=True).sqrt()
    scale = torch.maximum(g64.abs(), floor)
    rel32 = (g - g32).abs() / scale
    rel64 = (g - g64).abs() / scale
    ref_rel = (g32 - g64).abs() / scale
    ok32 = float((rel32 <= 1e-3).double().mean())
    lit = rel64 <= 1e-3
    ok = lit | ((g - g64).abs() <= 2.0 * band)
    need = ~lit
    worst = tuple(int(v) for v in divmod(int(rel64.argmax()), g.shape[1]))
    print("\n[%s] gradient components: %d; vs float32: %.2f %% within 1e-3 (max rel %.2e); vs float64: "
          "median %.1e, p99 %.1e, max %.2e at (chain, column) %s (float32 restatement max %.2e); %d components "
          "(%.2f %%) need the float32 band, max rel among them %.2e"
          % (name, g.numel(), 100 * ok32, float(rel32.max()), float(rel64.median()),
             float(torch.quantile(rel64.flatten(), 0.99)), float(rel64.max()), worst, float(ref_rel.max()),
             int(need.sum()), 100.0 * float(need.sum()) / g.numel(),
             float(rel64[need].max()) if need.any() else 0.0))
    assert ok32 >= 0.97
    assert bool(ok.all())
    assert float(need.sum()) <= 0.02 * g.numel()
    assert float(rel64.max()) <= 1e-2
    # the kernel's largest error stays inside the reference's own float32
    # noise band (its float32 gradient over 1-ulp input perturbations)
    band_rel = float((band / scale).max())
    print("[%s] float32 noise band: largest relative value %.2e" % (name, band_rel))
    assert float(rel64.max()) <= 2.0 * band_rel + 1e-3


# ------------------------------------------------------------------ least squares, configuration 3 shape
def _lstsq_setup(n, bs, seed, n_max=8):
    from gigalens_gb300.model import PhysicalModel
    from gigalens_gb300.simulator import SimulatorConfig
    from gigalens_gb300.cuda.profiles.light import shapelets
    from gigalens_gb300.cuda.profiles.mass import epl, shear

    phys = PhysicalModel([epl.EPL(50), shear.Shear()], [],
                         [shapelets.Shapelets(n_max, use_lstsq=True, interpolate=False)])
    omodel = dict(lenses=[("EPL", {"niter": 50}), ("SHEAR", {})], lens_light=[],
                  source_light=[("SHAPELETS", {"n_max": n_max})])
    ksub = W.gaussian_psf(W.FWHM, W.DELTA_PIX / 2, 21)
    cfg = SimulatorConfig(delta_pix=W.DELTA_PIX, num_pix=n, supersample=2, kernel_supersampled=ksub)
    ocfg = O.SimConfig(W.DELTA_PIX, n, 2, ksub.astype(np.float64))
    rng = np.random.default_rng(seed)
    lens = W.draw_params(bs, seed=seed)[0]
    src = {"beta": torch.tensor(rng.uniform(0.05, 0.2, bs), dtype=torch.float32),
           "center_x": torch.tensor(rng.normal(0, 0.05, bs), dtype=torch.float32),
           "center_y": torch.tensor(rng.normal(0, 0.05, bs), dtype=torch.float32)}
    xs = [[lens[0], lens[1]], [src]]
    ox = [[{k: v.double() for k, v in d.items()} for d in g] for g in xs]
    # observation: a shapelet source through the first chain's lens, plus noise
    basis = O.lstsq_basis(omodel, ocfg, ox)[0]
    coef = torch.tensor(rng.normal(size=basis.shape[-1]) * 2.0) * torch.exp(-0.2 * torch.arange(basis.shape[-1]))
    truth = (basis * coef).sum(-1).numpy()
    obs = (truth + rng.normal(scale=W.BG_RMS, size=(n, n))).astype(np.float32)
    err = np.sqrt(W.BG_RMS ** 2 + np.clip(obs, 0, None) / W.EXP_TIME).astype(np.float32)
    return phys, omodel, cfg, ocfg, xs, ox, obs, err


def test_lstsq_configuration3_shape_uneven_batch():
    """100x100 px with n_max = 8 (45 channels) and a 60x60 image in one
    launch (img_id per chain), against the float64 oracle: images within 1e-5
    of their maximum, logL within 1e-4 relative (no absolute term)."""
    from gigalens_gb300.cuda._plan import ModelLayout, Plan
    from gigalens_gb300.cuda.simulator import LensSimulator
    import ctypes

    sets = [_lstsq_setup(100, 6, 3), _lstsq_setup(60, 3, 4)]
    lay = ModelLayout(sets[0][0])
    ims = [dict(sim_config=s[2], observed=s[6], err_map=s[7]) for s in sets]
    plan = Plan(lay, ims)
    x = torch.cat([lay.flatten_params(s[4]) for s in sets]).float().cuda().contiguous()
    img_id = torch.tensor([0] * 6 + [1] * 3, dtype=torch.int32, device="cuda")
    bs = x.shape[0]
    nb, D = ctypes.c_size_t(0), ctypes.c_int(0)
    N.call("gl_lstsq_workspace", plan.handle, bs, ctypes.byref(nb), ctypes.byref(D))
    assert D.value == 45
    work = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    co = torch.empty(bs, D.value, device="cuda")
    img = torch.empty(bs, plan.max_pix, device="cuda")
    lg, c2 = torch.empty(bs, device="cuda"), torch.empty(bs, device="cuda")
    N.call("gl_lstsq", plan.handle, N.ptr(x), N.ptr(img_id), bs, N.ptr(work), nb.value, N.ptr(co), N.ptr(img),
           N.ptr(lg), N.ptr(c2), N.stream_ptr())
    torch.cuda.synchronize()
    lo = 0
    for k, (phys, omodel, cfg, ocfg, xs, ox, obs, err) in enumerate(sets):
        n = cfg.num_pix
        nb_k = len(ox[0][0]["theta_E"])
        ref = O.lstsq_simulate(omodel, ocfg, ox, obs.astype(np.float64), err.astype(np.float64))
        got = img[lo:lo + nb_k, : n * n].double().cpu().reshape(ref.shape)
        m = ref.abs().amax(dim=(-2, -1), keepdim=True)
        rel_max = float(((got - ref).abs() / m).max())
        ll_ref, c2_ref = O.backward_log_likelihood(ref, obs.astype(np.float64), err.astype(np.float64))
        rl = float(_rel(lg[lo:lo + nb_k].double().cpu(), ll_ref).max())
        rc = float(_rel(c2[lo:lo + nb_k].double().cpu(), c2_ref).max())
        print("\n[lstsq %dpx] image max |err|/max %.2e, logL max rel %.2e, chi2 max rel %.2e" % (n, rel_max, rl, rc))
        assert rel_max <= 1e-5
        assert rl <= 1e-4 and rc <= 1e-4
        lo += nb_k
