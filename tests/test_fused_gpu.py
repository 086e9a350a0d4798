"""Parity of the fused CUDA path with the float64 oracle.

Tolerances (spec bar, per quantity, against the float64 restatement):
  images       pixels above 1e-3 of their image's maximum, no absolute
               term: |d| <= 1e-5 |ref|, or 1e-5 |ref| + 2 band on at most
               0.1 % of them (band = float32 ray-shooting noise of the
               reference's own arithmetic, ``helpers.image_band``), relative
               error at most 2e-4 there; fainter pixels |d| <= 1e-6 max|ref|
               (``helpers.check_images``, which prints the figures)
  logL, logp   |d| <= 1e-4 |ref|
  chi^2        |d| <= 1e-4 |ref|
  gradients    per component, either |d| <= 1e-3 max(|ref|, 1e-2 rms_batch(ref))
               or |d| <= 2 band, where band = max |g32 - ref| over the float32
               evaluation of the same restatement (the reference's own
               precision) at the input and at four 1-ulp perturbations of it.
               Components dominated by Sersic cusps (n > 1: the coordinate
               derivative diverges as R^(1/n - 1)) are float32-noise-limited.
               At most 2 % of the components may use the band, with a
               relative error of at most 1e-2; both are printed.
"""
import math

import numpy as np
import pytest
import torch

from gigalens_gb300 import _native as N
from gigalens_gb300 import distributions as tfd
from gigalens_gb300.model import PhysicalModel
from gigalens_gb300.simulator import SimulatorConfig
from oracle import lens_oracle as O
from tests.helpers import (ORACLE_MODEL, as_batch, check_images, default_physmodel, default_prior, demo_truth,
                           flat_from_struct, gaussian_psf, image_band, load_golden)

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def _setup(num_pix, ss, ksub, bs, seed=0, delta=0.065, phys=None, omodel=None, prior=None):
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    prior = prior or default_prior()
    phys = phys or default_physmodel()
    omodel = omodel or ORACLE_MODEL
    cfg = SimulatorConfig(delta_pix=delta, num_pix=num_pix, supersample=ss, kernel_supersampled=ksub)
    ocfg = O.SimConfig(delta, num_pix, ss, None if ksub is None else ksub.astype(np.float64))
    # observed image: truth draw + noise (float64 oracle)
    truth = prior.sample(1, seed=seed + 100)
    im_t = O.simulate(omodel, ocfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in truth])
    rng = np.random.default_rng(seed)
    obs = im_t[0].numpy() + rng.normal(scale=0.2, size=(num_pix, num_pix))
    pm = ForwardProbModel(prior, obs.astype(np.float32), background_rms=0.2, exp_time=1000.0)
    sim = LensSimulator(phys, cfg, bs=bs)
    x_struct = prior.sample(bs, seed=seed)
    return dict(prior=prior, cfg=cfg, ocfg=ocfg, obs=obs.astype(np.float32), pm=pm, sim=sim,
                x_struct=x_struct, omodel=omodel)


def _oracle_loglik(s, xflat64, with_fp32=True):
    """float64 logL, chi^2, gradient; and the float32 gradient of the same restatement."""
    x = xflat64.clone().requires_grad_(True)
    ll, chi2 = O.forward_log_likelihood_flat(s["omodel"], s["ocfg"], x, s["obs"].astype(np.float64), 0.2, 1000.0)
    (g,) = torch.autograd.grad(ll.sum(), x)
    band = None
    if with_fp32:
        band = fp32_band(lambda xx: O.forward_log_likelihood_flat(
            s["omodel"], s["ocfg"], xx, s["obs"], 0.2, 1000.0, dtype=torch.float32)[0], xflat64.float(), g)
    return ll.detach(), chi2.detach(), (g, band)


def fp32_band(fn, x32, g64, n_perturb=4, seed=0):
    """Float32 noise band of a gradient: max over the unperturbed input and
    ``n_perturb`` 1-ulp perturbations of |g32 - g64|, with g32 the gradient of
    the restatement evaluated in float32 (the reference's precision)."""
    r = np.random.default_rng(seed)
    worst = torch.zeros_like(g64)
    for i in range(n_perturb + 1):
        pert = 0.0 if i == 0 else torch.tensor(r.choice([-1.0, 0.0, 1.0], size=tuple(x32.shape)) * 2.0 ** -23,
                                               dtype=torch.float32)
        xx = (x32 * (1 + pert)).detach().requires_grad_(True)
        (g32,) = torch.autograd.grad(fn(xx).sum(), xx)
        worst = torch.maximum(worst, (g32.double() - g64).abs())
    return worst


def _check_images(got, ref, omodel, ocfg, xflat, name="image", **limits):
    check_images(got, ref, image_band(omodel, ocfg, xflat), name, **limits)


def _check_scalar(got, ref, rtol, name=""):
    got = got.double().cpu()
    rel = (got - ref).abs() / ref.abs()
    print("\n[%s] max rel %.2e" % (name, float(rel.max())))
    assert bool(((got - ref).abs() <= rtol * ref.abs()).all()), "%s mismatch: max rel %.3g" % (name, float(rel.max()))


def _check_grad(got, ref, name="grad", max_rel=1e-2):
    ref, band = ref if isinstance(ref, tuple) else (ref, None)
    got = got.double().cpu()
    floor = 1e-2 * ref.pow(2).mean(dim=0, keepdim=True).sqrt()
    scale = torch.maximum(ref.abs(), floor)
    err = (got - ref).abs()
    lit = err <= 1e-3 * scale
    ok = lit if band is None else lit | (err <= 2.0 * band)
    rel = err / scale
    need = ~lit
    print("\n[%s] %d components: max rel %.2e; %d (%.2f %%) use the float32 band, max rel among them %.2e" % (
        name, rel.numel(), float(rel.max()), int(need.sum()), 100.0 * float(need.sum()) / rel.numel(),
        float(rel[need].max()) if bool(need.any()) else 0.0))
    worst = divmod(int(rel.argmax()), rel.shape[1])
    if band is not None:
        print("[%s] worst component (sample, parameter) %s: rel %.2e, float32 band %.2e of the scale" % (
            name, worst, float(rel[worst]), float((band / scale)[worst])))
    bad = (~ok).nonzero()
    assert bool(ok.all()), "%s mismatch at %s: rel %.3g (float32 band rel %s)" % (
        name, tuple(bad[0].tolist()), float(rel[tuple(bad[0].tolist())]),
        "n/a" if band is None else "%.3g" % float((band / scale)[tuple(bad[0].tolist())]))
    assert float(need.sum()) <= max(0.02 * rel.numel(), 1.0), "%s: %d components use the band" % (name, int(need.sum()))
    assert float(rel.max()) <= max_rel, name


CONFIGS = {
    # name: (num_pix, ss, supersampled kernel side, bs)
    "config0_60px_ss2_psf21": (60, 2, 21, 13),
    "config1_90px_ss2_psf41": (90, 2, 41, 9),
    "ss1_psf13": (48, 1, 13, 5),
    "ss2_nopsf": (40, 2, 0, 4),
    # PSF sizes k = 3 mod 4 at ss = 2: even sub-kernels, shifted transposed correlation
    "ss2_psf11": (44, 2, 11, 5),
    "ss2_psf23": (36, 2, 23, 4),
    # planes larger than a CTA's shared memory: per-CTA slices of global memory
    "gmem_100px_ss2_psf21": (100, 2, 21, 3),
    # the largest sub-kernel the kernels compile (side 25)
    "max_subkernel_ss2_psf49": (24, 2, 49, 3),
    "max_subkernel_ss1_psf25": (30, 1, 25, 3),
}


@pytest.mark.parametrize("name", list(CONFIGS))
def test_simulate_matches_oracle(name):
    n, ss, k, bs = CONFIGS[name]
    ksub = gaussian_psf(0.1, 0.065 / ss, k) if k else None
    s = _setup(n, ss, ksub, bs)
    img = s["sim"].simulate(s["x_struct"])
    ref = O.simulate(ORACLE_MODEL, s["ocfg"], [[{kk: v.double() for kk, v in d.items()} for d in g]
                                               for g in s["x_struct"]])
    _check_images(img.reshape(ref.shape), ref, ORACLE_MODEL, s["ocfg"], flat_from_struct(s["x_struct"]), name)


@pytest.mark.parametrize("name", list(CONFIGS))
def test_loglik_chi2_grad_match_oracle(name):
    n, ss, k, bs = CONFIGS[name]
    ksub = gaussian_psf(0.1, 0.065 / ss, k) if k else None
    s = _setup(n, ss, ksub, bs)
    plan = s["sim"].prob_plan(s["pm"])
    x = flat_from_struct(s["x_struct"]).float().cuda().contiguous()
    logL = torch.empty(bs, device="cuda")
    chi2 = torch.empty(bs, device="cuda")
    grad = torch.empty_like(x)
    N.call("gl_forward_grad", plan.handle, N.ptr(x), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad), None,
           N.stream_ptr())
    torch.cuda.synchronize()
    ll, c2, g = _oracle_loglik(s, x.double().cpu())
    _check_scalar(logL, ll, 1e-4, name="logL")
    _check_scalar(chi2, c2, 1e-4, name="chi2")
    _check_grad(grad, g)
    # value-only path gives the same logL and chi^2
    logL2 = torch.empty(bs, device="cuda")
    chi22 = torch.empty(bs, device="cuda")
    N.call("gl_forward", plan.handle, N.ptr(x), None, bs, N.ptr(logL2), N.ptr(chi22), None, None, N.stream_ptr())
    torch.cuda.synchronize()
    assert torch.equal(logL2, logL) and torch.equal(chi22, chi2)


def test_log_prob_and_autograd_match_oracle():
    """ForwardProbModel.log_prob (tf/model.py:53-86) incl. prior and bijector log-Jacobian."""
    s = _setup(60, 2, gaussian_psf(0.1, 0.0325, 21), 11, seed=5)
    pm, prior = s["pm"], s["prior"]
    z = pm.bij.inverse(s["x_struct"]).float().cuda().requires_grad_(True)
    logp, chi2 = pm.log_prob(s["sim"], z)
    logp.sum().backward()
    zc = z.detach().double().cpu().requires_grad_(True)
    xs = pm.bij.forward(zc)
    ll, ochi2 = O.forward_log_likelihood_flat(ORACLE_MODEL, s["ocfg"], flat_from_struct(xs), s["obs"].astype(np.float64),
                                              0.2, 1000.0)
    lp = ll + prior.log_prob(xs) + pm.unconstraining_bij.forward_log_det_jacobian(pm.pack_bij.forward(zc))
    (gz,) = torch.autograd.grad(lp.sum(), zc)
    def logpost32(zz):
        xs32 = pm.bij.forward(zz)
        l32, _ = O.forward_log_likelihood_flat(ORACLE_MODEL, s["ocfg"], flat_from_struct(xs32), s["obs"], 0.2,
                                               1000.0, dtype=torch.float32)
        return l32 + prior.log_prob(xs32) + pm.unconstraining_bij.forward_log_det_jacobian(pm.pack_bij.forward(zz))

    band = fp32_band(logpost32, z.detach().cpu(), gz)
    _check_scalar(logp.detach(), lp.detach(), 1e-4, name="logp")
    _check_scalar(chi2, ochi2.detach(), 1e-4, name="chi2")
    _check_grad(z.grad, (gz, band), "dlogp/dz")


def test_adjoint_is_weighted_gradient():
    s = _setup(60, 2, gaussian_psf(0.1, 0.0325, 21), 7, seed=2)
    plan = s["sim"].prob_plan(s["pm"])
    x = flat_from_struct(s["x_struct"]).float().cuda().contiguous()
    bs = x.shape[0]
    grad = torch.empty_like(x)
    N.call("gl_forward_grad", plan.handle, N.ptr(x), None, bs, None, None, N.ptr(grad), None, N.stream_ptr())
    w = torch.linspace(-2, 3, bs, device="cuda")
    dx = torch.empty_like(x)
    N.call("gl_adjoint", plan.handle, N.ptr(x), None, bs, N.ptr(w), N.ptr(dx), None, N.stream_ptr())
    torch.cuda.synchronize()
    assert torch.allclose(dx, grad * w[:, None], rtol=1e-6, atol=0)


def test_round_lens_single_term():
    """All ellipticities zero: the term-count rule gives one iteration (K = 1)."""
    prior = default_prior()
    s = _setup(40, 2, gaussian_psf(0.1, 0.0325, 13), 3, seed=7, prior=prior)
    xs = s["x_struct"]
    xs[0][0]["e1"] = torch.zeros(3)
    xs[0][0]["e2"] = torch.zeros(3)
    plan = s["sim"].prob_plan(s["pm"])
    x = flat_from_struct(xs).float().cuda().contiguous()
    logL = torch.empty(3, device="cuda")
    N.call("gl_forward", plan.handle, N.ptr(x), None, 3, N.ptr(logL), None, None, None, N.stream_ptr())
    torch.cuda.synchronize()
    ll, _, _ = _oracle_loglik(s, x.double().cpu(), with_fp32=False)
    _check_scalar(logL, ll, 1e-4, name="logL")


@pytest.mark.parametrize("variant", ["no_lens_light", "no_shear", "spherical_source"])
def test_model_families(variant):
    from gigalens_gb300.cuda.profiles.light import sersic
    from gigalens_gb300.cuda.profiles.mass import epl, shear

    base = default_prior()
    lens, ll, src = base.parts
    if variant == "no_lens_light":
        prior = tfd.JointDistributionSequential([lens, src])
        phys = PhysicalModel([epl.EPL(50), shear.Shear()], [], [sersic.SersicEllipse()])
        omodel = dict(lenses=[("EPL", {"niter": 50}), ("SHEAR", {})], lens_light=[],
                      source_light=[("SERSIC_ELLIPSE", {})])
    elif variant == "no_shear":
        prior = tfd.JointDistributionSequential([tfd.JointDistributionSequential([lens.parts[0]]), ll, src])
        phys = PhysicalModel([epl.EPL(50)], [sersic.SersicEllipse()], [sersic.SersicEllipse()])
        omodel = dict(lenses=[("EPL", {"niter": 50})], lens_light=[("SERSIC_ELLIPSE", {})],
                      source_light=[("SERSIC_ELLIPSE", {})])
    else:
        sp = dict(src.parts[0].parts)
        sp.pop("e1")
        sp.pop("e2")
        prior = tfd.JointDistributionSequential([lens, ll, tfd.JointDistributionSequential(
            [tfd.JointDistributionNamed(sp)])])
        phys = PhysicalModel([epl.EPL(50), shear.Shear()], [sersic.SersicEllipse()], [sersic.Sersic()])
        omodel = dict(lenses=[("EPL", {"niter": 50}), ("SHEAR", {})], lens_light=[("SERSIC_ELLIPSE", {})],
                      source_light=[("SERSIC", {})])
    s = _setup(48, 2, gaussian_psf(0.1, 0.0325, 21), 5, seed=11, phys=phys, omodel=omodel, prior=prior)
    plan = s["sim"].prob_plan(s["pm"])
    x = flat_from_struct(s["x_struct"]).float().cuda().contiguous()
    logL = torch.empty(5, device="cuda")
    grad = torch.empty_like(x)
    N.call("gl_forward_grad", plan.handle, N.ptr(x), None, 5, N.ptr(logL), None, N.ptr(grad), None, N.stream_ptr())
    torch.cuda.synchronize()
    ll, _, g = _oracle_loglik(s, x.double().cpu())
    _check_scalar(logL, ll, 1e-4, name="logL")
    _check_grad(grad, g)


def test_uneven_batch_two_image_sizes():
    """Samples of two different images (60x60 and 90x90) in one launch."""
    from gigalens_gb300.cuda._plan import ModelLayout, Plan

    prior = default_prior()
    phys = default_physmodel()
    lay = ModelLayout(phys)
    imgs, obs = [], []
    for n, k in [(60, 21), (90, 41)]:
        cfg = SimulatorConfig(delta_pix=0.065, num_pix=n, supersample=2, kernel_supersampled=gaussian_psf(0.1, 0.0325, k))
        o = np.random.default_rng(n).normal(scale=0.2, size=(n, n)).astype(np.float32) + 1.0
        imgs.append(dict(sim_config=cfg, observed=o, background_rms=0.2, exp_time=1000.0))
        obs.append(o)
    multi = Plan(lay, imgs)
    singles = [Plan(lay, [im]) for im in imgs]
    bs = 9
    x = flat_from_struct(prior.sample(bs, seed=3)).float().cuda().contiguous()
    img_id = torch.tensor([0, 1, 1, 0, 1, 0, 0, 1, 1], dtype=torch.int32, device="cuda")
    logL = torch.empty(bs, device="cuda")
    grad = torch.empty_like(x)
    N.call("gl_forward_grad", multi.handle, N.ptr(x), N.ptr(img_id), bs, N.ptr(logL), None, N.ptr(grad), None,
           N.stream_ptr())
    for i, p in enumerate(singles):
        sel = (img_id == i).nonzero().flatten()
        xs = x[sel].contiguous()
        l1 = torch.empty(len(sel), device="cuda")
        g1 = torch.empty_like(xs)
        N.call("gl_forward_grad", p.handle, N.ptr(xs), None, len(sel), N.ptr(l1), None, N.ptr(g1), None,
               N.stream_ptr())
        torch.cuda.synchronize()
        # the term count is per image group, so each group matches its own single-image launch
        assert torch.allclose(logL[sel], l1, rtol=1e-6) and torch.allclose(grad[sel], g1, rtol=1e-5, atol=1e-6)


def test_demo_fixture_on_gpu():
    """The reference's demo observation and PSF at the notebook's truth (ss = 1)."""
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    psf = load_golden("psf.npy").astype(np.float32)
    obs = load_golden("demo.npy").astype(np.float32)
    ksub = psf / psf.sum()
    cfg = SimulatorConfig(delta_pix=0.065, num_pix=60, supersample=1, kernel_supersampled=ksub)
    prior = default_prior()
    pm = ForwardProbModel(prior, obs, background_rms=0.2, exp_time=100.0)
    sim = LensSimulator(default_physmodel(), cfg, bs=1)
    truth = demo_truth()
    z = pm.bij.inverse([[{k: torch.tensor([v], dtype=torch.float32) for k, v in d.items()} for d in g]
                        for g in truth]).cuda()
    logp, chi2 = pm.log_prob(sim, z)
    ocfg = O.SimConfig(0.065, 60, 1, ksub.astype(np.float64))
    im = O.simulate(ORACLE_MODEL, ocfg, as_batch(truth))
    _, ochi2 = O.log_likelihood(im, obs.astype(np.float64), 0.2, 100.0)
    assert abs(float(chi2[0]) - float(ochi2[0])) <= 1e-4 * float(ochi2[0])
    assert 0.97 < float(chi2[0]) < 1.03


def test_launch_config_reports_the_kernel_shape():
    s = _setup(90, 2, gaussian_psf(0.1, 0.0325, 41), 4)
    plan = s["sim"].prob_plan(s["pm"])
    c = plan.launch_config(4096)
    assert c["threads_per_block"] == 512 and c["col_block"] == 16 and c["subkernel_side"] == 21
    assert c["blocks"] == torch.cuda.get_device_properties(0).multi_processor_count
    assert c["samples_per_cta"] * c["blocks"] >= 4096 and c["global_planes"] == 0 and c["family"] == 0
    assert c["smem_bytes"] > 200_000
    big = _setup(100, 2, gaussian_psf(0.1, 0.0325, 21), 2)
    cb = big["sim"].prob_plan(big["pm"]).launch_config(3)
    # the headline family keeps its compiled path with the planes in global memory
    assert cb["global_planes"] == 1 and cb["smem_bytes"] == 0 and cb["family"] == 0 and cb["blocks"] == 3


def test_empty_batches_are_no_ops():
    """bs = 0 through every entry point: success, and no output is written."""
    s = _setup(40, 2, gaussian_psf(0.1, 0.0325, 13), 2)
    plan = s["sim"].prob_plan(s["pm"])
    x = torch.zeros(1, 22, device="cuda")      # never read
    sentinel = torch.full((4,), 7.0, device="cuda")
    for fn, args in (("gl_forward", (N.ptr(sentinel), N.ptr(sentinel), None, None)),
                     ("gl_forward_grad", (N.ptr(sentinel), N.ptr(sentinel), N.ptr(sentinel), None)),
                     ("gl_log_prob", (N.ptr(sentinel), N.ptr(sentinel), N.ptr(sentinel), None))):
        N.call(fn, plan.handle, N.ptr(x), None, 0, *args, N.stream_ptr())
    torch.cuda.synchronize()
    assert torch.all(sentinel == 7.0)


def test_sample_results_do_not_depend_on_batch_neighbours():
    """A chain's log-likelihood, chi^2 and gradient are the same alone and in
    a batch (bitwise: fixed reduction order per sample), once the batch's
    EPL term count -- the reference's batch-coupled rule -- is the same."""
    s = _setup(40, 2, gaussian_psf(0.1, 0.0325, 13), 6, seed=3)
    x = flat_from_struct(s["x_struct"]).float().cuda().contiguous()
    e = (x[:, 2] ** 2 + x[:, 3] ** 2)           # EPL e1, e2 columns of the default model
    order = torch.argsort(e, descending=True)
    x = x[order].contiguous()                    # row 0 holds the most elliptical lens
    out = {}
    for bs in (6, 2):
        plan = s["sim"].prob_plan(s["pm"])
        logL, chi2 = torch.empty(bs, device="cuda"), torch.empty(bs, device="cuda")
        grad = torch.empty(bs, x.shape[1], device="cuda")
        xb = x[:bs].contiguous()
        N.call("gl_forward_grad", plan.handle, N.ptr(xb), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad), None,
               N.stream_ptr())
        torch.cuda.synchronize()
        out[bs] = (logL, chi2, grad)
    for a, b in zip(out[6], out[2]):
        assert torch.equal(a[:2], b[:2])


def test_rotated_anisotropic_pixel_grid():
    """A general transform_pix2angle (rotation by 30 degrees, pixel sides
    0.06" x 0.07"; simulator.py:91-125 grid, tf/simulator.py:19-29
    conversion factor det(T)): image, logL and gradient against the oracle."""
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    a = math.radians(30.0)
    R = np.array([[math.cos(a), -math.sin(a)], [math.sin(a), math.cos(a)]])
    T = (R @ np.diag([0.06, 0.07])).astype(np.float32)
    n, ss, bs = 40, 2, 4
    ksub = gaussian_psf(0.1, 0.0325, 13)
    cfg = SimulatorConfig(delta_pix=0.065, num_pix=n, supersample=ss, kernel_supersampled=ksub, transform_pix2angle=T)
    ocfg = O.SimConfig(0.065, n, ss, ksub.astype(np.float64), transform_pix2angle=T)
    prior = default_prior()
    truth = prior.sample(1, seed=101)
    im_t = O.simulate(ORACLE_MODEL, ocfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in truth])
    obs = (im_t[0].numpy() + np.random.default_rng(0).normal(scale=0.2, size=(n, n))).astype(np.float32)
    pm = ForwardProbModel(prior, obs, background_rms=0.2, exp_time=1000.0)
    sim = LensSimulator(default_physmodel(), cfg, bs=bs)
    xs = prior.sample(bs, seed=2)
    got = sim.simulate(xs).double().cpu()
    ref = O.simulate(ORACLE_MODEL, ocfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in xs])
    _check_images(got.reshape(ref.shape), ref, ORACLE_MODEL, ocfg, flat_from_struct(xs), "rotated grid")
    s = dict(omodel=ORACLE_MODEL, ocfg=ocfg, obs=obs)
    plan = sim.prob_plan(pm)
    x = flat_from_struct(xs).float().cuda().contiguous()
    logL, chi2, grad = torch.empty(bs, device="cuda"), torch.empty(bs, device="cuda"), torch.empty_like(x)
    N.call("gl_forward_grad", plan.handle, N.ptr(x), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad), None,
           N.stream_ptr())
    torch.cuda.synchronize()
    ll, c2, g = _oracle_loglik(s, x.double().cpu())
    _check_scalar(logL, ll, 1e-4, name="logL")
    _check_scalar(chi2, c2, 1e-4, name="chi2")
    _check_grad(grad, g)


def test_gradient_matches_fp64_central_differences_on_64_samples():
    """The 90x90 configuration's gradient check: 64 random samples, the
    kernel's d logL / dx against float64 central differences of the oracle
    (step 1e-6 max(1, |x|) per component), within 1e-3 relative or twice the
    float32 noise band of the reference's own arithmetic."""
    n, ss, bs = 90, 2, 64
    s = _setup(n, ss, gaussian_psf(0.1, 0.0325, 41), bs, seed=11)
    plan = s["sim"].prob_plan(s["pm"])
    x = flat_from_struct(s["x_struct"]).float().cuda().contiguous()
    logL, chi2, grad = torch.empty(bs, device="cuda"), torch.empty(bs, device="cuda"), torch.empty_like(x)
    N.call("gl_forward_grad", plan.handle, N.ptr(x), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad), None,
           N.stream_ptr())
    torch.cuda.synchronize()
    x64 = x.double().cpu()
    obs64 = s["obs"].astype(np.float64)
    fd = torch.zeros_like(x64)
    for j in range(x64.shape[1]):
        h = 1e-6 * torch.clamp(x64[:, j].abs(), min=1.0)
        e = torch.zeros_like(x64)
        e[:, j] = h
        lp, _ = O.forward_log_likelihood_flat(s["omodel"], s["ocfg"], x64 + e, obs64, 0.2, 1000.0)
        lm, _ = O.forward_log_likelihood_flat(s["omodel"], s["ocfg"], x64 - e, obs64, 0.2, 1000.0)
        fd[:, j] = (lp - lm) / (2 * h)
    band = fp32_band(lambda xx: O.forward_log_likelihood_flat(
        s["omodel"], s["ocfg"], xx, s["obs"], 0.2, 1000.0, dtype=torch.float32)[0], x64.float(), fd, n_perturb=2)
    _check_grad(grad, (fd, band), "d logL / dx vs FP64 central differences")
