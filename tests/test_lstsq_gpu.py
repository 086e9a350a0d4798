"""Least-squares path (``lstsq_simulate``, BackwardProbModel) against the
float64 oracle.  Images are compared relative to their maximum (bar 1e-5):
the solved amplitudes of nearly degenerate shapelet stacks are
ill-conditioned (as in the reference, whose float32 pinv has the same
conditioning), the fitted image is not.  logp and chi^2: 1e-4 relative."""
import math

import numpy as np
import pytest
import torch

from gigalens_gb300 import distributions as tfd
from gigalens_gb300.model import PhysicalModel
from gigalens_gb300.simulator import SimulatorConfig
from oracle import lens_oracle as O
from tests.helpers import gaussian_psf

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def shapelet_prior(n_max, with_lens_light=False, beta=(math.log(0.1), 0.15)):
    lens = tfd.JointDistributionSequential([
        tfd.JointDistributionNamed(dict(theta_E=tfd.LogNormal(0.0, 0.1), gamma=tfd.TruncatedNormal(2, 0.1, 1.5, 2.5),
                                        e1=tfd.Normal(0, 0.05), e2=tfd.Normal(0, 0.05),
                                        center_x=tfd.Normal(0, 0.02), center_y=tfd.Normal(0, 0.02))),
        tfd.JointDistributionNamed(dict(gamma1=tfd.Normal(0, 0.02), gamma2=tfd.Normal(0, 0.02)))])
    src = tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
        beta=tfd.LogNormal(*beta), center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05)))])
    parts = [lens]
    if with_lens_light:
        parts.append(tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
            R_sersic=tfd.LogNormal(0.0, 0.1), n_sersic=tfd.Uniform(2, 5), e1=tfd.Normal(0, 0.05),
            e2=tfd.Normal(0, 0.05), center_x=tfd.Normal(0, 0.02), center_y=tfd.Normal(0, 0.02)))]))
    parts.append(src)
    return tfd.JointDistributionSequential(parts)


def models(n_max, with_lens_light):
    from gigalens_gb300.cuda.profiles.light import sersic, shapelets
    from gigalens_gb300.cuda.profiles.mass import epl, shear

    ll = [sersic.SersicEllipse(use_lstsq=True)] if with_lens_light else []
    phys = PhysicalModel([epl.EPL(50), shear.Shear()], ll,
                         [shapelets.Shapelets(n_max, use_lstsq=True, interpolate=False)])
    omodel = dict(lenses=[("EPL", {"niter": 50}), ("SHEAR", {})],
                  lens_light=[("SERSIC_ELLIPSE", {})] if with_lens_light else [],
                  source_light=[("SHAPELETS", {"n_max": n_max})])
    return phys, omodel


def _obs(n, rng):
    yy, xx = np.mgrid[0:n, 0:n]
    r = np.hypot(xx - n / 2, yy - n / 2)
    ring = 5.0 * np.exp(-0.5 * ((r - n / 4) / 2.0) ** 2)
    return (ring + rng.normal(scale=0.1, size=(n, n))).astype(np.float32)


@pytest.mark.parametrize("n,ss,k,n_max,ll", [(40, 2, 21, 4, False), (48, 2, 13, 8, False), (36, 1, 13, 3, True),
                                            (44, 2, 11, 5, True), (32, 1, 11, 3, False), (120, 2, 21, 2, False),
                                            (32, 2, 13, 9, True)])   # the most channels: 55 shapelets + 1
def test_lstsq_simulate_matches_oracle(n, ss, k, n_max, ll):
    from gigalens_gb300.cuda.model import BackwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    prior = shapelet_prior(n_max, ll)
    phys, omodel = models(n_max, ll)
    ksub = gaussian_psf(0.1, 0.08 / ss, k)
    cfg = SimulatorConfig(delta_pix=0.08, num_pix=n, supersample=ss, kernel_supersampled=ksub)
    obs = _obs(n, np.random.default_rng(n))
    pm = BackwardProbModel(prior, obs, background_rms=0.1, exp_time=200.0)
    bs = 6
    sim = LensSimulator(phys, cfg, bs=bs)
    xs = prior.sample(bs, seed=1)
    img = sim.lstsq_simulate(xs, pm.observed_numpy, pm.err_numpy)
    ocfg = O.SimConfig(0.08, n, ss, ksub.astype(np.float64))
    ox = [[{kk: v.double() for kk, v in d.items()} for d in g] for g in xs]
    ref = O.lstsq_simulate(omodel, ocfg, ox, obs.astype(np.float64), pm.err_numpy.astype(np.float64))
    got = img.double().cpu().reshape(ref.shape)
    scale = ref.abs().amax(dim=(-2, -1), keepdim=True)
    rel = ((got - ref).abs() / scale).max()
    # BackwardProbModel likelihood and chi^2
    z = pm.bij.inverse(xs).float().cuda()
    logp, chi2 = pm.log_prob(sim, z)
    ll_ref, chi2_ref = O.backward_log_likelihood(ref, obs.astype(np.float64), pm.err_numpy.astype(np.float64))
    lp_ref = ll_ref + prior.log_prob(ox) + pm.unconstraining_bij.forward_log_det_jacobian(ox)
    rlp = float(((logp.double().cpu() - lp_ref).abs() / lp_ref.abs()).max())
    rc2 = float(((chi2.double().cpu() - chi2_ref).abs() / chi2_ref.abs()).max())
    print("\n[lstsq %d px n_max %d] image max |err|/max %.2e, logp max rel %.2e, chi2 max rel %.2e"
          % (n, n_max, float(rel), rlp, rc2))
    assert float(rel) <= 1e-5
    assert rlp <= 1e-4 and rc2 <= 1e-4


def test_lstsq_uneven_batch_two_images():
    """Samples of a 48x48 and a 32x32 observation in one launch."""
    from gigalens_gb300 import _native as N
    from gigalens_gb300.cuda._plan import ModelLayout, Plan
    from gigalens_gb300.cuda.simulator import LensSimulator

    n_max = 4
    prior = shapelet_prior(n_max)
    phys, _ = models(n_max, False)
    lay = ModelLayout(phys)
    rng = np.random.default_rng(0)
    ims = []
    for n in (48, 32):
        cfg = SimulatorConfig(delta_pix=0.08, num_pix=n, supersample=2, kernel_supersampled=gaussian_psf(0.1, 0.04, 13))
        ims.append(dict(sim_config=cfg, observed=_obs(n, rng), background_rms=0.1, exp_time=200.0))
    multi = Plan(lay, ims)
    singles = [Plan(lay, [im]) for im in ims]
    sim = LensSimulator(phys, ims[0]["sim_config"], bs=8)
    bs = 8
    x = torch.stack([v.reshape(-1) for v in tfd.flatten(prior.sample(bs, seed=2))], 1).float().cuda().contiguous()
    img_id = torch.tensor([0, 1, 1, 0, 0, 1, 0, 1], dtype=torch.int32, device="cuda")
    import ctypes
    nb = ctypes.c_size_t(0)
    D = ctypes.c_int(0)
    N.call("gl_lstsq_workspace", multi.handle, bs, ctypes.byref(nb), ctypes.byref(D))
    work = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    co = torch.empty(bs, D.value, device="cuda")
    lg = torch.empty(bs, device="cuda")
    N.call("gl_lstsq", multi.handle, N.ptr(x), N.ptr(img_id), bs, N.ptr(work), nb.value, N.ptr(co), None,
           N.ptr(lg), None, N.stream_ptr())
    for i, p in enumerate(singles):
        sel = (img_id == i).nonzero().flatten()
        r = sim.run_lstsq(p, x[sel], want_image=False, want_loglik=True)
        torch.cuda.synchronize()
        assert torch.allclose(lg[sel], r["logL"], rtol=1e-5)


@pytest.mark.parametrize("use_lstsq", [True, False])
@pytest.mark.parametrize("interpolate", [False, True])
@pytest.mark.parametrize("scale", [1.0, 4.0])
def test_shapelets_light_api(use_lstsq, interpolate, scale):
    """``tests/test_profiles.py:35-47`` of the reference: n_max=5, beta=1,
    5x5 N(0,1) points, rtol 1e-5 / atol 1e-4 (here against the oracle of
    the same mode); scale 4 spreads the points past the table's [-5, 5]."""
    from gigalens_gb300.cuda.profiles.light.shapelets import Shapelets

    rng = np.random.default_rng(0)
    shp = Shapelets(n_max=5, use_lstsq=use_lstsq, interpolate=interpolate)
    x = (scale * rng.normal(size=(5, 5, 1))).astype(np.float32)
    y = (scale * rng.normal(size=(5, 5, 1))).astype(np.float32)
    D = torch.float64
    if use_lstsq:
        got = shp.light(torch.tensor(x).cuda(), torch.tensor(y).cuda(), center_x=0.0, center_y=0.0, beta=1.0)
        ref = O.shapelets_basis(torch.tensor(x, dtype=D), torch.tensor(y, dtype=D), torch.tensor(0.0, dtype=D),
                                torch.tensor(0.0, dtype=D), torch.tensor(1.0, dtype=D), 5, interpolate)
    else:
        amps = rng.normal(size=(shp.n_layers, 1)).astype(np.float32)
        amp = {k: torch.tensor(a) for k, a in zip(shp._amp_names, amps)}
        got = shp.light(torch.tensor(x).cuda(), torch.tensor(y).cuda(), center_x=0.0, center_y=0.0, beta=1.0, **amp)
        ref = O.shapelets_light(torch.tensor(x, dtype=D), torch.tensor(y, dtype=D), torch.tensor(0.0, dtype=D),
                                torch.tensor(0.0, dtype=D), torch.tensor(1.0, dtype=D),
                                [torch.tensor(a, dtype=D) for a in amps], 5, interpolate)
    g = got.double().cpu().numpy().reshape(ref.shape)
    assert np.allclose(g, ref.numpy(), rtol=1e-5, atol=1e-4)
    assert np.abs(g - ref.numpy()).max() < 1e-6
    if interpolate and scale > 1:
        # the table's cut: points with |x| > 5 give exactly zero
        outside = (np.abs(x) > 5) | (np.abs(y) > 5)
        assert outside.any() and np.all(g.reshape(-1, *x.shape)[..., outside] == 0.0)


def test_lstsq_interpolated_shapelets_match_oracle():
    """lstsq_simulate with the reference's default Shapelets(interpolate=True):
    the basis is the tabulated functions, cut to zero past 5 beta."""
    from gigalens_gb300.cuda.model import BackwardProbModel
    from gigalens_gb300.cuda.profiles.light import sersic, shapelets
    from gigalens_gb300.cuda.profiles.mass import epl, shear
    from gigalens_gb300.cuda.simulator import LensSimulator

    n, ss, k, n_max = 40, 2, 21, 6
    prior = shapelet_prior(n_max, True)
    phys = PhysicalModel([epl.EPL(50), shear.Shear()], [sersic.SersicEllipse(use_lstsq=True)],
                         [shapelets.Shapelets(n_max, use_lstsq=True, interpolate=True)])
    omodel = dict(lenses=[("EPL", {"niter": 50}), ("SHEAR", {})], lens_light=[("SERSIC_ELLIPSE", {})],
                  source_light=[("SHAPELETS", {"n_max": n_max, "interpolate": True})])
    ksub = gaussian_psf(0.1, 0.08 / ss, k)
    cfg = SimulatorConfig(delta_pix=0.08, num_pix=n, supersample=ss, kernel_supersampled=ksub)
    obs = _obs(n, np.random.default_rng(n))
    pm = BackwardProbModel(prior, obs, background_rms=0.1, exp_time=200.0)
    bs = 6
    sim = LensSimulator(phys, cfg, bs=bs)
    xs = prior.sample(bs, seed=1)
    img = sim.lstsq_simulate(xs, pm.observed_numpy, pm.err_numpy)
    ocfg = O.SimConfig(0.08, n, ss, ksub.astype(np.float64))
    ox = [[{kk: v.double() for kk, v in d.items()} for d in g] for g in xs]
    ref = O.lstsq_simulate(omodel, ocfg, ox, obs.astype(np.float64), pm.err_numpy.astype(np.float64))
    got = img.double().cpu().reshape(ref.shape)
    scale = ref.abs().amax(dim=(-2, -1), keepdim=True)
    rel = float(((got - ref).abs() / scale).max())
    print("\n[lstsq interpolated shapelets] image max |err|/max %.2e" % rel)
    assert rel <= 1e-5
    # the cut matters at these scales: the exact basis gives another fit
    ox_exact = dict(omodel, source_light=[("SHAPELETS", {"n_max": n_max})])
    ref_exact = O.lstsq_simulate(ox_exact, ocfg, ox, obs.astype(np.float64), pm.err_numpy.astype(np.float64))
    assert float(((ref_exact - ref).abs() / scale).max()) > 1e-3


@pytest.mark.parametrize("gram", [1, 2])
def test_gram_accuracy(gram, monkeypatch):
    """G = A^T A against float64 from the same basis stack (both read from
    the workspace: X first, then G), for both Gram kernels.  1: tcgen05
    3xTF32, which keeps about 21 bits per product and sums in FP32 within
    each 1024-pixel segment (segments in float-float): ~5e-6 of max|G|.
    2: FP32 register tiles, each thread summing its pixel range in FP32 and
    the ranges added in a fixed order."""
    import ctypes

    from gigalens_gb300 import _native as N
    from gigalens_gb300.cuda import autotune
    from gigalens_gb300.cuda.simulator import LensSimulator

    monkeypatch.setenv("GIGALENS_GB300_AUTOTUNE", "0")   # keep the variant set below

    n, n_max = 40, 8
    prior = shapelet_prior(n_max, True)
    phys, _ = models(n_max, True)
    ksub = gaussian_psf(0.1, 0.04, 21)
    cfg = SimulatorConfig(delta_pix=0.08, num_pix=n, supersample=2, kernel_supersampled=ksub)
    obs = _obs(n, np.random.default_rng(7))
    err = np.sqrt(0.1 ** 2 + np.clip(obs, 0, None) / 200.0).astype(np.float32)
    bs = 5
    sim = LensSimulator(phys, cfg, bs=bs)
    plan = sim.lstsq_plan(obs, err)
    autotune.set_tuning(plan, lsq_gram=gram)
    assert autotune.get_tuning(plan)["lsq_gram"] == gram
    with pytest.raises(N.GigaLensCudaError):
        autotune.set_tuning(plan, lsq_gram=3)   # rejected, the plan keeps its variant
    assert autotune.get_tuning(plan)["lsq_gram"] == gram
    x = sim.layout.flatten_params(prior.sample(bs, seed=3))
    r = sim.run_lstsq(plan, x, want_image=False)
    torch.cuda.synchronize()
    D, P = r["D"], n * n
    up = lambda v: (v + 255) // 256 * 256
    w8 = r["work"]
    X = w8[: bs * D * P * 4].view(torch.float32).reshape(bs, D, P).double().cpu()
    off = up(bs * D * P * 4)
    G = w8[off: off + bs * D * D * 4].view(torch.float32).reshape(bs, D, D).double().cpu()
    A = X / torch.as_tensor(err.reshape(-1), dtype=torch.float64)
    G64 = A @ A.transpose(1, 2)
    rel = float(((G - G64).abs() / G64.abs().amax(dim=(1, 2), keepdim=True)).max())
    print("\n[Gram variant %d] max |G - G64| / max|G64| = %.2e" % (gram, rel))
    assert rel < 2e-5, rel
    assert torch.equal(G, G.transpose(1, 2))
    assert bool(torch.isfinite(r["coeffs"]).all())


def test_gram_variants_agree_on_the_solution(monkeypatch):
    """The full least-squares call (37 samples of a 60x60 image, 45 shapelet
    channels) with either Gram kernel: the same images and likelihoods to
    the accuracy the refinement passes leave, and the FP32 kernel bitwise
    reproducible."""
    from gigalens_gb300 import _native as N
    from gigalens_gb300.cuda import autotune
    from gigalens_gb300.cuda.simulator import LensSimulator

    monkeypatch.setenv("GIGALENS_GB300_AUTOTUNE", "0")
    n, n_max = 60, 8
    prior = shapelet_prior(n_max)
    phys, _ = models(n_max, False)
    cfg = SimulatorConfig(delta_pix=0.08, num_pix=n, supersample=2, kernel_supersampled=gaussian_psf(0.1, 0.04, 21))
    obs = _obs(n, np.random.default_rng(11))
    err = np.sqrt(0.1 ** 2 + np.clip(obs, 0, None) / 200.0).astype(np.float32)
    bs = 37
    sim = LensSimulator(phys, cfg, bs=bs)
    plan = sim.lstsq_plan(obs, err)
    x = sim.layout.flatten_params(prior.sample(bs, seed=5))
    out = {}
    for g in (1, 2, 2):
        autotune.set_tuning(plan, lsq_gram=g)
        r = sim.run_lstsq(plan, x, want_image=True, want_loglik=True)
        torch.cuda.synchronize()
        out.setdefault(g, []).append((r["img"].clone(), r["logL"].clone(), r["coeffs"].clone()))
    (i1, l1, _), = out[1]
    (i2, l2, c2), (i2b, l2b, c2b) = out[2]
    assert torch.equal(c2, c2b) and torch.equal(i2, i2b) and torch.equal(l2, l2b)
    rel = float(((i1 - i2).abs() / i1.abs().amax(dim=1, keepdim=True)).max())
    print("\n[Gram variants] image max |d|/max %.2e, logL max rel %.2e"
          % (rel, float(((l1 - l2).abs() / l1.abs()).max())))
    assert rel < 1e-5
    assert torch.allclose(l1, l2, rtol=1e-5)
