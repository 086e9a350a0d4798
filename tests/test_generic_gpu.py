"""Parity of the fused kernel's general path (models outside the compiled
families: SIS, SIE, TNFW, CoreSersic, explicit-amplitude shapelets, several
sources) and of the least-squares likelihood gradient with the float64
oracle.  Tolerances are those of tests/test_fused_gpu.py."""
import math

import numpy as np
import pytest
import torch

from gigalens_gb300 import _native as N
from gigalens_gb300 import distributions as tfd
from gigalens_gb300.model import PhysicalModel
from gigalens_gb300.simulator import SimulatorConfig
from oracle import lens_oracle as O
from tests.helpers import flat_from_struct, gaussian_psf
from tests.test_fused_gpu import _check_grad, _check_images, _check_scalar, fp32_band

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def _shear_prior():
    return tfd.JointDistributionNamed(dict(gamma1=tfd.Normal(0, 0.05), gamma2=tfd.Normal(0, 0.05)))


def _se_prior(R, Ie, cs=0.05):
    return tfd.JointDistributionNamed(dict(
        R_sersic=tfd.LogNormal(math.log(R), 0.15), n_sersic=tfd.Uniform(1, 4),
        e1=tfd.TruncatedNormal(0, 0.1, -0.3, 0.3), e2=tfd.TruncatedNormal(0, 0.1, -0.3, 0.3),
        center_x=tfd.Normal(0, cs), center_y=tfd.Normal(0, cs), Ie=tfd.LogNormal(math.log(Ie), 0.3)))


def _model(name):
    """(physical model, oracle model, prior) of each general-path case."""
    from gigalens_gb300.cuda.profiles.light import sersic, shapelets
    from gigalens_gb300.cuda.profiles.mass import epl, shear, sie, sis, tnfw

    if name == "sie_shear_coresersic_se":
        phys = PhysicalModel([sie.SIE(), shear.Shear()], [sersic.CoreSersic()], [sersic.SersicEllipse()])
        om = dict(lenses=[("SIE", {}), ("SHEAR", {})], lens_light=[("CORE_SERSIC", {})],
                  source_light=[("SERSIC_ELLIPSE", {})])
        prior = tfd.JointDistributionSequential([
            tfd.JointDistributionSequential([
                tfd.JointDistributionNamed(dict(theta_E=tfd.LogNormal(math.log(1.2), 0.1),
                                                e1=tfd.Normal(0, 0.1), e2=tfd.Normal(0, 0.1),
                                                center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05))),
                _shear_prior()]),
            tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
                R_sersic=tfd.LogNormal(math.log(1.0), 0.15), n_sersic=tfd.Uniform(2, 4),
                Rb=tfd.LogNormal(math.log(0.1), 0.2), alpha=tfd.Uniform(1.5, 3), gamma=tfd.Uniform(0.1, 0.5),
                e1=tfd.TruncatedNormal(0, 0.1, -0.3, 0.3), e2=tfd.TruncatedNormal(0, 0.1, -0.3, 0.3),
                center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05),
                Ie=tfd.LogNormal(math.log(200.0), 0.3)))]),
            tfd.JointDistributionSequential([_se_prior(0.25, 150.0, 0.2)]),
        ])
    elif name in ("sie_shear_se_se", "sis_shear_se_se"):
        # compiled signatures of the general path (family 5: SIE, 6: SIS)
        mass = sie.SIE() if name.startswith("sie") else sis.SIS()
        phys = PhysicalModel([mass, shear.Shear()], [sersic.SersicEllipse()], [sersic.SersicEllipse()])
        om = dict(lenses=[(name[:3].upper(), {}), ("SHEAR", {})], lens_light=[("SERSIC_ELLIPSE", {})],
                  source_light=[("SERSIC_ELLIPSE", {})])
        lens = dict(theta_E=tfd.LogNormal(math.log(1.2), 0.1), center_x=tfd.Normal(0, 0.05),
                    center_y=tfd.Normal(0, 0.05))
        if name.startswith("sie"):
            lens.update(e1=tfd.Normal(0, 0.1), e2=tfd.Normal(0, 0.1))
        prior = tfd.JointDistributionSequential([
            tfd.JointDistributionSequential([tfd.JointDistributionNamed(lens), _shear_prior()]),
            tfd.JointDistributionSequential([_se_prior(1.0, 300.0)]),
            tfd.JointDistributionSequential([_se_prior(0.25, 150.0, 0.2)]),
        ])
    elif name == "epl_tnfw_shear_se":
        phys = PhysicalModel([epl.EPL(50), tnfw.TNFW(), shear.Shear()], [], [sersic.SersicEllipse()])
        om = dict(lenses=[("EPL", {"niter": 50}), ("TNFW", {}), ("SHEAR", {})], lens_light=[],
                  source_light=[("SERSIC_ELLIPSE", {})])
        prior = tfd.JointDistributionSequential([
            tfd.JointDistributionSequential([
                tfd.JointDistributionNamed(dict(theta_E=tfd.LogNormal(math.log(1.25), 0.1),
                                                gamma=tfd.TruncatedNormal(2, 0.1, 1.6, 2.4),
                                                e1=tfd.Normal(0, 0.1), e2=tfd.Normal(0, 0.1),
                                                center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05))),
                tfd.JointDistributionNamed(dict(Rs=tfd.LogNormal(math.log(0.5), 0.1),
                                                alpha_Rs=tfd.LogNormal(math.log(0.05), 0.2),
                                                r_trunc=tfd.LogNormal(math.log(5.0), 0.1),
                                                center_x=tfd.Normal(0.6, 0.05), center_y=tfd.Normal(-0.4, 0.05))),
                _shear_prior()]),
            tfd.JointDistributionSequential([_se_prior(0.25, 150.0, 0.2)]),
        ])
    elif name == "sis_se_two_sources":
        phys = PhysicalModel([sis.SIS()], [sersic.SersicEllipse()], [sersic.SersicEllipse(), sersic.Sersic()])
        om = dict(lenses=[("SIS", {})], lens_light=[("SERSIC_ELLIPSE", {})],
                  source_light=[("SERSIC_ELLIPSE", {}), ("SERSIC", {})])
        prior = tfd.JointDistributionSequential([
            tfd.JointDistributionSequential([
                tfd.JointDistributionNamed(dict(theta_E=tfd.LogNormal(math.log(1.2), 0.1),
                                                center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05)))]),
            tfd.JointDistributionSequential([_se_prior(1.0, 300.0)]),
            tfd.JointDistributionSequential([
                _se_prior(0.25, 150.0, 0.2),
                tfd.JointDistributionNamed(dict(R_sersic=tfd.LogNormal(math.log(0.15), 0.15),
                                                n_sersic=tfd.Uniform(1, 3), center_x=tfd.Normal(0.2, 0.1),
                                                center_y=tfd.Normal(-0.1, 0.1),
                                                Ie=tfd.LogNormal(math.log(80.0), 0.3)))]),
        ])
    elif name in ("sis_shapelets_explicit", "sis_shapelets_interp"):
        n_max = 3
        interp = name == "sis_shapelets_interp"
        sh = shapelets.Shapelets(n_max, use_lstsq=False, interpolate=interp)
        phys = PhysicalModel([sis.SIS()], [], [sh])
        om = dict(lenses=[("SIS", {})], lens_light=[],
                  source_light=[("SHAPELETS", {"n_max": n_max, "interpolate": interp})])
        amps = {a: tfd.Normal(0.0, 20.0) for a in sh._amp_names}
        prior = tfd.JointDistributionSequential([
            tfd.JointDistributionSequential([
                tfd.JointDistributionNamed(dict(theta_E=tfd.LogNormal(math.log(1.2), 0.1),
                                                center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05)))]),
            tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
                beta=tfd.LogNormal(math.log(0.15), 0.1), center_x=tfd.Normal(0, 0.1),
                center_y=tfd.Normal(0, 0.1), **amps))]),
        ])
    else:
        raise KeyError(name)
    return phys, om, prior


def _setup(name, num_pix=40, ss=2, k=13, bs=6, seed=0):
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    phys, om, prior = _model(name)
    ksub = gaussian_psf(0.1, 0.065 / ss, k)
    cfg = SimulatorConfig(delta_pix=0.065, num_pix=num_pix, supersample=ss, kernel_supersampled=ksub)
    ocfg = O.SimConfig(0.065, num_pix, ss, ksub.astype(np.float64))
    truth = prior.sample(1, seed=seed + 100)
    im_t = O.simulate(om, ocfg, [[{kk: v.double() for kk, v in d.items()} for d in g] for g in truth])
    rng = np.random.default_rng(seed)
    obs = (im_t[0].numpy() + rng.normal(scale=0.2, size=(num_pix, num_pix))).astype(np.float32)
    pm = ForwardProbModel(prior, obs, background_rms=0.2, exp_time=1000.0)
    sim = LensSimulator(phys, cfg, bs=bs)
    return dict(phys=phys, om=om, prior=prior, ocfg=ocfg, obs=obs, pm=pm, sim=sim,
                x_struct=prior.sample(bs, seed=seed))


# Models whose images are worse conditioned in float32 than the EPL + Sersic
# family, so that more pixels sit inside the float32 band (all of them must):
#  - TNFW sums terms of order tau^2 that cancel to O(x^2 ln x) near its centre
#    (tf/profiles/mass/tnfw.py:14-38); the reference's float32 formula is off
#    by percents there, and every ray through the centre inherits it;
#  - explicit shapelet amplitudes make signed sums, so pixels near a zero of
#    the image have large relative errors at any precision.
IMAGE_LIMITS = {
    "epl_tnfw_shear_se": dict(band_fraction=1e-2, max_rel=2e-3),
    "sis_shapelets_explicit": dict(band_fraction=1e-2, max_rel=5e-4),
    "sis_shapelets_interp": dict(band_fraction=1e-2, max_rel=5e-4),
}

# Largest relative gradient error allowed where the float32 restatement's own
# noise band exceeds the default 1e-2: in sis_shear_se_se one sample's shear
# gradient is a sum over pixels that cancels (measured band 1.32e-2 of the
# component's scale, kernel error 1.13e-2, inside twice the band).
GRAD_LIMITS = {"sis_shear_se_se": 2e-2}

GRAD_CASES = ["sie_shear_coresersic_se", "epl_tnfw_shear_se", "sis_se_two_sources", "sis_shapelets_explicit",
              "sis_shapelets_interp", "sie_shear_se_se", "sis_shear_se_se"]
# the model family each case's plan must take (4: run-time general path; 5, 6:
# the compiled SIE / SIS + shear signatures)
CASE_FAMILY = {"sie_shear_se_se": 5, "sis_shear_se_se": 6, "sie_shear_coresersic_se": 4, "epl_tnfw_shear_se": 4,
               "sis_se_two_sources": 4, "sis_shapelets_explicit": 4, "sis_shapelets_interp": 4}


@pytest.mark.parametrize("name", GRAD_CASES)
def test_general_path_simulate(name):
    s = _setup(name)
    img = s["sim"].simulate(s["x_struct"])
    ref = O.simulate(s["om"], s["ocfg"], [[{k: v.double() for k, v in d.items()} for d in g]
                                          for g in s["x_struct"]])
    _check_images(img.reshape(ref.shape), ref, s["om"], s["ocfg"], flat_from_struct(s["x_struct"]), name,
                  **IMAGE_LIMITS.get(name, {}))


@pytest.mark.parametrize("name", GRAD_CASES)
def test_general_path_loglik_grad(name):
    s = _setup(name)
    plan = s["sim"].prob_plan(s["pm"])
    x = flat_from_struct(s["x_struct"]).float().cuda().contiguous()
    bs = x.shape[0]
    cfg = plan.launch_config(bs)
    assert cfg["family"] == CASE_FAMILY[name]
    # the compiled signatures keep 40x40 px planes in shared memory
    assert cfg["global_planes"] == (1 if CASE_FAMILY[name] == 4 else 0)
    logL = torch.empty(bs, device="cuda")
    chi2 = torch.empty(bs, device="cuda")
    grad = torch.empty_like(x)
    N.call("gl_forward_grad", plan.handle, N.ptr(x), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad), None,
           N.stream_ptr())
    torch.cuda.synchronize()
    x64 = x.double().cpu().requires_grad_(True)
    ll, c2 = O.forward_log_likelihood_flat(s["om"], s["ocfg"], x64, s["obs"].astype(np.float64), 0.2, 1000.0)
    (g,) = torch.autograd.grad(ll.sum(), x64)
    band = fp32_band(lambda xx: O.forward_log_likelihood_flat(s["om"], s["ocfg"], xx, s["obs"], 0.2, 1000.0,
                                                              dtype=torch.float32)[0], x.cpu(), g)
    _check_scalar(logL, ll.detach(), 1e-4, name="logL")
    _check_scalar(chi2, c2.detach(), 1e-4, name="chi2")
    _check_grad(grad, (g, band), max_rel=GRAD_LIMITS.get(name, 1e-2))


@pytest.mark.parametrize("name", ["sie_shear_se_se", "sis_shear_se_se"])
def test_signature_global_planes(name):
    """The compiled signatures' global-plane kernels: 100x100 px planes exceed
    shared memory (likelihood, chi^2 and gradient against the oracle)."""
    s = _setup(name, num_pix=100, bs=4, seed=1)
    plan = s["sim"].prob_plan(s["pm"])
    x = flat_from_struct(s["x_struct"]).float().cuda().contiguous()
    bs = x.shape[0]
    cfg = plan.launch_config(bs)
    assert cfg["family"] == CASE_FAMILY[name] and cfg["global_planes"] == 1
    logL = torch.empty(bs, device="cuda")
    chi2 = torch.empty(bs, device="cuda")
    grad = torch.empty_like(x)
    N.call("gl_forward_grad", plan.handle, N.ptr(x), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad), None,
           N.stream_ptr())
    torch.cuda.synchronize()
    x64 = x.double().cpu().requires_grad_(True)
    ll, c2 = O.forward_log_likelihood_flat(s["om"], s["ocfg"], x64, s["obs"].astype(np.float64), 0.2, 1000.0)
    (g,) = torch.autograd.grad(ll.sum(), x64)
    band = fp32_band(lambda xx: O.forward_log_likelihood_flat(s["om"], s["ocfg"], xx, s["obs"], 0.2, 1000.0,
                                                              dtype=torch.float32)[0], x.cpu(), g)
    _check_scalar(logL, ll.detach(), 1e-4, name="logL")
    _check_scalar(chi2, c2.detach(), 1e-4, name="chi2")
    _check_grad(grad, (g, band), max_rel=GRAD_LIMITS.get(name, 1e-2))


def test_general_path_log_prob_autograd():
    """ForwardProbModel.log_prob on the general path (prior + bijector in the kernel)."""
    s = _setup("sie_shear_coresersic_se", bs=5, seed=3)
    pm, prior = s["pm"], s["prior"]
    z = pm.bij.inverse(s["x_struct"]).float().cuda().requires_grad_(True)
    logp, _ = pm.log_prob(s["sim"], z)
    logp.sum().backward()
    zc = z.detach().double().cpu().requires_grad_(True)
    xs = pm.bij.forward(zc)
    ll, _ = O.forward_log_likelihood_flat(s["om"], s["ocfg"], flat_from_struct(xs), s["obs"].astype(np.float64),
                                          0.2, 1000.0)
    lp = ll + prior.log_prob(xs) + pm.unconstraining_bij.forward_log_det_jacobian(pm.pack_bij.forward(zc))
    (gz,) = torch.autograd.grad(lp.sum(), zc)

    def logpost32(zz):
        xs32 = pm.bij.forward(zz)
        l32, _ = O.forward_log_likelihood_flat(s["om"], s["ocfg"], flat_from_struct(xs32), s["obs"], 0.2, 1000.0,
                                               dtype=torch.float32)
        return l32 + prior.log_prob(xs32) + pm.unconstraining_bij.forward_log_det_jacobian(pm.pack_bij.forward(zz))

    band = fp32_band(logpost32, z.detach().cpu(), gz)
    _check_scalar(logp.detach(), lp.detach(), 1e-4, name="logp")
    _check_grad(z.grad, (gz, band), "dlogp/dz")


def test_explicit_shapelet_amplitude_gradients_drive_map():
    """With explicit shapelet amplitudes (Shapelets(use_lstsq=False)) the MAP
    runs on the general path and raises the log posterior."""
    from gigalens_gb300.cuda.inference import ModellingSequence
    from gigalens_gb300.cuda.optimizers import Adam

    s = _setup("sis_shapelets_explicit", bs=8, seed=4)
    seq = ModellingSequence(s["phys"], s["pm"], s["sim"].sim_config)
    z0 = s["pm"].bij.inverse(s["x_struct"]).float()
    lp0, _ = s["pm"].log_prob(s["sim"], z0.cuda())
    z = seq.MAP(Adam(1e-2), start=s["x_struct"], num_steps=60)
    lp1, _ = s["pm"].log_prob(s["sim"], z)
    assert torch.isfinite(lp1).all() and float(lp1.max()) > float(lp0.max())


def _value_band(fn, args64, n_perturb=8, seed=0):
    """max |f32 - f64| of fn over its float32 evaluation at the inputs and at
    1-ulp perturbations of them (the reference computes in float32)."""
    ref = fn(*args64)
    r = np.random.default_rng(seed)
    worst = None
    for i in range(n_perturb + 1):
        a32 = []
        for a in args64:
            a = a.float()
            if i:
                a = a * (1 + torch.tensor(r.choice([-1.0, 0.0, 1.0], size=tuple(a.shape)) * 2.0 ** -23,
                                          dtype=torch.float32))
            a32.append(a)
        out = fn(*a32)
        outs = out if isinstance(out, tuple) else (out,)
        refs = ref if isinstance(ref, tuple) else (ref,)
        d = [(o.double() - rr).abs() for o, rr in zip(outs, refs)]
        worst = d if worst is None else [torch.maximum(w, dd) for w, dd in zip(worst, d)]
    return ref, worst


@pytest.mark.parametrize("kind", ["TNFW", "CORE_SERSIC"])
def test_profile_eval_new_types(kind):
    """Elementwise deriv / light against the float64 oracle: within 1e-5 relative
    or four times the float32 noise band of the same formula (the GPU's and the
    CPU's float32 transcendental functions differ by ulps).  TNFW's g(x) sums
    terms of order tau^2 that cancel to O(x^2 ln x) near the centre, where the
    reference's own float32 evaluation is off by percents."""
    from gigalens_gb300.cuda.profiles.light import sersic
    from gigalens_gb300.cuda.profiles.mass import tnfw

    r = np.random.default_rng(1)
    x = torch.tensor(r.normal(size=4000) * 1.5, dtype=torch.float32)
    y = torch.tensor(r.normal(size=4000) * 1.5, dtype=torch.float32)
    if kind == "TNFW":
        p = dict(Rs=0.7, alpha_Rs=0.3, r_trunc=4.0, center_x=0.1, center_y=-0.2)
        ax, ay = tnfw.TNFW().deriv(x, y, **p)
        pv = [torch.tensor(p[k], dtype=torch.float64) for k in ["Rs", "alpha_Rs", "r_trunc", "center_x", "center_y"]]
        (rx, ry), (bx, by) = _value_band(lambda xx, yy, *q: O.tnfw_deriv(xx, yy, *q), [x.double(), y.double()] + pv)
        for got, ref, band in ((ax, rx, bx), (ay, ry, by)):
            err = (got.double().cpu() - ref).abs()
            ok = (err <= 1e-5 * ref.abs() + 1e-6 * float(ref.abs().max())) | (err <= 4 * band)
            assert bool(ok.all()), float((err / ref.abs()).max())
    else:
        p = dict(R_sersic=0.9, n_sersic=3.0, Rb=0.1, alpha=2.0, gamma=0.3, e1=0.05, e2=-0.1, center_x=0.05,
                 center_y=0.0, Ie=100.0)
        got = sersic.CoreSersic().light(x, y, **p)
        pv = [torch.tensor(p[k], dtype=torch.float64) for k in
              ["R_sersic", "n_sersic", "Rb", "alpha", "gamma", "e1", "e2", "center_x", "center_y", "Ie"]]
        ref, (band,) = _value_band(lambda xx, yy, *q: O.core_sersic_light(xx, yy, *q), [x.double(), y.double()] + pv)
        err = (got.double().cpu() - ref).abs()
        ok = (err <= 1e-5 * ref.abs() + 1e-6 * float(ref.abs().max())) | (err <= 4 * band)
        assert bool(ok.all()), float((err / ref.abs()).max())


# ------------------------------------------------------------- least-squares gradient
def _lsq_setup(bs=5, num_pix=40, n_max=3, seed=0, lens_light=True):
    """The BackwardProbModel case: EPL + shear, shapelet source (and a Sersic
    lens light, both solved linearly).  Without the lens light the model is
    the compiled EPL + shear + shapelets signature of the general path."""
    from gigalens_gb300.cuda.profiles.light import sersic, shapelets
    from gigalens_gb300.cuda.profiles.mass import epl, shear

    phys = PhysicalModel([epl.EPL(50), shear.Shear()], [sersic.SersicEllipse(use_lstsq=True)] if lens_light else [],
                         [shapelets.Shapelets(n_max, use_lstsq=True, interpolate=False)])
    om = dict(lenses=[("EPL", {"niter": 50}), ("SHEAR", {})],
              lens_light=[("SERSIC_ELLIPSE", {})] if lens_light else [],
              source_light=[("SHAPELETS", {"n_max": n_max})])
    groups = [tfd.JointDistributionSequential([
        tfd.JointDistributionNamed(dict(theta_E=tfd.LogNormal(math.log(1.25), 0.1),
                                        gamma=tfd.TruncatedNormal(2, 0.1, 1.6, 2.4),
                                        e1=tfd.Normal(0, 0.1), e2=tfd.Normal(0, 0.1),
                                        center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05))),
        _shear_prior()])]
    if lens_light:
        groups.append(tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
            R_sersic=tfd.LogNormal(math.log(1.0), 0.15), n_sersic=tfd.Uniform(2, 4),
            e1=tfd.TruncatedNormal(0, 0.1, -0.3, 0.3), e2=tfd.TruncatedNormal(0, 0.1, -0.3, 0.3),
            center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05)))]))
    groups.append(tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
        beta=tfd.LogNormal(math.log(0.12), 0.1), center_x=tfd.Normal(0, 0.1), center_y=tfd.Normal(0, 0.1)))]))
    prior = tfd.JointDistributionSequential(groups)
    ksub = gaussian_psf(0.1, 0.0325, 13)
    cfg = SimulatorConfig(delta_pix=0.065, num_pix=num_pix, supersample=2, kernel_supersampled=ksub)
    ocfg = O.SimConfig(0.065, num_pix, 2, ksub.astype(np.float64))
    # observation: the least-squares image of a truth draw with fixed amplitudes, plus noise
    truth = prior.sample(1, seed=seed + 50)
    basis = O.lstsq_basis(om, ocfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in truth])
    D = basis.shape[-1]
    amps = torch.tensor(np.random.default_rng(seed).normal(size=D) * 5.0 + 3.0)
    amps[0] = 300.0
    rng = np.random.default_rng(seed + 1)
    obs = ((basis[0] * amps).sum(-1).numpy() + rng.normal(scale=0.2, size=(num_pix, num_pix))).astype(np.float32)
    err = np.sqrt(np.float32(0.2) ** 2 + np.clip(obs, 0, None) / np.float32(1000.0)).astype(np.float32)
    from gigalens_gb300.cuda.simulator import LensSimulator
    sim = LensSimulator(phys, cfg, bs=bs)
    return dict(phys=phys, om=om, prior=prior, ocfg=ocfg, obs=obs, err=err, sim=sim,
                x_struct=prior.sample(bs, seed=seed))


def _oracle_backward(s, x, dtype=torch.float64):
    params = O.unflatten(s["om"], x, lstsq=True)
    npd = np.float64 if dtype == torch.float64 else np.float32
    im = O.lstsq_simulate(s["om"], s["ocfg"], params, s["obs"].astype(npd), s["err"].astype(npd), dtype=dtype)
    return O.backward_log_likelihood(im, s["obs"].astype(npd), s["err"].astype(npd))


@pytest.mark.parametrize("num_pix,lens_light", [(40, True), (100, True), (40, False), (100, False)])
def test_lstsq_grad_matches_oracle_through_pinv(num_pix, lens_light):
    """gl_lstsq_grad (envelope theorem at the solved coefficients) against the
    float64 oracle differentiated through pinv, as TensorFlow differentiates
    tf/model.py:152-158.  100 px planes exceed shared memory and run from
    global memory.  Without lens light the model is the compiled EPL + shear +
    shapelets signature; with it, the run-time general path."""
    s = _lsq_setup(num_pix=num_pix, bs=5 if num_pix < 64 else 3, lens_light=lens_light)
    plan = s["sim"].lstsq_plan(s["obs"], s["err"])
    x = flat_from_struct(s["x_struct"]).float().cuda().contiguous()
    r = s["sim"].run_lstsq(plan, x, want_image=False, want_loglik=True)
    bs = x.shape[0]
    logL = torch.empty(bs, device="cuda")
    chi2 = torch.empty(bs, device="cuda")
    grad = torch.empty_like(x)
    N.call("gl_lstsq_grad", plan.handle, N.ptr(x), None, bs, N.ptr(r["coeffs"]), N.ptr(logL), N.ptr(chi2),
           N.ptr(grad), N.stream_ptr())
    torch.cuda.synchronize()
    x64 = x.double().cpu().requires_grad_(True)
    ll, c2 = _oracle_backward(s, x64)
    (g,) = torch.autograd.grad(ll.sum(), x64)
    band = fp32_band(lambda xx: _oracle_backward(s, xx, torch.float32)[0], x.cpu(), g)
    # the fused recomputation of the image agrees with the least-squares path
    _check_scalar(logL, ll.detach(), 1e-4, name="logL")
    _check_scalar(r["logL"], ll.detach(), 1e-4, name="lstsq logL")
    _check_scalar(chi2, c2.detach(), 1e-4, name="chi2")
    _check_grad(grad, (g, band), "dlogL/dx")


def test_backward_prob_model_autograd():
    """BackwardProbModel.log_prob gradient end to end (prior, bijector and the
    reference's fldj-at-x convention, tf/model.py:160)."""
    from gigalens_gb300.cuda.model import BackwardProbModel

    s = _lsq_setup(bs=4, seed=2)
    pm = BackwardProbModel(s["prior"], s["obs"], background_rms=0.2, exp_time=1000.0)
    z = pm.bij.inverse(s["x_struct"]).float().cuda().requires_grad_(True)
    lp, _ = pm.log_prob(s["sim"], z)
    lp.sum().backward()
    zc = z.detach().double().cpu().requires_grad_(True)
    xs = pm.bij.forward(zc)
    ll, _ = _oracle_backward(s, flat_from_struct(xs))
    ref = ll + s["prior"].log_prob(xs) + pm.unconstraining_bij.forward_log_det_jacobian(xs)
    (gz,) = torch.autograd.grad(ref.sum(), zc)
    _check_scalar(lp.detach(), ref.detach(), 1e-4, name="logp")
    _check_grad(z.grad, gz, "dlogp/dz")
