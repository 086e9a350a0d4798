"""The benchmark configurations of this path, as data generators.

* ``config0`` / ``config1``: 60x60 px and 90x90 px at 0.065"/px,
  supersampling 2, Gaussian PSF of FWHM 0.1" (11x11 and 21x21 at base scale;
  the supersampled 21x21 / 41x41 kernel is generated directly on the fine
  grid), EPL(50) + external shear, elliptical Sersic lens light and source.
* ``draw_params``: the configurations' parameter distributions --
  theta_E ~ U(1, 1.6), gamma ~ U(1.8, 2.3), e1, e2 ~ N(0, 0.1), centre ~
  N(0, 0.05); shear ~ N(0, 0.05); lens light R ~ U(0.5, 1.5), n ~ U(2, 6),
  e ~ N(0, 0.1), centre ~ N(0, 0.05), log10 Ie ~ U(0, 1.5); source
  R ~ U(0.05, 0.4), n ~ U(0.5, 4), centre ~ U(-0.3, 0.3), log10 Ie ~
  U(0.5, 2), e ~ TruncatedNormal(0, 0.15, -0.5, 0.5) (the reference's
  ``tests/conftest.py:61-62`` form, which the configuration leaves open).
* ``config_prior``: a prior whose supports hold those distributions, for
  the bijector and the prior term of ``log_prob``.
* ``observe``: Poisson noise at the exposure time plus Gaussian background.
"""
import math

import numpy as np
import torch

from . import distributions as tfd
from .simulator import SimulatorConfig

DELTA_PIX = 0.065
FWHM = 0.1
BG_RMS = 0.2
EXP_TIME = 1000.0
NITER = 50


def gaussian_psf(fwhm, pixel, side):
    """Unit-sum Gaussian sampled at pixel centres (odd side)."""
    sigma = fwhm / (2.0 * math.sqrt(2.0 * math.log(2.0)))
    r = (np.arange(side) - (side - 1) / 2.0) * pixel
    g = np.exp(-0.5 * (r / sigma) ** 2)
    k = np.outer(g, g)
    return (k / k.sum()).astype(np.float32)


def sim_config(num_pix, psf_base_side, supersample=2):
    ksub = gaussian_psf(FWHM, DELTA_PIX / supersample, supersample * psf_base_side - (supersample - 1))
    return SimulatorConfig(delta_pix=DELTA_PIX, num_pix=num_pix, supersample=supersample,
                           kernel=gaussian_psf(FWHM, DELTA_PIX, psf_base_side), kernel_supersampled=ksub)


def config0():
    return sim_config(60, 11)


def config1():
    return sim_config(90, 21)


def physical_model():
    from .model import PhysicalModel
    from .cuda.profiles.light import sersic
    from .cuda.profiles.mass import epl, shear

    return PhysicalModel([epl.EPL(NITER), shear.Shear()], [sersic.SersicEllipse()], [sersic.SersicEllipse()])


def config_prior():
    ie_ll = tfd.LogNormal(0.75 * math.log(10), 0.75 * math.log(10) / math.sqrt(3))
    ie_src = tfd.LogNormal(1.25 * math.log(10), 0.75 * math.log(10) / math.sqrt(3))
    return tfd.JointDistributionSequential([
        tfd.JointDistributionSequential([
            tfd.JointDistributionNamed(dict(theta_E=tfd.Uniform(1.0, 1.6), gamma=tfd.Uniform(1.8, 2.3),
                                            e1=tfd.Normal(0, 0.1), e2=tfd.Normal(0, 0.1),
                                            center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05))),
            tfd.JointDistributionNamed(dict(gamma1=tfd.Normal(0, 0.05), gamma2=tfd.Normal(0, 0.05)))]),
        tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
            R_sersic=tfd.Uniform(0.5, 1.5), n_sersic=tfd.Uniform(2, 6), e1=tfd.Normal(0, 0.1),
            e2=tfd.Normal(0, 0.1), center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05), Ie=ie_ll))]),
        tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
            R_sersic=tfd.Uniform(0.05, 0.4), n_sersic=tfd.Uniform(0.5, 4),
            e1=tfd.TruncatedNormal(0, 0.15, -0.5, 0.5), e2=tfd.TruncatedNormal(0, 0.15, -0.5, 0.5),
            center_x=tfd.Uniform(-0.3, 0.3), center_y=tfd.Uniform(-0.3, 0.3), Ie=ie_src))]),
    ])


def draw_params(n, seed):
    """Parameter structure of n lenses from the configuration's distributions."""
    r = np.random.default_rng(seed)
    f = lambda a: torch.tensor(np.asarray(a, dtype=np.float32))

    def tn(size):   # TruncatedNormal(0, 0.15, -0.5, 0.5) by rejection
        out = r.normal(0, 0.15, size)
        bad = np.abs(out) >= 0.5
        while bad.any():
            out[bad] = r.normal(0, 0.15, int(bad.sum()))
            bad = np.abs(out) >= 0.5
        return out

    lens = {"theta_E": f(r.uniform(1.0, 1.6, n)), "gamma": f(r.uniform(1.8, 2.3, n)),
            "e1": f(r.normal(0, 0.1, n)), "e2": f(r.normal(0, 0.1, n)),
            "center_x": f(r.normal(0, 0.05, n)), "center_y": f(r.normal(0, 0.05, n))}
    sh = {"gamma1": f(r.normal(0, 0.05, n)), "gamma2": f(r.normal(0, 0.05, n))}
    ll = {"R_sersic": f(r.uniform(0.5, 1.5, n)), "n_sersic": f(r.uniform(2, 6, n)),
          "e1": f(r.normal(0, 0.1, n)), "e2": f(r.normal(0, 0.1, n)),
          "center_x": f(r.normal(0, 0.05, n)), "center_y": f(r.normal(0, 0.05, n)),
          "Ie": f(10 ** r.uniform(0, 1.5, n))}
    src = {"R_sersic": f(r.uniform(0.05, 0.4, n)), "n_sersic": f(r.uniform(0.5, 4, n)),
           "e1": f(tn(n)), "e2": f(tn(n)),
           "center_x": f(r.uniform(-0.3, 0.3, n)), "center_y": f(r.uniform(-0.3, 0.3, n)),
           "Ie": f(10 ** r.uniform(0.5, 2, n))}
    return [[lens, sh], [ll], [src]]


def flat(params):
    """Nested parameter structure -> (n, d) tensor in packing order."""
    return torch.stack([torch.as_tensor(v).reshape(-1) for v in tfd.flatten(params)], dim=1)


def observe(img, seed=None, exp_time=EXP_TIME, bg_rms=BG_RMS, generator=None):
    """Poisson(img * t) / t + N(0, bg^2), on img's device."""
    if generator is None:
        generator = torch.Generator(device=img.device)
        generator.manual_seed(0 if seed is None else int(seed))
    counts = torch.poisson(torch.clamp(img, min=0) * exp_time, generator=generator) / exp_time
    return counts + bg_rms * torch.randn(img.shape, device=img.device, generator=generator)
