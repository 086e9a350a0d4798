"""Shared test inputs: the reference's default prior and physical model
(``tests/conftest.py:21-80`` of GIGA-Lens), the synthetic configurations of
the benchmark workloads, and adapters to the oracle."""
import math
import os

import numpy as np
import torch

from gigalens_gb300 import distributions as tfd

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

ORACLE_MODEL = dict(lenses=[("EPL", {"niter": 50}), ("SHEAR", {})], lens_light=[("SERSIC_ELLIPSE", {})],
                    source_light=[("SERSIC_ELLIPSE", {})])


def default_prior():
    """``tests/conftest.py:21-73`` of the reference."""
    lens_prior = tfd.JointDistributionSequential([
        tfd.JointDistributionNamed(dict(theta_E=tfd.LogNormal(math.log(1.25), 0.25),
                                        gamma=tfd.TruncatedNormal(2, 0.25, 1, 3),
                                        e1=tfd.Normal(0, 0.1), e2=tfd.Normal(0, 0.1),
                                        center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05))),
        tfd.JointDistributionNamed(dict(gamma1=tfd.Normal(0, 0.05), gamma2=tfd.Normal(0, 0.05))),
    ])
    lens_light_prior = tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
        R_sersic=tfd.LogNormal(math.log(1.0), 0.15), n_sersic=tfd.Uniform(2, 6),
        e1=tfd.TruncatedNormal(0, 0.1, -0.3, 0.3), e2=tfd.TruncatedNormal(0, 0.1, -0.3, 0.3),
        center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05), Ie=tfd.LogNormal(math.log(500.0), 0.3)))])
    source_light_prior = tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
        R_sersic=tfd.LogNormal(math.log(0.25), 0.15), n_sersic=tfd.Uniform(0.5, 4),
        e1=tfd.TruncatedNormal(0, 0.15, -0.5, 0.5), e2=tfd.TruncatedNormal(0, 0.15, -0.5, 0.5),
        center_x=tfd.Normal(0, 0.25), center_y=tfd.Normal(0, 0.25), Ie=tfd.LogNormal(math.log(150.0), 0.5)))])
    return tfd.JointDistributionSequential([lens_prior, lens_light_prior, source_light_prior])


def default_physmodel(niter=50):
    from gigalens_gb300.model import PhysicalModel
    from gigalens_gb300.cuda.profiles.light import sersic
    from gigalens_gb300.cuda.profiles.mass import epl, shear

    return PhysicalModel([epl.EPL(niter), shear.Shear()], [sersic.SersicEllipse(use_lstsq=False)],
                         [sersic.SersicEllipse(use_lstsq=False)])


def gaussian_psf(fwhm_arcsec, pixel_arcsec, side):
    """Normalised Gaussian PSF sampled at pixel centres (odd side)."""
    sigma = fwhm_arcsec / (2.0 * math.sqrt(2.0 * math.log(2.0)))
    r = (np.arange(side) - (side - 1) / 2.0) * pixel_arcsec
    g = np.exp(-0.5 * (r / sigma) ** 2)
    k = np.outer(g, g)
    return (k / k.sum()).astype(np.float32)


def demo_truth():
    """True parameters of the reference's demo (``tf-demo.ipynb`` cell 5)."""
    return [[{'theta_E': 1.1, 'gamma': 2.0, 'e1': 0.1, 'e2': 0.1, 'center_x': 0.1, 'center_y': 0.0},
             {'gamma1': -0.01, 'gamma2': 0.03}],
            [{'R_sersic': 0.8, 'n_sersic': 2.5, 'e1': 0.09534746574143645, 'e2': 0.14849487967198177,
              'center_x': 0.1, 'center_y': 0.0, 'Ie': 499.3695906504067}],
            [{'R_sersic': 0.25, 'n_sersic': 1.5, 'e1': 0., 'e2': 0., 'center_x': 0.09566681002252231,
              'center_y': -0.0639623054267272, 'Ie': 149.58828877085668}]]


def as_batch(params, dtype=torch.float64):
    return [[{k: torch.tensor([v], dtype=dtype) for k, v in d.items()} for d in g] for g in params]


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name))


def flat_from_struct(struct):
    return torch.stack([torch.as_tensor(v).reshape(-1) for v in tfd.flatten(struct)], dim=1)


def image_band(omodel, ocfg, xflat, n_pert=8, seed=1):
    """Float32 noise band of simulated images, per pixel: the largest
    |image - float64 image| over the oracle with float32 ray shooting (the
    rest in float64) at the input and at ``n_pert`` 1-ulp perturbations of
    the lens parameters.  Near a steep lensed source cusp, float32
    deflections alone move a pixel by up to ~1e-4 of its value; the reference
    computes in float32 and carries the same noise."""
    from oracle import lens_oracle as O

    x32 = torch.as_tensor(xflat).float()
    x64 = x32.double()
    lens_cols = [i for i, (g, _, _) in enumerate(O.flat_layout(omodel)) if g == 0]
    ref = O.simulate(omodel, ocfg, O.unflatten(omodel, x64))
    r = np.random.default_rng(seed)
    band = torch.zeros_like(ref)
    for i in range(n_pert + 1):
        xq = x64.clone()
        if i:
            pert = torch.tensor(r.choice([-1.0, 0.0, 1.0], size=(x32.shape[0], len(lens_cols))) * 2.0 ** -23,
                                dtype=torch.float32)
            xq[:, lens_cols] = (x32[:, lens_cols] * (1 + pert)).double()
        im = O.simulate(omodel, ocfg, O.unflatten(omodel, xq), ray_dtype=torch.float32)
        band = torch.maximum(band, (im - ref).abs())
    return band


def check_images(got, ref, band, name="image", fraction=1e-3, band_fraction=1e-3, max_rel=2e-4):
    """Per-pixel bar on pixels above ``fraction`` of their image's maximum,
    no absolute term: |got - ref| <= 1e-5 |ref|, or <= 1e-5 |ref| + 2 band
    on at most ``band_fraction`` of them (``band``: ``image_band``), with a
    relative error of at most ``max_rel`` there.  Fainter pixels:
    |got - ref| <= 1e-6 of the image's maximum.  Prints the figures."""
    got = got.double().cpu().reshape(ref.shape)
    m = ref.abs().amax(dim=(-2, -1), keepdim=True)
    sel = ref.abs() > fraction * m
    err = (got - ref).abs()
    lit = err <= 1e-5 * ref.abs()
    ok = err <= 1e-5 * ref.abs() + 2.0 * band
    need = sel & ~lit
    rel = err / ref.abs()
    faint = float((err / m)[~sel].max()) if bool((~sel).any()) else 0.0
    print("\n[%s] %d pixels above %.0e of max: max rel %.2e; %d (%.3f %%) need the float32 band (max rel %.2e); "
          "fainter pixels: max |err|/max %.2e" % (
              name, int(sel.sum()), fraction, float(rel[sel].max()), int(need.sum()),
              100.0 * float(need.sum()) / max(int(sel.sum()), 1), float(rel[need].max()) if bool(need.any()) else 0.0,
              faint))
    assert bool(ok[sel].all()), "%s: pixels outside 1e-5 + 2 band" % name
    assert float(need.sum()) <= max(band_fraction * float(sel.sum()), 2.0), "%s: %d pixels need the band" % (
        name, int(need.sum()))
    assert float(rel[sel].max()) <= max_rel, name
    assert faint <= 1e-6, name
