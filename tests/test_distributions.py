"""Prior distributions, bijectors and parameter packing (host side, CPU)."""
import math

import numpy as np
import pytest
import torch
from scipy import stats

from gigalens_gb300 import distributions as tfd
from gigalens_gb300.cuda.model import ForwardProbModel


def test_leaf_log_probs_match_scipy():
    x = torch.tensor([0.3, 1.1, 1.9, 2.7], dtype=torch.float64)
    assert np.allclose(tfd.Normal(0.5, 0.7).log_prob(x), stats.norm(0.5, 0.7).logpdf(x.numpy()))
    assert np.allclose(tfd.LogNormal(0.2, 0.3).log_prob(x),
                       stats.lognorm(s=0.3, scale=math.exp(0.2)).logpdf(x.numpy()))
    assert np.allclose(tfd.Uniform(0.0, 2.0).log_prob(x)[:3], stats.uniform(0, 2).logpdf(x.numpy()[:3]))
    assert tfd.Uniform(0.0, 2.0).log_prob(x)[3] == -math.inf
    t = tfd.TruncatedNormal(2.0, 0.25, 1.0, 3.0)
    ref = stats.truncnorm((1 - 2) / 0.25, (3 - 2) / 0.25, loc=2, scale=0.25).logpdf(x.numpy())
    got = t.log_prob(x).numpy()
    assert got[0] == -math.inf and np.allclose(got[1:], ref[1:])


def test_flatten_order_sorts_dict_keys(default_prior):
    s = default_prior.sample(2, seed=0)
    leaves = tfd.flatten(s)
    assert len(leaves) == 22
    names = []
    for g in s:
        for d in g:
            names += sorted(d.keys())
    assert names[:8] == ["center_x", "center_y", "e1", "e2", "gamma", "theta_E", "gamma1", "gamma2"]
    assert names[8:15] == ["Ie", "R_sersic", "center_x", "center_y", "e1", "e2", "n_sersic"]


def test_bij(default_prior):
    # tests/tf/test_model.py:10-16 of the reference
    model = ForwardProbModel(default_prior, np.ones((20, 20)), 1, 1)
    sample = default_prior.sample(5, seed=0)
    back = model.bij.forward(model.bij.inverse(sample))
    for a, b in zip(tfd.flatten(back), tfd.flatten(sample)):
        assert torch.allclose(a, b, rtol=1e-5, atol=1e-6)


def test_prior(default_prior):
    # tests/tf/test_model.py:19-26 of the reference: one log-det term per sample
    model = ForwardProbModel(default_prior, np.ones((20, 20)), 1, 1)
    z = model.bij.inverse(default_prior.sample(5, seed=0))
    det = model.unconstraining_bij.forward_log_det_jacobian(model.pack_bij.forward(z))
    assert det.numel() == 5


def test_sigmoid_fldj_matches_autograd():
    b = tfd.Sigmoid(1.0, 3.0)
    z = torch.linspace(-6, 6, 25, dtype=torch.float64, requires_grad=True)
    x = b.forward(z)
    (dx,) = torch.autograd.grad(x.sum(), z)
    assert torch.allclose(b.forward_log_det_jacobian(z.detach()), torch.log(dx))
    assert torch.allclose(b.inverse(x.detach()), z.detach(), atol=1e-9)


def test_samples_inside_support(default_prior):
    s = default_prior.sample(2000, seed=4)
    lp = default_prior.log_prob(s)
    assert torch.isfinite(lp).all()
