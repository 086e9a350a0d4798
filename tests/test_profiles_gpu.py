"""Elementwise profile API (MassProfile.deriv / LightProfile.light) on the GPU
against the float64 oracle, at the reference's own test points
(``tests/test_profiles.py`` of GIGA-Lens: 10^4 N(0,1) points, rtol 1e-5 /
atol 1e-4), plus a tighter float32-level bound."""
import math

import numpy as np
import pytest
import torch

from oracle import lens_oracle as O

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def _pts(n=10000):
    rng = np.random.default_rng(0)
    return rng.normal(size=n).astype(np.float32), rng.normal(size=n).astype(np.float32)


def _cmp(got, ref, rtol=1e-5, atol=1e-4, tight=2e-6):
    g = got.detach().double().cpu().numpy()
    r = ref.detach().double().numpy()
    assert np.allclose(g, r, rtol=rtol, atol=atol)          # the reference's own tolerance
    scale = np.abs(r).max()
    assert np.abs(g - r).max() <= tight * max(scale, 1.0), np.abs(g - r).max() / scale


@pytest.mark.parametrize("theta_E,gamma,e1,e2", [(1.0, 2.0, 0.0, 0.0), (1.2, 2.2, -0.1, 0.1), (1.1, 1.8, 0.2, 0.15)])
def test_epl(theta_E, gamma, e1, e2):
    from gigalens_gb300.cuda.profiles.mass.epl import EPL

    x, y = _pts()
    ax, ay = EPL(100).deriv(torch.tensor(x).cuda(), torch.tensor(y).cuda(), theta_E=theta_E, gamma=gamma,
                            e1=e1, e2=e2, center_x=0.0, center_y=0.0)
    k = O.epl_term_count(e1, e2, 100)
    T = lambda v: torch.tensor(v, dtype=torch.float64)
    rx, ry = O.epl_deriv(torch.tensor(x, dtype=torch.float64), torch.tensor(y, dtype=torch.float64), T(theta_E),
                         T(gamma), T(e1), T(e2), T(0.0), T(0.0), k)
    _cmp(ax, rx)
    _cmp(ay, ry)


def test_epl_batch_term_count_and_broadcast():
    """Per-point parameters: the term count is the batch rule over all points."""
    from gigalens_gb300.cuda.profiles.mass.epl import EPL

    rng = np.random.default_rng(1)
    x, y = _pts(4096)
    e1 = rng.normal(0, 0.15, 4096).astype(np.float32)
    e2 = rng.normal(0, 0.15, 4096).astype(np.float32)
    ax, ay = EPL(50).deriv(torch.tensor(x).cuda(), torch.tensor(y).cuda(), theta_E=1.3, gamma=2.1,
                           e1=torch.tensor(e1).cuda(), e2=torch.tensor(e2).cuda(), center_x=0.01, center_y=-0.02)
    k = O.epl_term_count(e1, e2, 50)
    D = lambda v: torch.tensor(v, dtype=torch.float64)
    rx, ry = O.epl_deriv(D(x), D(y), D(1.3), D(2.1), D(e1), D(e2), D(0.01), D(-0.02), k)
    _cmp(ax, rx)
    _cmp(ay, ry)


def test_shear_sis_sie():
    from gigalens_gb300.cuda.profiles.mass.shear import Shear
    from gigalens_gb300.cuda.profiles.mass.sie import SIE
    from gigalens_gb300.cuda.profiles.mass.sis import SIS

    x, y = _pts()
    X, Y = torch.tensor(x).cuda(), torch.tensor(y).cuda()
    D = lambda v: torch.tensor(v, dtype=torch.float64)
    xd, yd = D(x), D(y)
    for g1, g2 in [(0.0, 0.0), (0.1, 0.1), (-0.03, 0.05)]:
        ax, ay = Shear().deriv(X, Y, gamma1=g1, gamma2=g2)
        rx, ry = O.shear_deriv(xd, yd, D(g1), D(g2))
        _cmp(ax, rx)
        _cmp(ay, ry)
    for th in [1.0, 1.2]:
        ax, ay = SIS().deriv(X, Y, theta_E=th, center_x=0.0, center_y=0.0)
        rx, ry = O.sis_deriv(xd, yd, D(th), D(0.0), D(0.0))
        _cmp(ax, rx)
        _cmp(ay, ry)
    for th, e1, e2 in [(1.0, 1e-3, 1e-3), (1.2, 0.1, -0.1)]:
        ax, ay = SIE().deriv(X, Y, theta_E=th, e1=e1, e2=e2, center_x=0.0, center_y=0.0)
        rx, ry = O.sie_deriv(xd, yd, D(th), D(e1), D(e2), D(0.0), D(0.0))
        _cmp(ax, rx, tight=2e-5)
        _cmp(ay, ry, tight=2e-5)


def test_sersic_ellipse_half_light_and_points():
    from gigalens_gb300.cuda.profiles.light.sersic import Sersic, SersicEllipse

    se = SersicEllipse(use_lstsq=False)
    p = dict(R_sersic=1.0, n_sersic=2.0, center_x=0.0, center_y=0.0, e1=0.0, e2=0.0, Ie=5.0)
    a = se.light(torch.tensor([0.0]).cuda(), torch.tensor([1.0]).cuda(), **p)
    assert math.isclose(float(a[0]), 5.0, rel_tol=1e-6)           # tests/test_profiles.py:17-26
    x, y = _pts(1000)
    D = lambda v: torch.tensor(v, dtype=torch.float64)
    for q in [dict(R_sersic=1.0, n_sersic=2.0, e1=0.0, e2=0.0, center_x=0.0, center_y=0.0, Ie=5.0),
              dict(R_sersic=0.3, n_sersic=4.0, e1=0.1, e2=-0.2, center_x=0.05, center_y=0.02, Ie=100.0)]:
        got = se.light(torch.tensor(x).cuda(), torch.tensor(y).cuda(), **q)
        ref = O.sersic_ellipse_light(D(x), D(y), *[D(q[k]) for k in
                                                   ["R_sersic", "n_sersic", "e1", "e2", "center_x", "center_y", "Ie"]])
        _cmp(got, ref, tight=1e-5)
    got = Sersic().light(torch.tensor(x).cuda(), torch.tensor(y).cuda(), R_sersic=0.5, n_sersic=1.5, center_x=0.1,
                         center_y=0.0, Ie=3.0)
    ref = O.sersic_light(D(x), D(y), D(0.5), D(1.5), D(0.1), D(0.0), D(3.0))
    _cmp(got, ref, tight=1e-5)
