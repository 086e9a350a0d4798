"""gl_lstsq_noalloc: the least-squares launch for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

Checked through the C ABI against gl_lstsq with a caller-allocated
workspace, on two calls in a row (the second call finds the first call's
contents in the shared scratch), and again after a larger batch of other
data has overwritten, with different values, every byte of scratch that the
first call uses.
Both entry points run the same deterministic launch sequence (no atomics,
fixed reduction orders), so the results must be bitwise equal: a read of a
scratch element that the call did not write first would show as a
difference.  This file sorts last so that a run that stops at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest
import torch

from gigalens_gb300 import _native as N
from gigalens_gb300 import distributions as tfd
from gigalens_gb300.model import PhysicalModel
from gigalens_gb300.simulator import SimulatorConfig
from tests.helpers import gaussian_psf

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def _plan_and_inputs(bs, seed=3):
    from gigalens_gb300.cuda._plan import ModelLayout, Plan
    from gigalens_gb300.cuda.profiles.light import shapelets
    from gigalens_gb300.cuda.profiles.mass import epl, shear

    phys = PhysicalModel([epl.EPL(50), shear.Shear()], [], [shapelets.Shapelets(6, use_lstsq=True, interpolate=False)])
    prior = tfd.JointDistributionSequential([
        tfd.JointDistributionSequential([
            tfd.JointDistributionNamed(dict(theta_E=tfd.LogNormal(0.0, 0.1), gamma=tfd.TruncatedNormal(2, 0.1, 1.5, 2.5),
                                            e1=tfd.Normal(0, 0.05), e2=tfd.Normal(0, 0.05),
                                            center_x=tfd.Normal(0, 0.02), center_y=tfd.Normal(0, 0.02))),
            tfd.JointDistributionNamed(dict(gamma1=tfd.Normal(0, 0.02), gamma2=tfd.Normal(0, 0.02)))]),
        tfd.JointDistributionSequential([tfd.JointDistributionNamed(dict(
            beta=tfd.LogNormal(np.log(0.1), 0.15), center_x=tfd.Normal(0, 0.05), center_y=tfd.Normal(0, 0.05)))]),
    ])
    n = 40
    rng = np.random.default_rng(7)
    yy, xx = np.mgrid[0:n, 0:n]
    obs = (4.0 * np.exp(-0.5 * ((np.hypot(xx - n / 2, yy - n / 2) - n / 4) / 2.0) ** 2)
           + rng.normal(scale=0.1, size=(n, n))).astype(np.float32)
    cfg = SimulatorConfig(delta_pix=0.08, num_pix=n, supersample=2, kernel_supersampled=gaussian_psf(0.1, 0.04, 13))
    plan = Plan(ModelLayout(phys), [dict(sim_config=cfg, observed=obs, background_rms=0.1, exp_time=200.0)])
    x = torch.stack([v.reshape(-1) for v in tfd.flatten(prior.sample(bs, seed=seed))], 1).float().cuda().contiguous()
    return plan, x


def _run_workspace(plan, x):
    bs = x.shape[0]
    nb, D = ctypes.c_size_t(0), ctypes.c_int(0)
    N.call("gl_lstsq_workspace", plan.handle, bs, ctypes.byref(nb), ctypes.byref(D))
    work = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    co = torch.empty(bs, D.value, device="cuda")
    img = torch.empty(bs, plan.max_pix, device="cuda")
    lg, c2 = torch.empty(bs, device="cuda"), torch.empty(bs, device="cuda")
    N.call("gl_lstsq", plan.handle, N.ptr(x), None, bs, N.ptr(work), nb.value, N.ptr(co), N.ptr(img), N.ptr(lg),
           N.ptr(c2), N.stream_ptr())
    torch.cuda.synchronize()
    return co, img, lg, c2, D.value


def _run_noalloc(plan, x, D):
    bs = x.shape[0]
    co = torch.full((bs, D), float("nan"), device="cuda")
    img = torch.full((bs, plan.max_pix), float("nan"), device="cuda")
    lg, c2 = torch.full((bs,), float("nan"), device="cuda"), torch.full((bs,), float("nan"), device="cuda")
    N.call("gl_lstsq_noalloc", plan.handle, N.ptr(x), None, bs, N.ptr(co), N.ptr(img), N.ptr(lg), N.ptr(c2),
           N.stream_ptr())
    torch.cuda.synchronize()
    return co, img, lg, c2


def _assert_bitwise(got, want, what):
    for name, a, b in zip(("coeffs", "image", "logL", "chi2"), got, want):
        assert torch.isfinite(a).all(), (what, name)
        assert torch.equal(a, b), "%s: %s differs (max |d| %.3g)" % (what, name, float((a - b).abs().max()))


def test_noalloc_matches_workspace_entry_point_twice():
    plan, x = _plan_and_inputs(12)
    co, img, lg, c2, D = _run_workspace(plan, x)
    for call in range(2):
        _assert_bitwise(_run_noalloc(plan, x, D), (co, img, lg, c2), "call %d" % call)
    # a larger batch of other data in between overwrites every byte of scratch
    # that the 12-chain call uses; the next call must not see those values
    plan_b, xb = _plan_and_inputs(29, seed=11)
    _run_noalloc(plan_b, xb, D)
    _assert_bitwise(_run_noalloc(plan, x, D), (co, img, lg, c2), "after another batch")


def test_noalloc_rejects_batches_beyond_its_scratch():
    plan, x = _plan_and_inputs(2)
    nb = ctypes.c_size_t(0)
    N.call("gl_lstsq_workspace", plan.handle, 1, ctypes.byref(nb), None)
    too_many = 2 * int((64 << 20) // nb.value) + 8
    xx = x[:1].expand(too_many, -1).contiguous()
    co = torch.empty(too_many, 64, device="cuda")
    rc = N.lib().gl_lstsq_noalloc(plan.handle, N.ptr(xx), None, too_many, N.ptr(co), None, None, None,
                                  N.stream_ptr())
    assert rc == N.GL_ERR_INVALID
    assert b"fixed" in N.lib().gl_last_error()
