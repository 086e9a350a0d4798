"""Failure detection without a GPU fault.

* Non-finite parameters injected from the host: the fused kernel's
  per-sample status word (bit 0: non-finite logL / log posterior, bit 1:
  non-finite gradient) must describe exactly what it returned, NaN light
  must be zeroed as in the reference (``tf/simulator.py:81``), and the
  other samples of the batch must not change by a single bit.
* The least-squares Gram kernel's bounded waits on the tensor cores: with
  the wait limit lowered to zero polls through the test hook, every wait of
  its pipeline runs out; the kernel must record the timeout in the status
  word, drain its MMAs, free its tensor memory and return, the solve must
  return NaN coefficients, and the next call on the same plan (default
  limit) must give the results of a clean run bit for bit.
"""
import ctypes
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

# columns of the flat vector (packing order: sorted keys per profile)
COL = {("lens", "theta_E"): 5, ("lens_light", "Ie"): 8, ("lens_light", "R_sersic"): 9,
       ("source", "center_x"): 17, ("source", "Ie"): 15, ("source", "R_sersic"): 16}


def _setup(bs=8, n=40):
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    cfg = W.sim_config(n, 7)
    ocfg = O.SimConfig(W.DELTA_PIX, n, 2, np.asarray(cfg.kernel_supersampled, np.float64))
    truth = W.draw_params(1, seed=50)
    im = O.simulate(ORACLE_MODEL, ocfg, [[{k: v.double() for k, v in d.items()} for d in g] for g in truth])
    obs = W.observe(im.float(), seed=3)[0].numpy()
    pm = ForwardProbModel(W.config_prior(), obs, background_rms=W.BG_RMS, exp_time=W.EXP_TIME)
    sim = LensSimulator(W.physical_model(), cfg, bs=bs)
    x = flat_from_struct(W.draw_params(bs, seed=51)).float()
    return sim, pm, ocfg, obs, x


def _run(plan, x):
    bs = x.shape[0]
    xd = x.cuda().contiguous()
    logL, chi2 = torch.empty(bs, device="cuda"), torch.empty(bs, device="cuda")
    grad = torch.empty_like(xd)
    status = torch.full((bs,), -1, dtype=torch.int32, device="cuda")
    N.call("gl_forward_grad", plan.handle, N.ptr(xd), None, bs, N.ptr(logL), N.ptr(chi2), N.ptr(grad),
           N.ptr(status), N.stream_ptr())
    torch.cuda.synchronize()
    return logL.cpu(), chi2.cpu(), grad.cpu(), status.cpu()


def test_packing_columns_of_the_injection():
    names = [(g, p, k) for (g, p, k) in O.flat_layout(ORACLE_MODEL)]
    group = {0: "lens", 1: "lens_light", 2: "source"}
    for (grp, key), col in COL.items():
        g, p, k = names[col]
        assert group[g] == grp and k == key and (grp != "lens" or p == 0)


def test_injected_nonfinite_parameters_set_the_status_word():
    sim, pm, ocfg, obs, x = _setup()
    plan = sim.prob_plan(pm)
    clean = _run(plan, x)
    assert bool((clean[3] == 0).all())
    bad = x.clone()
    bad[1, COL[("source", "center_x")]] = float("nan")     # source light NaN everywhere -> zeroed
    bad[3, COL[("lens_light", "Ie")]] = float("inf")        # image +inf -> noise model NaN
    bad[4, COL[("lens", "theta_E")]] = float("nan")         # deflection NaN -> source zeroed
    bad[6, COL[("source", "R_sersic")]] = 0.0               # R / R_sersic = inf
    logL, chi2, grad, status = _run(plan, bad)
    # the status word describes exactly what was returned
    for b in range(x.shape[0]):
        want = (0 if math.isfinite(float(logL[b])) else 1) | (0 if bool(torch.isfinite(grad[b]).all()) else 2)
        assert int(status[b]) == want, (b, int(status[b]), want)
    # samples without injected values are bitwise unchanged
    for b in (0, 2, 5, 7):
        assert torch.equal(logL[b], clean[0][b]) and torch.equal(grad[b], clean[2][b]), b
        assert int(status[b]) == 0
    assert int(status[3]) & 1
    # NaN light is zeroed (tf/simulator.py:81) after lens light and source are
    # summed: a NaN source blanks every pixel, and the likelihood is the one
    # of an empty model image, as the oracle gives for the same input
    for b in (1, 4):
        assert int(status[b]) & 1 == 0, b
        ll_ref, c2_ref = O.forward_log_likelihood_flat(ORACLE_MODEL, ocfg, bad[b:b + 1].double(),
                                                       obs.astype(np.float64), W.BG_RMS, W.EXP_TIME)
        assert math.isfinite(float(ll_ref))
        assert abs(float(logL[b]) - float(ll_ref)) <= 1e-4 * abs(float(ll_ref)), (b, float(logL[b]), float(ll_ref))
        assert abs(float(chi2[b]) - float(c2_ref)) <= 1e-4 * abs(float(c2_ref))
    # zeroed pixels pass no gradient (TensorFlow's where() would give NaN
    # through the NaN branch): every component is exactly 0, except those of
    # the lens whose own parameter is NaN (their chain rule multiplies zero
    # sums by NaN partials, as TensorFlow's would)
    assert bool((grad[1] == 0).all())
    assert bool((grad[4, 8:] == 0).all()), grad[4]


def test_log_prob_status_flags_nonfinite_log_posterior():
    sim, pm, ocfg, obs, x = _setup(bs=4)
    plan = sim.prob_plan(pm)
    z = pm.bij.inverse(W.draw_params(4, seed=52)).float().cuda().contiguous()
    z[2, COL[("lens_light", "Ie")]] = float("inf")
    logp, chi2 = torch.empty(4, device="cuda"), torch.empty(4, device="cuda")
    g = torch.empty_like(z)
    status = torch.full((4,), -1, dtype=torch.int32, device="cuda")
    N.call("gl_log_prob", plan.handle, N.ptr(z), None, 4, N.ptr(logp), N.ptr(chi2), N.ptr(g), N.ptr(status),
           N.stream_ptr())
    torch.cuda.synchronize()
    for b in range(4):
        assert int(status[b]) == (0 if math.isfinite(float(logp[b])) else 1), b
    assert int(status[2]) == 1 and int(status[0]) == 0


def _lstsq_case():
    from gigalens_gb300.cuda._plan import ModelLayout, Plan
    from gigalens_gb300.model import PhysicalModel
    from gigalens_gb300.simulator import SimulatorConfig
    from gigalens_gb300.cuda.profiles.light import shapelets
    from gigalens_gb300.cuda.profiles.mass import epl, shear

    phys = PhysicalModel([epl.EPL(50), shear.Shear()], [], [shapelets.Shapelets(4, use_lstsq=True, interpolate=False)])
    n = 32
    rng = np.random.default_rng(9)
    obs = (1.0 + rng.normal(scale=0.1, size=(n, n))).astype(np.float32)
    cfg = SimulatorConfig(delta_pix=0.08, num_pix=n, supersample=2, kernel_supersampled=W.gaussian_psf(0.1, 0.04, 13))
    plan = Plan(ModelLayout(phys), [dict(sim_config=cfg, observed=obs, background_rms=0.1, exp_time=200.0)])
    lens = W.draw_params(6, seed=8)[0]
    src = {"beta": torch.tensor(rng.uniform(0.05, 0.2, 6), dtype=torch.float32),
           "center_x": torch.tensor(rng.normal(0, 0.05, 6), dtype=torch.float32),
           "center_y": torch.tensor(rng.normal(0, 0.05, 6), dtype=torch.float32)}
    x = flat_from_struct([[lens[0], lens[1]], [src]]).float().cuda().contiguous()
    return plan, x


def _lstsq(plan, x, work, nb, D):
    bs = x.shape[0]
    co = torch.empty(bs, D, device="cuda")
    lg = torch.empty(bs, device="cuda")
    N.call("gl_lstsq", plan.handle, N.ptr(x), None, bs, N.ptr(work), nb, N.ptr(co), None, N.ptr(lg), None,
           N.stream_ptr())
    st = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    N.call("gl_lstsq_status", plan.handle, bs, N.ptr(work), N.ptr(st), N.stream_ptr())
    torch.cuda.synchronize()
    return co.cpu(), lg.cpu(), int(st[0])


def test_gram_wait_timeout_returns_status_and_nan_then_recovers():
    from gigalens_gb300.cuda import autotune

    plan, x = _lstsq_case()
    autotune.set_tuning(plan, lsq_gram=1)   # the tensor-core Gram, whose pipeline waits are bounded
    bs = x.shape[0]
    nb, D = ctypes.c_size_t(0), ctypes.c_int(0)
    N.call("gl_lstsq_workspace", plan.handle, bs, ctypes.byref(nb), ctypes.byref(D))
    work = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    co0, lg0, st0 = _lstsq(plan, x, work, nb.value, D.value)
    assert st0 == 0 and bool(torch.isfinite(co0).all())
    try:
        N.call("gl_test_set_wait_polls", 0)
        co1, lg1, st1 = _lstsq(plan, x, work, nb.value, D.value)
    finally:
        N.call("gl_test_set_wait_polls", -1)
    assert st1 == 1
    assert bool(torch.isnan(co1).all()) and bool(torch.isnan(lg1).all())
    # the kernel returned and freed its tensor memory: the same plan works again
    for _ in range(2):
        co2, lg2, st2 = _lstsq(plan, x, work, nb.value, D.value)
        assert st2 == 0 and torch.equal(co2, co0) and torch.equal(lg2, lg0)
