"""SVI and HMC of the CUDA substrate: the reference's smoke tests
(``tests/tf/test_model.py:45-72``) plus a statistical check of the sampler."""
import math

import numpy as np
import pytest
import torch

from gigalens_gb300 import distributions as tfd
from gigalens_gb300.simulator import SimulatorConfig

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def _seq(prior, phys, data=(np.zeros((20, 20)), 0.1, 100), cfg=None):
    from gigalens_gb300.cuda.inference import ModellingSequence
    from gigalens_gb300.cuda.model import ForwardProbModel

    pm = ForwardProbModel(prior, *data)
    cfg = cfg or SimulatorConfig(delta_pix=0.05, num_pix=20)
    return ModellingSequence(phys, pm, cfg), pm


def test_vi(default_prior, default_physmodel):
    from gigalens_gb300.cuda.optimizers import Adam

    seq, pm = _seq(default_prior, default_physmodel)
    start = pm.bij.inverse(default_prior.sample(2, seed=0))[0]
    q_z, losses = seq.SVI(optimizer=Adam(0), start=start, n_vi=5, num_steps=5)
    assert torch.allclose(q_z.mean().cpu(), start.float())
    q_z, losses = seq.SVI(optimizer=Adam(1e-3), start=start, n_vi=5, num_steps=5)
    assert not torch.allclose(q_z.mean().cpu(), start.float())
    assert losses.shape == (5,) and torch.isfinite(losses).all()


def test_hmc(default_prior, default_physmodel):
    from gigalens_gb300.cuda.optimizers import Adam

    seq, pm = _seq(default_prior, default_physmodel)
    start = pm.bij.inverse(default_prior.sample(2, seed=0))[0]
    q_z, _ = seq.SVI(optimizer=Adam(0), start=start, n_vi=2, num_steps=2)
    num_results = 5
    samples, stats = seq.HMC(q_z, n_hmc=3, init_eps=0.3, init_l=3, max_leapfrog_steps=5, num_burnin_steps=3,
                             num_results=num_results)
    assert len(samples) == num_results and samples.shape == (5, 3, 22)


def test_hmc_fixed_trajectory_graph_matches_target_when_likelihood_is_flat(default_prior, default_physmodel):
    """Background noise 1e4 makes the likelihood flat over the prior, so the
    posterior is the prior: HMC (fixed L = 8, CUDA-graph iterations) must
    reproduce the unconstrained prior's moments."""
    from gigalens_gb300.cuda.diagnostics import potential_scale_reduction
    from gigalens_gb300.cuda.inference import MultivariateNormalTriL

    seq, pm = _seq(default_prior, default_physmodel, data=(np.zeros((20, 20)), 1e4, 100))
    zs = pm.bij.inverse(default_prior.sample(20000, seed=5)).double()
    mean, cov = zs.mean(0), torch.cov(zs.T)
    q = MultivariateNormalTriL(mean.float().cuda(), torch.linalg.cholesky(cov).float().cuda())
    samples, stats = seq.HMC(q, init_eps=0.5, init_l=8, n_hmc=512, num_burnin_steps=60, num_results=150,
                             adapt_trajectory=False, seed=4)
    s = samples.double().cpu()
    acc = float(stats["accept_ratio"][60:].mean())
    assert 0.5 < acc <= 1.0
    flat = s.reshape(-1, s.shape[-1])
    sd = cov.diagonal().sqrt()
    # unconstrained prior mean and std, per parameter
    assert ((flat.mean(0) - mean).abs() / sd).max() < 0.1
    assert ((flat.std(0) / sd) - 1).abs().max() < 0.1
    assert potential_scale_reduction(s.float()).max() < 1.05


def test_map_svi_hmc_sequence_runs(default_prior, default_physmodel):
    """MAP -> best -> SVI -> HMC (the reference's modelling sequence)."""
    from gigalens_gb300.cuda.diagnostics import effective_sample_size, potential_scale_reduction
    from gigalens_gb300.cuda.optimizers import Adam, PolynomialDecay
    from gigalens_gb300.cuda.simulator import LensSimulator
    from tests.helpers import gaussian_psf

    rng = np.random.default_rng(0)
    cfg = SimulatorConfig(delta_pix=0.1, num_pix=24, supersample=2, kernel_supersampled=gaussian_psf(0.2, 0.05, 9))
    truth_sim = LensSimulator(default_physmodel, cfg, bs=1)
    truth = default_prior.sample(1, seed=3)
    img = truth_sim.simulate(truth).cpu().numpy()
    obs = img + rng.normal(scale=0.2, size=img.shape)
    seq, pm = _seq(default_prior, default_physmodel, data=(obs, 0.2, 100.0), cfg=cfg)
    z = seq.MAP(Adam(PolynomialDecay(1e-2, 100, 1e-3)), n_samples=64, num_steps=100, seed=0)
    lps, _ = pm.log_prob(LensSimulator(default_physmodel, cfg, bs=64), z)
    best = z[torch.argmax(lps)]
    q_z, losses = seq.SVI(Adam(PolynomialDecay(0.0, 50, 4e-3, 2)), best, n_vi=64, num_steps=100)
    assert torch.isfinite(losses).all()
    samples, stats = seq.HMC(q_z, n_hmc=32, num_burnin_steps=20, num_results=30, init_l=3, max_leapfrog_steps=10)
    assert torch.isfinite(samples).all()
    rh = potential_scale_reduction(samples.cpu())
    ess = effective_sample_size(samples.cpu())
    assert rh.shape == (22,) and ess.shape == (22,)


def test_distributed_flags_single_process(default_prior, default_physmodel):
    """Without a process group the distributed drivers run every chain, and
    best() is the argmax of the MAP log posterior."""
    from gigalens_gb300.cuda.optimizers import Adam
    from gigalens_gb300.cuda.simulator import LensSimulator
    from tests.helpers import gaussian_psf

    rng = np.random.default_rng(1)
    cfg = SimulatorConfig(delta_pix=0.1, num_pix=24, supersample=2, kernel_supersampled=gaussian_psf(0.2, 0.05, 9))
    truth = default_prior.sample(1, seed=4)
    img = LensSimulator(default_physmodel, cfg, bs=1).simulate(truth).cpu().numpy()
    obs = img + rng.normal(scale=0.2, size=img.shape)
    seq, pm = _seq(default_prior, default_physmodel, data=(obs, 0.2, 100.0), cfg=cfg)
    z = seq.MAP(Adam(1e-2), n_samples=16, num_steps=10, seed=0, distributed=True)
    assert z.shape[0] == 16
    lps, _ = pm.log_prob(LensSimulator(default_physmodel, cfg, bs=16), z)
    assert torch.equal(seq.best(), z[torch.argmax(lps)])
    q_z, losses = seq.SVI(Adam(1e-3), seq.best(), n_vi=8, num_steps=3, distributed=True)
    assert torch.isfinite(losses).all()


def test_hmc_chees_and_dual_averaging_match_target_when_likelihood_is_flat(default_prior, default_physmodel):
    """The reference's adaptive kernel (GradientBasedTrajectoryLengthAdaptation
    + DualAveragingStepSizeAdaptation, tf/inference.py:111-125) on a flat
    likelihood: the chains reproduce the unconstrained prior's moments."""
    from gigalens_gb300.cuda.diagnostics import potential_scale_reduction
    from gigalens_gb300.cuda.inference import MultivariateNormalTriL

    seq, pm = _seq(default_prior, default_physmodel, data=(np.zeros((20, 20)), 1e4, 100))
    zs = pm.bij.inverse(default_prior.sample(20000, seed=6)).double()
    mean, cov = zs.mean(0), torch.cov(zs.T)
    q = MultivariateNormalTriL(mean.float().cuda(), torch.linalg.cholesky(cov).float().cuda())
    samples, stats = seq.HMC(q, init_eps=0.3, init_l=3, n_hmc=512, num_burnin_steps=100, num_results=150,
                             max_leapfrog_steps=30, seed=5)
    s = samples.double().cpu()
    acc = float(stats["accept_ratio"][100:].mean())
    assert 0.5 < acc <= 1.0
    assert int(stats["leapfrog_steps"][-1]) >= 1
    flat = s.reshape(-1, s.shape[-1])
    sd = cov.diagonal().sqrt()
    assert ((flat.mean(0) - mean).abs() / sd).max() < 0.1
    assert ((flat.std(0) / sd) - 1).abs().max() < 0.1
    assert potential_scale_reduction(s.float()).max() < 1.05


def test_hmc_chees_graph_equals_eager(default_prior, default_physmodel):
    """The adaptive warm-up (ChEES trajectory lengths + dual-averaging step
    size) replayed from CUDA graphs, one per leapfrog count, draws exactly
    what the eager run draws for the same seed."""
    from gigalens_gb300.cuda.inference import MultivariateNormalTriL

    seq, pm = _seq(default_prior, default_physmodel, data=(np.zeros((20, 20)), 1e4, 100))
    zs = pm.bij.inverse(default_prior.sample(4000, seed=6)).double()
    mean, cov = zs.mean(0), torch.cov(zs.T)
    q = MultivariateNormalTriL(mean.float().cuda(), torch.linalg.cholesky(cov).float().cuda())
    runs = []
    for use_graph in (False, True):
        samples, stats = seq.HMC(q, init_eps=0.3, init_l=3, n_hmc=64, num_burnin_steps=40, num_results=12,
                                 max_leapfrog_steps=12, seed=7, use_graph=use_graph)
        runs.append((samples.cpu(), stats))
    (s0, st0), (s1, st1) = runs
    assert torch.equal(st0["leapfrog_steps"], st1["leapfrog_steps"])
    assert len(set(st1["leapfrog_steps"][:32].tolist())) > 1          # the lengths really vary
    assert st1["graphs"] > 3 and st0["graphs"] == 0
    assert torch.equal(st0["step_size"].cpu(), st1["step_size"].cpu())
    assert torch.equal(s0, s1)
