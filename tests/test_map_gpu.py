"""ModellingSequence.MAP on the GPU, mirroring ``tests/tf/test_model.py:29-42``
of the reference, plus graph-vs-eager equality of the captured step."""
import numpy as np
import pytest
import torch

from gigalens_gb300 import distributions as tfd
from gigalens_gb300.simulator import SimulatorConfig

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def test_map(default_prior, default_physmodel, default_data):
    from gigalens_gb300.cuda.inference import ModellingSequence
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.optimizers import Adam

    prob_model = ForwardProbModel(default_prior, *default_data)
    sim_config = SimulatorConfig(delta_pix=0.05, num_pix=20)
    model_seq = ModellingSequence(default_physmodel, prob_model, sim_config)
    start = prob_model.prior.sample(2, seed=0)
    ret = model_seq.MAP(Adam(0), start, n_samples=2, num_steps=5, seed=0)
    end = prob_model.bij.forward(ret.cpu())
    for a, b in zip(tfd.flatten(start), tfd.flatten(end)):
        assert torch.allclose(a, b, rtol=1e-5, atol=1e-6)
    ret = model_seq.MAP(Adam(1e-3), start, n_samples=2, num_steps=5, seed=0)
    end = prob_model.bij.forward(ret.cpu())
    assert not all(torch.allclose(a, b) for a, b in zip(tfd.flatten(start), tfd.flatten(end)))


def test_map_graph_equals_eager_and_improves(default_prior, default_physmodel):
    from gigalens_gb300.cuda.inference import ModellingSequence
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.optimizers import Adam, PolynomialDecay
    from tests.helpers import gaussian_psf

    rng = np.random.default_rng(0)
    obs = rng.normal(scale=0.2, size=(32, 32)).astype(np.float32) + 0.5
    pm = ForwardProbModel(default_prior, obs, background_rms=0.2, exp_time=100.0)
    cfg = SimulatorConfig(delta_pix=0.1, num_pix=32, supersample=2, kernel_supersampled=gaussian_psf(0.2, 0.05, 9))
    seq = ModellingSequence(default_physmodel, pm, cfg)
    start = default_prior.sample(16, seed=1)
    opt = lambda: Adam(PolynomialDecay(1e-2, 30, 1e-3))
    a = seq.MAP(opt(), start, n_samples=16, num_steps=30, use_graph=True)
    hist = seq.map_chi2_history.cpu()
    b = seq.MAP(opt(), start, n_samples=16, num_steps=30, use_graph=False)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    assert torch.isfinite(hist).all() and hist[-1] < hist[0]
