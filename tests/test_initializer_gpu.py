"""Learned MAP initialiser: its hand-written forward/backward kernels against a
float64 CPU reference of the same network (same BF16-rounded weights), and
what the trained network gains over prior-draw initialisation."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def _reference_forward(net, x64):
    """The same architecture in float64 torch-CPU, weights = the BF16 copies."""
    params = {}
    h = x64
    for i, L in enumerate(net.convs):
        Wt = net.W(i).float().double().cpu().reshape(net.ch, L["cin"], 3, 3).requires_grad_(True)
        bt = net.b(i).double().cpu().requires_grad_(True)
        params["W%d" % i], params["b%d" % i] = Wt, bt
        h = F.relu(F.conv2d(h, Wt, bt, stride=L["s"], padding=1))
    h = h.reshape(h.shape[0], -1)
    W4 = net.W(4).float().double().cpu().requires_grad_(True)
    b4 = net.b(4).double().cpu().requires_grad_(True)
    W5 = net.W(5).float().double().cpu().requires_grad_(True)
    b5 = net.b(5).double().cpu().requires_grad_(True)
    params.update(W4=W4, b4=b4, W5=W5, b5=b5)
    h = F.relu(h @ W4.T + b4)
    out = h @ W5.T + b5
    return out, params


def _nll(out, t, d):
    mu, raw = out[:, :d], out[:, d:]
    ls = torch.clamp(raw, -12.0, 12.0)
    r = (t - mu) * torch.exp(-ls)
    return (ls + 0.5 * r * r).mean()


def test_cnn_forward_and_gradients_match_float64_reference():
    from gigalens_gb300.cuda.initializer import LensCNN

    torch.manual_seed(0)
    net = LensCNN(d=22, seed=3)
    # non-trivial biases so every ReLU pattern is exercised
    for i in range(6):
        net.b(i).copy_(0.05 * torch.randn_like(net.b(i)))
    B = 3
    x = torch.randn(B, 1, 64, 64, device="cuda")
    t = torch.randn(B, 22, device="cuda")
    net.grad.zero_()
    net.loss_grad(x, t)
    out_gpu = net.forward(x).T.double().cpu()          # [B, 2d]
    torch.cuda.synchronize()
    out_ref, params = _reference_forward(net, x.double().cpu())
    assert torch.allclose(out_gpu, out_ref.detach(), rtol=1e-4, atol=1e-4 * float(out_ref.detach().abs().max()))
    loss = _nll(out_ref, t.double().cpu(), 22)
    loss.backward()
    for i in range(6):
        gW = net.gW(i).double().cpu().reshape(params["W%d" % i].shape)
        gb = net.gb(i).double().cpu()
        rW, rb = params["W%d" % i].grad, params["b%d" % i].grad
        assert torch.allclose(gW, rW, rtol=1e-3, atol=1e-4 * float(rW.abs().max())), i
        assert torch.allclose(gb, rb, rtol=1e-3, atol=1e-4 * float(rb.abs().max()) + 1e-12), i


def test_learned_init_beats_prior_draws_on_unseen_lenses():
    """Trained for a few epochs on 32k simulated pairs, the network's proposals
    have a higher log posterior than prior draws on lenses it never saw."""
    from gigalens_gb300 import distributions as tfd
    from gigalens_gb300 import workloads as W
    from gigalens_gb300.cuda.initializer import LearnedInitializer, LensCNN, make_training_set, train
    from gigalens_gb300.cuda.model import ForwardProbModel
    from gigalens_gb300.cuda.simulator import LensSimulator

    prior = W.config_prior()
    bij = tfd.Chain([prior.experimental_default_event_space_bijector(), tfd.Pack(prior.sample(seed=0))])
    imgs, zs = make_training_set(32768, seed=11, prob_bijector=bij)
    net = LensCNN(d=22, seed=0)
    hist = train(net, imgs, zs, epochs=8, batch=512, lr=2e-3)
    h = hist.cpu()
    assert torch.isfinite(h).all() and h[-20:].mean() < h[:20].mean() - 0.2
    init = LearnedInitializer(net)
    cfg = W.config0()
    sim1 = LensSimulator(W.physical_model(), cfg, bs=1)
    gains = []
    for k in range(4):
        truth = W.draw_params(1, seed=900 + k)
        img = sim1.simulate_flat(W.flat(truth).cuda())
        obs = W.observe(img, seed=900 + k)[0].cpu().numpy()
        pm = ForwardProbModel(prior, obs, background_rms=W.BG_RMS, exp_time=W.EXP_TIME)
        sim = LensSimulator(W.physical_model(), cfg, bs=256)
        zp = pm.bij.inverse(prior.sample(256, seed=500 + k)).cuda().float()
        z, fell_back = init.propose(obs, 256, pm, sim, seed=k, prior_z=zp)
        lp_learned, _ = pm.log_prob(sim, z)
        lp_prior, _ = pm.log_prob(sim, zp)
        # the best starting point of the ensemble, learned vs prior draws
        gains.append(float(lp_learned.max() - lp_prior.max()))
    assert sum(g > 0 for g in gains) >= 3, gains
