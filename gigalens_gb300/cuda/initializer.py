"""Learned MAP initialiser.

A small CNN reads the observed image and proposes a Gaussian over the
unconstrained parameters; MAP starts its ensemble from draws of that
Gaussian instead of prior draws (the reference's hook is ``MAP(start=...)``,
``gigalens/inference.py:34-57``).  Architecture: 64x64 single-channel
input (a 60x60 image is zero-padded by 2 px per side), four 3x3 convolutions
of 32 channels (stride 1, then stride 2 three times) with ReLU, a 2048->256
ReLU layer and a 256->2d output layer giving the mean and log-standard
deviation of the d standardised unconstrained parameters.  Activations are
channel-major ([C][B][H][W]) so each convolution pass is one GEMM over
batch x pixels.  Weights are
stored in BF16 (the GEMM reads them as BF16 and accumulates in FP32) with
FP32 master copies for Adam.  Every layer's forward and backward pass runs on
this library's kernels (``gl_nn_*``), and one training step is one CUDA
graph.

The network is trained on (image, parameter) pairs generated by this
simulator under the configuration's noise model (``workloads.observe``).
Proposals are judged by the log posterior: when the log posterior at the
network's point proposal is below the median over prior draws, MAP starts
from the prior draws instead.
"""
import math
import time

import numpy as np
import torch

from .. import _native as N
from .. import workloads as W


def _c(fn, *args):
    N.call(fn, *args)


class LensCNN:
    def __init__(self, d=22, size=64, ch=32, hidden=256, seed=0, device=None):
        self.d, self.size, self.ch, self.hidden = d, size, ch, hidden
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dev = dev
        # conv layers: (cin, H_in, stride)
        self.convs = []
        h = size
        cin = 1
        for i, s in enumerate([1, 2, 2, 2]):
            ho = (h - 1) // s + 1
            self.convs.append(dict(cin=cin, H=h, s=s, Ho=ho))
            h, cin = ho, ch
        self.feat = ch * h * h
        shapes = []
        for L in self.convs:
            shapes += [("W", (ch, L["cin"] * 9)), ("b", (ch,))]
        shapes += [("W", (hidden, self.feat)), ("b", (hidden,)), ("W", (2 * d, hidden)), ("b", (2 * d,))]
        self.offsets = []
        off = 0
        for kind, shp in shapes:
            n = int(np.prod(shp))
            self.offsets.append((kind, shp, off, n))
            off = (off + n + 63) // 64 * 64       # keep every tensor 256-byte aligned
        self.n_params = off
        g = torch.Generator().manual_seed(seed)
        master = torch.zeros(off, dtype=torch.float32)
        for i, (kind, shp, o, n) in enumerate(self.offsets):
            if kind == "W":
                fan_in = shp[1]
                std = math.sqrt(2.0 / fan_in) if i < len(self.offsets) - 2 else 0.01
                master[o:o + n] = torch.randn(n, generator=g) * std
        self.master = master.to(dev)
        self.wbf = torch.empty(off, dtype=torch.bfloat16, device=dev)
        self.grad = torch.zeros(off, dtype=torch.float32, device=dev)
        self._cast()
        self._bufs = {}
        self.t_mean = torch.zeros(d, device=dev)
        self.t_std = torch.ones(d, device=dev)

    # ------------------------------------------------------------ parameters
    def _view(self, buf, i):
        kind, shp, o, n = self.offsets[i]
        return buf[o:o + n].view(*shp)

    def W(self, i):          # bf16 weights of layer i (0..5)
        return self._view(self.wbf, 2 * i)

    def b(self, i):
        return self._view(self.master, 2 * i + 1)

    def gW(self, i):
        return self._view(self.grad, 2 * i)

    def gb(self, i):
        return self._view(self.grad, 2 * i + 1)

    def _cast(self, stream=None):
        _c("gl_nn_cast_bf16", N.ptr(self.master), N.ptr(self.wbf), self.n_params, N.stream_ptr(stream))

    def state_dict(self):
        return dict(master=self.master.cpu(), t_mean=self.t_mean.cpu(), t_std=self.t_std.cpu(),
                    d=self.d, size=self.size, ch=self.ch, hidden=self.hidden)

    def load_state_dict(self, sd):
        self.master.copy_(sd["master"].to(self.dev))
        self.t_mean.copy_(sd["t_mean"].to(self.dev))
        self.t_std.copy_(sd["t_std"].to(self.dev))
        self._cast()

    # ------------------------------------------------------------ buffers
    def _buffers(self, B):
        if B in self._bufs:
            return self._bufs[B]
        dev, ch = self.dev, self.ch
        f = lambda *s: torch.empty(*s, dtype=torch.float32, device=dev)
        bufs = dict(col=[], act=[], dcol=[], dact=[])
        for L in self.convs:          # channel-major: [channels][B * pixels]
            BP = B * L["Ho"] * L["Ho"]
            bufs["col"].append(f(L["cin"] * 9, BP))
            bufs["act"].append(f(ch, BP))
            bufs["dcol"].append(f(L["cin"] * 9, BP) if L["cin"] > 1 else None)
            bufs["dact"].append(f(ch, BP))
        bufs["a4b"] = f(B, self.feat)
        bufs["da4b"] = f(B, self.feat)
        bufs["h1"] = f(self.hidden, B)
        bufs["out"] = f(2 * self.d, B)
        bufs["dout"] = f(2 * self.d, B)
        bufs["dh1"] = f(self.hidden, B)
        bufs["da4T"] = f(self.feat, B)
        bufs["tT"] = f(self.d, B)
        bufs["loss"] = f(self.d, B)
        self._bufs[B] = bufs
        return bufs

    @staticmethod
    def _ksplit(M, N, K, target=608):
        tiles = ((N + 127) // 128) * ((M + 31) // 32) if M <= 32 else ((N + 63) // 64) * ((M + 63) // 64)
        return int(max(1, min((target + tiles - 1) // tiles, K // 512)))

    def _gemm(self, tA, tB, bf, m, n, k, A, lda, Bm, ldb, C, ldc, s, ksplit=1):
        _c("gl_nn_gemm", tA, tB, bf, m, n, k, 1.0, N.ptr(A), lda, 0, N.ptr(Bm), ldb, 0, 0.0, N.ptr(C), ldc, 0, 1,
           int(ksplit), s)

    # ------------------------------------------------------------ passes
    def forward(self, x, stream=None):
        """x [B, 1, size, size] -> out [2d][B] (means, log-sigma)."""
        B = x.shape[0]
        bf = self._buffers(B)
        s = N.stream_ptr(stream)
        prev = x.contiguous()          # [1][B][H][W] == [B][1][H][W]
        for i, L in enumerate(self.convs):
            BP = B * L["Ho"] * L["Ho"]
            K = L["cin"] * 9
            col, act = bf["col"][i], bf["act"][i]
            _c("gl_nn_im2col3x3", N.ptr(prev), B, L["cin"], L["H"], L["H"], L["s"], N.ptr(col), s)
            self._gemm(0, 0, 1, self.ch, BP, K, self.W(i), K, col, BP, act, BP, s)
            _c("gl_nn_bias_act", N.ptr(act), N.ptr(self.b(i)), 1, self.ch, BP, 1, s)
            prev = act
        P4 = self.convs[-1]["Ho"] ** 2
        _c("gl_nn_permute01", N.ptr(bf["act"][3]), self.ch, B, P4, N.ptr(bf["a4b"]), s)
        h1, out = bf["h1"], bf["out"]
        self._gemm(0, 1, 1, self.hidden, B, self.feat, self.W(4), self.feat, bf["a4b"], self.feat, h1, B, s)
        _c("gl_nn_bias_act", N.ptr(h1), N.ptr(self.b(4)), 1, self.hidden, B, 1, s)
        self._gemm(0, 0, 1, 2 * self.d, B, self.hidden, self.W(5), self.hidden, h1, B, out, B, s)
        _c("gl_nn_bias_act", N.ptr(out), N.ptr(self.b(5)), 1, 2 * self.d, B, 0, s)
        return out

    def backward(self, dout, stream=None):
        """Gradients of all parameters (into ``self.grad``) from dout [2d][B]."""
        B = dout.shape[1]
        bf = self._buffers(B)
        s = N.stream_ptr(stream)
        h1, out, dh1 = bf["h1"], bf["out"], bf["dh1"]
        d2 = 2 * self.d
        _c("gl_nn_bias_act_backward", N.ptr(dout), N.ptr(out), 1, d2, B, 0, N.ptr(self.gb(5)), s)
        self._gemm(0, 1, 0, d2, self.hidden, B, dout, B, h1, B, self.gW(5), self.hidden, s,
                   self._ksplit(d2, self.hidden, B))
        self._gemm(1, 0, 1, self.hidden, B, d2, self.W(5), self.hidden, dout, B, dh1, B, s)
        _c("gl_nn_bias_act_backward", N.ptr(dh1), N.ptr(h1), 1, self.hidden, B, 1, N.ptr(self.gb(4)), s)
        self._gemm(0, 0, 0, self.hidden, self.feat, B, dh1, B, bf["a4b"], self.feat, self.gW(4), self.feat, s,
                   self._ksplit(self.hidden, self.feat, B))
        self._gemm(1, 0, 1, self.feat, B, self.hidden, self.W(4), self.feat, dh1, B, bf["da4T"], B, s)
        _c("gl_nn_transpose", N.ptr(bf["da4T"]), self.feat, B, N.ptr(bf["da4b"]), s)
        P4 = self.convs[-1]["Ho"] ** 2
        _c("gl_nn_permute01", N.ptr(bf["da4b"]), B, self.ch, P4, N.ptr(bf["dact"][3]), s)
        for i in range(3, -1, -1):
            L = self.convs[i]
            BP = B * L["Ho"] * L["Ho"]
            K = L["cin"] * 9
            dact, act, col = bf["dact"][i], bf["act"][i], bf["col"][i]
            _c("gl_nn_bias_act_backward", N.ptr(dact), N.ptr(act), 1, self.ch, BP, 1, N.ptr(self.gb(i)), s)
            self._gemm(0, 1, 0, self.ch, K, BP, dact, BP, col, BP, self.gW(i), K, s, self._ksplit(self.ch, K, BP))
            if i > 0:
                dcol = bf["dcol"][i]
                self._gemm(1, 0, 1, K, BP, self.ch, self.W(i), K, dact, BP, dcol, BP, s)
                _c("gl_nn_col2im3x3", N.ptr(dcol), B, L["cin"], L["H"], L["H"], L["s"], N.ptr(bf["dact"][i - 1]), s)

    def loss_grad(self, x, target, stream=None):
        """Mean Gaussian NLL over a batch (target [B, d], standardised) and all gradients."""
        B = x.shape[0]
        bf = self._buffers(B)
        s = N.stream_ptr(stream)
        out = self.forward(x, stream)
        _c("gl_nn_transpose", N.ptr(target.contiguous()), B, self.d, N.ptr(bf["tT"]), s)
        _c("gl_nn_gauss_nll", N.ptr(out), N.ptr(bf["tT"]), B, self.d, N.ptr(bf["loss"]), N.ptr(bf["dout"]), s)
        self.backward(bf["dout"], stream)
        return bf["loss"]

    def predict(self, x):
        """(mu, log_sigma) of the unconstrained parameters, each [B, d]."""
        out = self.forward(x)
        mu = out[: self.d].T * self.t_std + self.t_mean
        ls = torch.clamp(out[self.d:].T, -12.0, 12.0) + torch.log(self.t_std)
        return mu, ls


def preprocess(images, size=64, bg_rms=W.BG_RMS):
    """[n, N, N] images -> [n, 1, size, size] network input (asinh stretch, zero pad)."""
    n, h, w = images.shape
    p0, p1 = (size - h) // 2, (size - w) // 2
    x = torch.zeros((n, 1, size, size), dtype=torch.float32, device=images.device)
    x[:, 0, p0:p0 + h, p1:p1 + w] = torch.asinh(images / (2.0 * bg_rms)) / 4.0
    return x


def make_training_set(n, seed, prob_bijector, sim_config=None, chunk=8192, device=None):
    """n (image, standardised z) pairs from this simulator (config-0 geometry by default)."""
    from .simulator import LensSimulator

    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    cfg = sim_config or W.config0()
    sim = LensSimulator(W.physical_model(), cfg, bs=chunk)
    imgs = torch.empty((n, 1, 64, 64), dtype=torch.float32, device=dev)
    zs = torch.empty((n, 22), dtype=torch.float32, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    for i0 in range(0, n, chunk):
        m = min(chunk, n - i0)
        params = W.draw_params(m, seed * 1000003 + i0)
        x = W.flat(params).to(dev).contiguous()
        img = sim.simulate_flat(x)
        obs = W.observe(img, generator=gen)
        imgs[i0:i0 + m] = preprocess(obs)
        # a draw that rounds onto a Uniform bound maps to +-inf; keep targets finite
        z = torch.nan_to_num(prob_bijector.inverse(params).to(torch.float32), nan=0.0, posinf=30.0, neginf=-30.0)
        zs[i0:i0 + m] = z.clamp(-30.0, 30.0).to(dev)
    return imgs, zs


def train(net, imgs, zs, epochs=20, batch=1024, lr=1e-3, seed=0, use_graph=True, log_every=0):
    """Adam on the mean Gaussian NLL; returns the per-step loss history (device)."""
    from .optimizers import Adam, AdamState, PolynomialDecay

    n = imgs.shape[0]
    net.t_mean.copy_(zs.mean(0))
    net.t_std.copy_(zs.std(0).clamp_min(1e-6))
    steps_per_epoch = max(n // batch, 1)
    total = steps_per_epoch * epochs
    state = AdamState(net.master, Adam(PolynomialDecay(lr, max(total, 1), lr / 10)))
    xb = torch.empty((batch, 1, imgs.shape[2], imgs.shape[3]), dtype=torch.float32, device=imgs.device)
    tb = torch.empty((batch, net.d), dtype=torch.float32, device=imgs.device)
    hist = torch.zeros(total, device=imgs.device)
    g = torch.Generator(device=imgs.device)
    g.manual_seed(seed)

    def step():
        loss = net.loss_grad(xb, tb)
        hist.index_copy_(0, state.step.long().clamp_(max=total - 1), loss.mean().reshape(1))
        state.apply(net.grad)
        net._cast()

    graph = None
    it = 0
    for ep in range(epochs):
        perm = torch.randperm(n, device=imgs.device, generator=g)
        for k in range(steps_per_epoch):
            idx = perm[k * batch:(k + 1) * batch]
            torch.index_select(imgs, 0, idx, out=xb)
            torch.index_select(zs, 0, idx, out=tb)
            tb.sub_(net.t_mean).div_(net.t_std)
            if not use_graph or it == 0:
                step()
            else:
                if graph is None:
                    s = torch.cuda.Stream()
                    s.wait_stream(torch.cuda.current_stream())
                    graph = torch.cuda.CUDAGraph()
                    with torch.cuda.stream(s):
                        with torch.cuda.graph(graph, stream=s):
                            step()
                    torch.cuda.current_stream().wait_stream(s)
                graph.replay()
            it += 1
    return hist


class LearnedInitializer:
    """Proposes MAP starting ensembles from the trained network."""

    def __init__(self, net: LensCNN):
        self.net = net

    def propose(self, observed, n_chains, prob_model, simulator, seed=0, prior_z=None, spread=1.0):
        """Unconstrained MAP start ``(n_chains, d)`` for one observation and whether
        it fell back to prior draws.

        The network's point proposal (its mean) is judged by the log posterior:
        if it is below the median log posterior of ``n_chains`` prior draws, the
        prior draws are returned; otherwise chain 0 is the mean and the others
        are drawn from N(mean, (spread * sigma)^2)."""
        dev = self.net.dev
        obs = torch.as_tensor(np.asarray(observed, dtype=np.float32), device=dev)[None]
        mu, ls = self.net.predict(preprocess(obs))
        if prior_z is None:
            prior_z = prob_model.bij.inverse(prob_model.prior.sample(n_chains, seed=seed + 1)).to(dev, torch.float32)
        lp_prior, _ = prob_model.log_prob(simulator, prior_z.contiguous())
        lp_mean, _ = prob_model.log_prob(simulator, mu.contiguous())
        med = torch.nan_to_num(lp_prior, nan=-float("inf")).median()
        if not bool(torch.nan_to_num(lp_mean, nan=-float("inf"))[0] >= med):
            return prior_z.detach(), True
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        eps = torch.randn((n_chains, self.net.d), device=dev, generator=g)
        eps[0] = 0.0
        z = (mu + spread * torch.exp(ls) * eps).contiguous()
        return z.detach(), False


def _map_time(seq, start_z, lr, num_steps, threshold, check_every=1):
    """Wall seconds for MAP from ``start_z`` to reach best chi^2 <= threshold
    (None if not within num_steps), and the steps taken.  The stop test runs
    every ``check_every`` steps (1: the wall time ends at the step that
    reached the threshold)."""
    from .optimizers import Adam

    z_struct = seq.prob_model.bij.forward(start_z)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq.MAP(Adam(lr), start=z_struct, n_samples=start_z.shape[0], num_steps=num_steps, stop_chi2=threshold,
            check_every=check_every)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    hist = seq.map_chi2_history[: seq.map_steps_run].detach().cpu()
    hit = (hist <= threshold).nonzero()
    if len(hit) == 0:
        return None, seq.map_steps_run, el
    return el, int(hit[0]) + 1, el


def evaluate_time_to_map(net, n_lenses=256, n_chains=4096, num_steps=350, lr=5e-3, threshold=1.05, seed=10_000,
                         check_every=1):
    """Time to chi^2/dof <= threshold (the reference's per-pixel mean chi^2,
    tf/model.py:84-86) for MAP from prior draws and from the learned proposal,
    on ``n_lenses`` unseen config-0 lenses.  The learned time includes the
    network and the proposal's log-posterior evaluations."""
    from .inference import ModellingSequence
    from .model import ForwardProbModel
    from .simulator import LensSimulator

    prior = W.config_prior()
    cfg = W.config0()
    phys = W.physical_model()
    sim1 = LensSimulator(phys, cfg, bs=1)
    init = LearnedInitializer(net)
    rows = []
    for k in range(n_lenses):
        truth = W.draw_params(1, seed=seed + k)
        img = sim1.simulate_flat(W.flat(truth).to(net.dev))
        obs = W.observe(img, seed=seed + k)[0].cpu().numpy()
        pm = ForwardProbModel(prior, obs, background_rms=W.BG_RMS, exp_time=W.EXP_TIME)
        seq = ModellingSequence(phys, pm, cfg)
        sim = LensSimulator(phys, cfg, bs=n_chains)
        prior_z = pm.bij.inverse(prior.sample(n_chains, seed=seed + 7 * k + 1)).to(net.dev, torch.float32)
        t_prior, s_prior, _ = _map_time(seq, prior_z, lr, num_steps, threshold, check_every)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        z, fell_back = init.propose(obs, n_chains, pm, sim, seed=k, prior_z=prior_z)
        torch.cuda.synchronize()
        t_prop = time.perf_counter() - t0
        t_learn, s_learn, _ = _map_time(seq, z, lr, num_steps, threshold, check_every)
        rows.append(dict(lens=k, prior_s=t_prior, prior_steps=s_prior, learned_s=None if t_learn is None else
                         t_learn + t_prop, learned_steps=s_learn, proposal_s=t_prop, fell_back=fell_back))
    inf = float("inf")
    tp = np.array([r["prior_s"] if r["prior_s"] is not None else inf for r in rows])
    tl = np.array([r["learned_s"] if r["learned_s"] is not None else inf for r in rows])
    summary = dict(n_lenses=n_lenses, n_chains=n_chains, max_steps=num_steps, lr=lr, threshold=threshold,
                   prior_reached=float(np.isfinite(tp).mean()), learned_reached=float(np.isfinite(tl).mean()),
                   prior_median_s=float(np.median(tp)), learned_median_s=float(np.median(tl)),
                   fallbacks=int(sum(r["fell_back"] for r in rows)))
    both = np.isfinite(tp) & np.isfinite(tl)
    if both.any():
        summary["median_ratio_learned_over_prior_where_both_reached"] = float(np.median(tl[both] / tp[both]))
    # lenses where a prior draw already meets the threshold after one step do
    # not discriminate between the starts: the ratio over the others
    hard = both & np.array([r["prior_steps"] is not None and r["prior_steps"] > 1 for r in rows])
    summary["lenses_prior_needs_more_than_one_step"] = int(hard.sum())
    if hard.any():
        summary["median_ratio_where_prior_needs_more_than_one_step"] = float(np.median(tl[hard] / tp[hard]))
        summary["median_s_where_prior_needs_more_than_one_step"] = dict(prior=float(np.median(tp[hard])),
                                                                        learned=float(np.median(tl[hard])))
    summary["check_every"] = check_every
    return summary, rows


def main(argv=None):
    """Train the initialiser on simulated pairs and measure time-to-MAP, learned vs prior init."""
    import argparse
    import json

    from .. import distributions as tfd

    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=2_000_000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lenses", type=int, default=256)
    ap.add_argument("--chains", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=350)
    ap.add_argument("--map-lr", type=float, default=5e-3)
    ap.add_argument("--check-every", type=int, default=1, help="MAP steps between stop tests")
    ap.add_argument("--out", default=None, help="write the summary and per-lens rows as JSON here")
    args = ap.parse_args(argv)
    torch.cuda.set_device(0)
    prior = W.config_prior()
    bij = tfd.Chain([prior.experimental_default_event_space_bijector(), tfd.Pack(prior.sample(seed=0))])
    t0 = time.perf_counter()
    imgs, zs = make_training_set(args.pairs, seed=1, prob_bijector=bij)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = LensCNN(d=22, seed=0)
    t0 = time.perf_counter()
    hist = train(net, imgs, zs, epochs=args.epochs, batch=args.batch, lr=args.lr)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del imgs, zs
    summary, rows = evaluate_time_to_map(net, args.lenses, args.chains, args.steps, args.map_lr,
                                         check_every=args.check_every)
    summary.update(pairs=args.pairs, epochs=args.epochs, datagen_s=t_data, train_s=t_train,
                   train_steps=int(hist.numel()), final_loss=float(hist[-50:].mean()))
    print(json.dumps({"metric": "time-to-MAP chi2/dof<=1.05, learned vs prior init", **summary}), flush=True)
    if args.out:
        with open(args.out, "w") as fh:
            json.dump(dict(summary=summary, rows=rows), fh, indent=1)
    return summary, rows


if __name__ == "__main__":
    main()
