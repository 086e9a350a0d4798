"""``ModellingSequence`` of the CUDA substrate (``gigalens/tf/inference.py``).

MAP (``tf/inference.py:17-41``): multi-start Adam on the unconstrained
parameters of ``n_samples`` chains.  One iteration is two launches of this
library -- the fused log-posterior+gradient kernel and the Adam kernel --
captured once in a CUDA graph and replayed; chi^2 stays on the device (the
reference synchronises every step for its progress bar, ``:40``; here the
per-step minimum is recorded on the device in ``map_chi2_history``).

SVI (``tf/inference.py:43-73``): full-covariance Gaussian guide
``MultivariateNormalTriL(loc, FillScaleTriL(Exp diag, shift 1e-6))``, the
reparameterised reverse-KL loss of ``tfp.vi.fit_surrogate_posterior``
(mean over ``n_vi`` draws of log q(z) - log p(z)), Adam on (loc, raw scale);
the whole step (draws, fused kernel, autograd of the guide, Adam) is one
CUDA graph.

HMC (``tf/inference.py:75-141``): preconditioned HMC with momentum
p ~ N(0, Sigma_q^-1) (precision = the SVI covariance, as
``MultivariateNormalPrecisionFactorLinearOperator(chol(Sigma), Sigma)``),
leapfrog, Metropolis correction per chain, dual-averaging step-size
adaptation (Hoffman & Gelman 2014 as in TFP's
``DualAveragingStepSizeAdaptation``: target 0.75, shrinkage 0.05, t0 10,
kappa 0.75, log-harmonic-mean-exp over chains) and, optionally, ChEES
trajectory-length adaptation (Hoffman, Radul & Sountsov 2021) over the first
80 % of the burn-in.  With a fixed trajectory (``adapt_trajectory=False``)
one full HMC iteration (L leapfrog steps) is one CUDA graph.  TFP's random
streams are not reproduced; the samplers are checked statistically.
"""
import functools
import math

import numpy as np
import torch

from .. import inference as _inf
from . import distributed as D
from .model import _LogProb, log_prob_and_grad
from .optimizers import Adam, AdamState
from .simulator import LensSimulator


def _cuda_dev():
    return torch.device("cuda", torch.cuda.current_device())


def _nvtx_stage(name):
    """An NVTX range (host side) around one driver stage, so a timeline
    profile shows MAP, SVI and HMC beside the library's own call ranges."""
    def wrap(fn):
        @functools.wraps(fn)
        def run(*args, **kwargs):
            with torch.cuda.nvtx.range(name):
                return fn(*args, **kwargs)
        return run
    return wrap


class ModellingSequence(_inf.ModellingSequenceInterface):
    map_chi2_history = None

    @_nvtx_stage("ModellingSequence.MAP")
    def MAP(self, optimizer: Adam = None, start=None, n_samples=500, num_steps=350, seed=0, use_graph=True,
            stop_chi2=None, check_every=25, distributed=False):
        """Multi-start Adam; returns the unconstrained parameters of all chains.

        ``stop_chi2``: stop early once the best chain's chi^2 is <= this value
        (checked every ``check_every`` steps; ``map_steps_run`` records the
        steps taken).  ``distributed``: with a process group, this rank runs its
        contiguous share of the chains (the same chains a single process would
        run) and returns them; ``best()`` gives the global best chain."""
        optimizer = optimizer if optimizer is not None else Adam(1e-3)
        dev = _cuda_dev()
        prior = self.prob_model.prior
        start = prior.sample(n_samples, seed=seed) if start is None else start
        z0 = torch.as_tensor(self.prob_model.bij.inverse(start), dtype=torch.float32)
        if distributed:
            lo, hi = D.shard_range(z0.shape[0])
            z0 = z0[lo:hi]
        trial = z0.to(dev).contiguous().clone()
        n = trial.shape[0]
        lens_sim = LensSimulator(self.phys_model, self.sim_config, bs=n)
        plan = lens_sim.prob_plan(self.prob_model)
        self._map_plan = plan
        P = float(self.prob_model.observed_numpy.size)
        logp = torch.empty(n, dtype=torch.float32, device=dev)
        chi2 = torch.empty(n, dtype=torch.float32, device=dev)
        grad = torch.empty_like(trial)
        state = AdamState(trial, optimizer)
        hist = torch.full((max(num_steps, 1),), float("nan"), dtype=torch.float32, device=dev)
        scale = -1.0 / (n * P)   # loss = mean_b(-logp_b / P)  (tf/inference.py:32)

        def step():
            log_prob_and_grad(plan, trial, logp, chi2, grad)
            idx = state.step.long().clamp_(max=hist.numel() - 1)
            hist.index_copy_(0, idx, torch.nan_to_num(chi2, nan=float("inf")).amin().reshape(1))
            state.apply(grad, scale)

        self.map_steps_run = 0
        if num_steps <= 0:
            return trial

        def reached(done):
            return stop_chi2 is not None and float(hist[:done].min()) <= stop_chi2

        if not use_graph:
            for i in range(num_steps):
                step()
                if (i + 1) % check_every == 0 and reached(i + 1):
                    self.map_steps_run = i + 1
                    break
            else:
                self.map_steps_run = num_steps
        else:
            # one eager step outside capture (allocator warm-up), then capture one step
            step()
            done = 1
            if not reached(done):
                s = torch.cuda.Stream()
                s.wait_stream(torch.cuda.current_stream())
                g = torch.cuda.CUDAGraph()
                with torch.cuda.stream(s):
                    with torch.cuda.graph(g, stream=s):
                        step()
                torch.cuda.current_stream().wait_stream(s)
                while done < num_steps:
                    n = min(check_every if stop_chi2 is not None else num_steps, num_steps - done)
                    with torch.cuda.nvtx.range("MAP steps"):
                        for _ in range(n):
                            g.replay()
                    done += n
                    if reached(done):
                        break
            self.map_steps_run = done
        self.map_chi2_history = hist
        self.map_chi2 = chi2
        self.map_log_prob = logp
        self.map_z = trial
        return trial

    def best(self):
        """The MAP chain with the highest log posterior (over every rank when
        the MAP was distributed), as the reference picks the SVI start."""
        log_prob_and_grad(self._map_plan, self.map_z, self.map_log_prob, self.map_chi2, None)
        return D.global_best(self.map_z, self.map_log_prob)

    # ------------------------------------------------------------------ SVI
    @_nvtx_stage("ModellingSequence.SVI")
    def SVI(self, optimizer, start, n_vi=250, init_scales=1e-3, num_steps=500, seed=2, use_graph=True,
            distributed=False):
        """Returns ``(q_z, losses)`` like the reference (unconstrained space).

        ``distributed``: with a process group each rank draws its share of the
        ``n_vi`` samples (seed + rank) and the ELBO and its gradient are summed
        over ranks every step (``jax/inference.py:112-117``); steps run eagerly."""
        dev = _cuda_dev()
        rank, world = D.rank_world() if distributed else (0, 1)
        n_total = n_vi
        if world > 1:
            lo, hi = D.shard_range(n_vi)
            n_vi = hi - lo
            seed = seed + rank
            use_graph = False
        start = torch.as_tensor(start, dtype=torch.float32).reshape(-1).to(dev)
        d = start.numel()
        scale = torch.as_tensor(np.ones(d, np.float32) * init_scales if np.size(init_scales) == 1
                                else np.asarray(init_scales, np.float32), device=dev)
        ntril = d * (d - 1) // 2
        theta = torch.zeros(2 * d + ntril, dtype=torch.float32, device=dev)
        theta[:d] = start
        theta[d:2 * d] = torch.log(scale - 1e-6)        # FillScaleTriL: diag = exp(raw) + 1e-6
        theta.requires_grad_(True)
        rows, cols = torch.tril_indices(d, d, -1, device=dev)
        diag_idx = torch.arange(d, device=dev)
        lens_sim = LensSimulator(self.phys_model, self.sim_config, bs=n_vi)
        plan = lens_sim.prob_plan(self.prob_model)
        state = AdamState(theta, optimizer if optimizer is not None else Adam(1e-3))
        losses = torch.zeros(max(num_steps, 1), dtype=torch.float32, device=dev)
        log2pi = math.log(2 * math.pi)
        torch.cuda.manual_seed(seed)
        grad_buf = torch.zeros_like(theta)

        def scale_tril(th):
            L = torch.zeros(d, d, dtype=th.dtype, device=dev)
            L = L.index_put((rows, cols), th[2 * d:])
            return L.index_put((diag_idx, diag_idx), torch.exp(th[d:2 * d]) + 1e-6)

        def step():
            eps = torch.randn(n_vi, d, device=dev)
            L = scale_tril(theta)
            z = theta[:d] + eps @ L.T
            logp, _ = _LogProb.apply(z, plan, None)
            logq = -0.5 * (eps * eps).sum(1) - torch.log(torch.diagonal(L)).sum() - 0.5 * d * log2pi
            loss = (logq - logp).sum() / n_total
            (g,) = torch.autograd.grad(loss, theta)
            grad_buf.copy_(g)
            if world > 1:
                # the one exchange: ELBO and gradient summed over ranks
                import torch.distributed as dist
                dist.all_reduce(grad_buf)
                loss = loss.detach().clone()
                dist.all_reduce(loss)
            losses.index_copy_(0, state.step.long().clamp_(max=losses.numel() - 1), loss.detach().reshape(1))
            state.apply(grad_buf)

        if num_steps > 0:
            _run_steps(step, num_steps, use_graph)
        with torch.no_grad():
            q_z = MultivariateNormalTriL(theta.detach()[:d].clone(), scale_tril(theta.detach()).clone())
        return q_z, losses[:num_steps]

    # ------------------------------------------------------------------ HMC
    @_nvtx_stage("ModellingSequence.HMC")
    def HMC(self, q_z, init_eps=0.3, init_l=3, n_hmc=50, num_burnin_steps=250, num_results=750,
            max_leapfrog_steps=30, seed=3, adapt_trajectory=True, adapt_step_size=True,
            target_accept_prob=0.75, use_graph=True, distributed=False, step_size_reduce="harmonic"):
        """Returns ``(samples, sample_stats)``; samples ``(num_results, n_hmc, d)``
        in unconstrained space.  ``distributed``: each rank runs its share of
        the ``n_hmc`` chains (seed + rank) with its own adaptation and returns
        its samples; ``distributed.gather_chains(samples, dim=1)`` joins them.
        ``step_size_reduce``: how the step-size adaptation combines the chains'
        acceptance probabilities, "harmonic" (the reference's, TFP's default)
        or "mean" (not dominated by the least-accepting of many chains)."""
        if distributed:
            rank, _ = D.rank_world()
            lo, hi = D.shard_range(n_hmc)
            n_hmc = hi - lo
            seed = seed + rank
        dev = _cuda_dev()
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        lens_sim = LensSimulator(self.phys_model, self.sim_config, bs=n_hmc)
        plan = lens_sim.prob_plan(self.prob_model)
        # the guide's Cholesky factor: Sigma = Lq Lq^T without re-factoring Sigma
        Lq = q_z.scale_tril.to(dev, torch.float32).contiguous()
        cov = Lq @ Lq.T
        d = cov.shape[0]
        z = q_z.sample(n_hmc, generator=gen).to(dev).contiguous()
        torch.cuda.manual_seed(seed)   # leapfrog draws use the default generator (graph-capturable)
        logp = torch.empty(n_hmc, device=dev)
        chi2 = torch.empty(n_hmc, device=dev)
        g = torch.empty_like(z)
        log_prob_and_grad(plan, z, logp, chi2, g)
        n_adapt = int(num_burnin_steps * 0.8)
        da = _DualAveraging(init_eps, target_accept_prob, dev, reduce=step_size_reduce)
        chees = _ChEES(init_l * init_eps, max_leapfrog_steps, dev) if adapt_trajectory else None
        total = num_burnin_steps + num_results
        samples = torch.empty((num_results, n_hmc, d), dtype=torch.float32, device=dev)
        acc_trace = torch.empty(total, dtype=torch.float32, device=dev)
        eps_trace = torch.empty(total, dtype=torch.float32, device=dev)
        L_trace = []
        # buffers reused by every iteration (graph-stable)
        zp, gp, lpp = torch.empty_like(z), torch.empty_like(g), torch.empty_like(logp)
        p0 = torch.empty_like(z)
        pp = torch.empty_like(z)
        u_acc = torch.empty(n_hmc, device=dev)
        z_before = torch.empty_like(z)
        log_acc = torch.empty(n_hmc, device=dev)
        it_dev = torch.zeros(1, dtype=torch.int64, device=dev)   # iteration index (trace slot)
        L_host = torch.empty(1, dtype=torch.int32).pin_memory()
        eps_dev = da.step_size                  # (1,) device tensor

        def kinetic(p):
            q = p @ Lq                          # K = 0.5 p^T Sigma p = 0.5 |Lq^T p|^2
            return 0.5 * (q * q).sum(1)

        def leapfrog(L):
            xi = torch.randn(n_hmc, d, device=dev)
            p0.copy_(torch.linalg.solve_triangular(Lq.T, xi.T, upper=True).T)   # p ~ N(0, Sigma^-1)
            zp.copy_(z)
            gp.copy_(g)
            pp.copy_(p0 + 0.5 * eps_dev * gp)
            for i in range(L):
                zp.add_(eps_dev * (pp @ cov))
                log_prob_and_grad(plan, zp, lpp, chi2, gp)
                pp.add_((eps_dev if i < L - 1 else 0.5 * eps_dev) * gp)
            log_accept = (lpp - kinetic(pp)) - (logp - kinetic(p0))
            log_accept = torch.nan_to_num(log_accept, nan=-float("inf"))
            u_acc.copy_(torch.rand(n_hmc, device=dev))
            accept = torch.log(u_acc) < log_accept
            z.copy_(torch.where(accept[:, None], zp, z))
            g.copy_(torch.where(accept[:, None], gp, g))
            logp.copy_(torch.where(accept, lpp, logp))
            log_acc.copy_(log_accept)

        # Per iteration: `pre` (the trajectory length on the device), the
        # leapfrog transition of that length, `post` (traces and adaptation on
        # the device).  With use_graph each piece is a CUDA graph, one per
        # leapfrog count; the host reads only the count (one 4-byte copy) to
        # pick the graph.  A piece runs eagerly the first time and is captured
        # afterwards, so graph and eager runs execute the same kernels with the
        # same random numbers.
        def pre(adapting):
            if chees is None:
                return None

            def f():
                if adapting:
                    z_before.copy_(z)
                    chees.draw_steps(eps_dev)
                else:
                    chees.final_steps(eps_dev)
            return f

        def post(adapting, at_end):
            def f():
                acc_trace.index_copy_(0, it_dev, torch.exp(torch.clamp(log_acc, max=0.0)).mean().reshape(1))
                if adapt_step_size and adapting:
                    da.update(log_acc)
                elif adapt_step_size and at_end:
                    da.finalize()
                if chees is not None and adapting:
                    chees.update(z_before, z, pp @ cov, log_acc, eps_dev)
                eps_trace.index_copy_(0, it_dev, eps_dev)
                it_dev.add_(1)
            return f

        graphs = {}

        def run(key, fn):
            if fn is None:
                return
            if not use_graph:
                fn()
                return
            gph = graphs.get(key)
            if gph is None:
                fn()                            # this iteration's real work
                graphs[key] = _capture_only(fn)
            else:
                gph.replay()

        for it in range(total):
            adapting = it < n_adapt
            torch.cuda.nvtx.range_push("HMC iteration")
            run(("pre", adapting), pre(adapting))
            if chees is not None:
                L_host.copy_(chees.L_dev, non_blocking=False)
                L = int(L_host[0])
            else:
                L = int(init_l)
            L_trace.append(L)
            run(("leap", L), lambda: leapfrog(L))
            run(("post", adapting, it == n_adapt), post(adapting, it == n_adapt))
            if it >= num_burnin_steps:
                samples[it - num_burnin_steps].copy_(z)
            torch.cuda.nvtx.range_pop()
        stats = {"accept_ratio": acc_trace, "step_size": eps_trace,
                 "leapfrog_steps": torch.tensor(L_trace), "target_log_prob": logp,
                 "graphs": len(graphs)}
        return samples, stats


def _capture_only(fn):
    """Capture ``fn`` in a CUDA graph without running it (the caller has just
    run it eagerly, which also warmed up the libraries it calls)."""
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            fn()
    torch.cuda.current_stream().wait_stream(s)
    return g


def _run_steps(step, num_steps, use_graph):
    """Run ``step`` ``num_steps`` times: eagerly once, then from a CUDA graph."""
    step()
    if num_steps == 1:
        return
    if not use_graph:
        for _ in range(num_steps - 1):
            step()
        return
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            step()
    torch.cuda.current_stream().wait_stream(s)
    for _ in range(num_steps - 1):
        g.replay()


class MultivariateNormalTriL:
    """The SVI guide: N(loc, L L^T) in unconstrained space."""

    def __init__(self, loc, scale_tril):
        self.loc = loc
        self.scale_tril = scale_tril

    def mean(self):
        return self.loc

    def covariance(self):
        return self.scale_tril @ self.scale_tril.T

    def sample(self, n=(), seed=None, generator=None):
        shape = (n,) if isinstance(n, int) else tuple(n)
        if generator is None:
            generator = torch.Generator(device=self.loc.device)
            generator.manual_seed(0 if seed is None else int(seed))
        eps = torch.randn(*shape, self.loc.numel(), device=self.loc.device, generator=generator)
        return self.loc + eps @ self.scale_tril.T

    def log_prob(self, z):
        r = torch.linalg.solve_triangular(self.scale_tril, (z - self.loc).reshape(-1, self.loc.numel()).T,
                                          upper=False).T
        d = self.loc.numel()
        return (-0.5 * (r * r).sum(1) - torch.log(torch.diagonal(self.scale_tril)).sum()
                - 0.5 * d * math.log(2 * math.pi))


class _DualAveraging:
    """Shared step size adapted toward ``target`` acceptance.  ``reduce``
    combines the chains' acceptance probabilities: "harmonic" (the
    log-harmonic-mean-exp of TFP's DualAveragingStepSizeAdaptation default,
    which the least-accepting chains dominate) or "mean" (their average)."""

    def __init__(self, init_eps, target, dev, shrinkage=0.05, t0=10.0, kappa=0.75, reduce="harmonic"):
        if reduce not in ("harmonic", "mean"):
            raise ValueError("step_size_reduce must be 'harmonic' or 'mean'")
        self.reduce = reduce
        self.step_size = torch.tensor([float(init_eps)], device=dev)
        self.mu = math.log(10.0 * init_eps)
        self.target, self.gamma, self.t0, self.kappa = target, shrinkage, t0, kappa
        self.err_sum = torch.zeros(1, device=dev)
        self.log_avg = torch.tensor([math.log(init_eps)], device=dev)
        self.t = torch.zeros(1, device=dev)   # updates so far (on the device: graph-replayable)

    def update(self, log_accept):
        self.t.add_(1.0)
        t = self.t
        la = torch.clamp(log_accept, max=0.0)
        if self.reduce == "mean":
            p = torch.exp(la).mean()
        else:
            # log-harmonic-mean-exp of the acceptance ratios over chains
            red = -(torch.logsumexp(-la, 0) - math.log(la.numel()))
            p = torch.exp(red)
        self.err_sum.add_(self.target - p)
        log_eps = self.mu - torch.sqrt(t) / self.gamma * self.err_sum / (t + self.t0)
        w = torch.pow(t, -self.kappa)
        self.log_avg.copy_(w * log_eps + (1 - w) * self.log_avg)
        self.step_size.copy_(torch.exp(log_eps))

    def finalize(self):
        self.step_size.copy_(torch.exp(self.log_avg))


class _ChEES:
    """Trajectory length adaptation by the ChEES criterion (jittered lengths,
    Adam on log T with learning rate 0.025, beta1 = 0).  All state lives on
    the device, so the adapting iterations replay as CUDA graphs; the
    leapfrog count of the next transition is ``L_dev``."""

    def __init__(self, init_T, max_steps, dev, lr=0.025, beta2=0.95):
        self.max_steps = int(max_steps)
        self.lr, self.b2 = lr, beta2
        self.logT = torch.tensor([math.log(max(init_T, 1e-6))], device=dev)
        self.avg_logT = self.logT.clone()
        self.v = torch.zeros(1, device=dev)
        self.k = torch.zeros(1, device=dev)
        self.u = torch.ones(1, device=dev)
        self.L_dev = torch.ones(1, dtype=torch.int32, device=dev)

    def _steps(self, T, eps):
        L = torch.ceil(T / torch.clamp(eps, min=1e-12))
        self.L_dev.copy_(torch.clamp(torch.nan_to_num(L, nan=1.0), 1.0, float(self.max_steps)).to(torch.int32))

    def draw_steps(self, eps):
        """Jitter u ~ U(0.001, 1) (the default CUDA generator) and L = ceil(u T / eps)."""
        self.u.copy_(torch.rand(1, device=self.u.device) * 0.999 + 0.001)
        self._steps(torch.exp(self.logT) * self.u, eps)

    def final_steps(self, eps):
        self._steps(torch.exp(self.avg_logT), eps)

    def update(self, z0, z1, v1, log_accept, eps):
        a = torch.exp(torch.clamp(log_accept, max=0.0))
        m0 = z0.mean(0, keepdim=True)
        m1 = z1.mean(0, keepdim=True)
        diff = ((z1 - m1) ** 2).sum(1) - ((z0 - m0) ** 2).sum(1)
        gT = (a * diff * ((z1 - m1) * v1).sum(1)).sum() / a.sum().clamp_min(1e-12) * self.u
        g = -gT * torch.exp(self.logT)          # gradient of -ChEES with respect to log T
        ok = torch.isfinite(g)
        g = torch.where(ok, g, torch.zeros_like(g))
        k = self.k + ok.float()
        v = torch.where(ok, self.b2 * self.v + (1 - self.b2) * g * g, self.v)
        vhat = v / (1 - torch.pow(torch.full_like(k, self.b2), k)).clamp_min(1e-30)
        logT = self.logT - self.lr * g / (torch.sqrt(vhat) + 1e-8)
        logT = torch.minimum(logT, torch.log(self.max_steps * torch.clamp(eps, min=1e-12)))
        w = torch.pow(k.clamp_min(1.0), -0.75)
        avg = w * logT + (1 - w) * self.avg_logT
        self.logT.copy_(torch.where(ok, logT, self.logT))
        self.avg_logT.copy_(torch.where(ok, avg, self.avg_logT))
        self.v.copy_(v)
        self.k.copy_(k)
