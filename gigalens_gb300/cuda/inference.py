"""``ModellingSequence`` of the CUDA substrate (``gigalens/tf/inference.py``).

MAP: multi-start Adam on the unconstrained parameters of ``n_samples``
chains (``tf/inference.py:17-41``).  One iteration is two device launches --
the fused log-posterior+gradient kernel and the Adam kernel -- captured once
in a CUDA graph and replayed ``num_steps`` times; chi^2 of every chain stays
on the device (the reference synchronises every step for its progress bar,
``tf/inference.py:40``; here the per-step minimum is recorded on the device in
``map_chi2_history``).
"""
import torch

from .. import inference as _inf
from .model import log_prob_and_grad
from .optimizers import Adam, AdamState
from .simulator import LensSimulator


def _cuda_dev():
    return torch.device("cuda", torch.cuda.current_device())


class ModellingSequence(_inf.ModellingSequenceInterface):
    map_chi2_history = None

    def MAP(self, optimizer: Adam = None, start=None, n_samples=500, num_steps=350, seed=0, use_graph=True):
        optimizer = optimizer if optimizer is not None else Adam(1e-3)
        dev = _cuda_dev()
        prior = self.prob_model.prior
        start = prior.sample(n_samples, seed=seed) if start is None else start
        z0 = torch.as_tensor(self.prob_model.bij.inverse(start), dtype=torch.float32)
        trial = z0.to(dev).contiguous().clone()
        n = trial.shape[0]
        lens_sim = LensSimulator(self.phys_model, self.sim_config, bs=n)
        plan = lens_sim.prob_plan(self.prob_model)
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

        if num_steps <= 0:
            return trial
        if not use_graph:
            for _ in range(num_steps):
                step()
        else:
            # one eager step outside capture (allocator warm-up), then capture one step
            step()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    step()
            torch.cuda.current_stream().wait_stream(s)
            for _ in range(num_steps - 1):
                g.replay()
        self.map_chi2_history = hist
        self.map_chi2 = chi2
        self.map_log_prob = logp
        return trial

    def SVI(self, optimizer, start, n_vi=250, init_scales=1e-3, num_steps=500, seed=2):
        raise NotImplementedError

    def HMC(self, q_z, init_eps=0.3, init_l=3, n_hmc=50, num_burnin_steps=250, num_results=750,
            max_leapfrog_steps=30, seed=3):
        raise NotImplementedError
