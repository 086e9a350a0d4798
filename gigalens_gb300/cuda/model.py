"""Probabilistic models of the CUDA substrate (``gigalens/tf/model.py``).

``ForwardProbModel.log_prob`` is one kernel launch (``gl_log_prob``): the
unconstraining bijector, the simulation, the Gaussian likelihood with
model-based noise, chi^2, the prior log density and the bijector's
log-Jacobian, and -- when ``z`` requires a gradient -- the hand-written
adjoint, all per sample on the GPU.  The gradient is exposed through a
``torch.autograd.Function``.
"""
import numpy as np
import torch

from .. import _native as N
from . import autotune
from .. import distributions as dist
from .. import model as _model


class _LogProb(torch.autograd.Function):
    @staticmethod
    def forward(ctx, z, plan, img_id):
        z = z.detach().to(torch.float32).contiguous()
        bs = z.shape[0]
        logp = torch.empty(bs, dtype=torch.float32, device=z.device)
        chi2 = torch.empty(bs, dtype=torch.float32, device=z.device)
        need = ctx.needs_input_grad[0]
        grad = torch.empty_like(z) if need else None
        N.call("gl_log_prob", plan.handle, N.ptr(z), N.ptr(img_id), bs, N.ptr(logp), N.ptr(chi2), N.ptr(grad),
               None, N.stream_ptr())
        ctx.mark_non_differentiable(chi2)
        if need:
            ctx.save_for_backward(grad)
        return logp, chi2

    @staticmethod
    def backward(ctx, g_logp, g_chi2):
        (grad,) = ctx.saved_tensors
        return grad * g_logp.unsqueeze(1), None, None


def log_prob_and_grad(plan, z, logp=None, chi2=None, grad=None, img_id=None, stream=None):
    """Fused ``logp, chi2, d logp / dz`` into caller buffers (graph-capturable;
    the plan's launch shape is tuned on the first call outside a capture)."""
    autotune.ensure_fused(plan, z, img_id)
    bs = z.shape[0]
    N.call("gl_log_prob", plan.handle, N.ptr(z), N.ptr(img_id), bs, N.ptr(logp), N.ptr(chi2), N.ptr(grad),
           None, N.stream_ptr(stream))


class ForwardProbModel(_model.ProbabilisticModel):
    """Log posterior with the simulated image as the noise-variance estimator
    (``tf/model.py:9-86``).  Linear parameters are not solved for."""

    def __init__(self, prior, observed_image=None, background_rms=None, exp_time=None):
        super().__init__(prior)
        obs = observed_image.detach().cpu().numpy() if torch.is_tensor(observed_image) else observed_image
        self.observed_numpy = np.asarray(obs, dtype=np.float32)
        self.background_rms_value = float(background_rms)
        self.exp_time_value = float(exp_time)
        self.observed_image = torch.as_tensor(self.observed_numpy)
        self.background_rms = torch.tensor(self.background_rms_value)
        self.exp_time = torch.tensor(self.exp_time_value)
        example = prior.sample(seed=0)
        self.pack_bij = dist.Pack(example)
        self.unconstraining_bij = prior.experimental_default_event_space_bijector()
        self.bij = dist.Chain([self.unconstraining_bij, self.pack_bij])

    def log_prob(self, simulator, z):
        """Unconstrained log posterior ``(bs,)`` and chi^2 ``(bs,)`` of ``z`` ``(bs, d)``."""
        plan = simulator.prob_plan(self)
        z = torch.as_tensor(z)
        if z.device.type != "cuda":
            z = z.to(torch.device("cuda", torch.cuda.current_device()))
        if z.dim() == 1:
            z = z[None]
        autotune.ensure_fused(plan, z.detach().to(torch.float32).contiguous())
        return _LogProb.apply(z, plan, None)


class _LstsqLogL(torch.autograd.Function):
    """Likelihood of the least-squares image: value by ``gl_lstsq``, gradient by
    ``gl_lstsq_grad`` (the coefficients minimise chi^2 for the fixed noise map,
    so the derivative through them vanishes)."""

    @staticmethod
    def forward(ctx, x, simulator, plan):
        r = simulator.run_lstsq(plan, x.detach(), want_image=False, want_loglik=True)
        ctx.mark_non_differentiable(r["chi2"])
        ctx.simulator, ctx.plan = simulator, plan
        ctx.save_for_backward(x.detach(), r["coeffs"])
        return r["logL"], r["chi2"]

    @staticmethod
    def backward(ctx, g_logL, g_chi2):
        x, coeffs = ctx.saved_tensors
        grad = ctx.simulator.lstsq_loglik_grad(ctx.plan, x, coeffs)
        return grad * g_logL.unsqueeze(1), None, None


class BackwardProbModel(_model.ProbabilisticModel):
    """Log posterior with the observed image as the noise estimator and the
    linear light amplitudes solved by least squares (``tf/model.py:89-163``).

    ``fldj_of_x`` keeps the reference's TensorFlow behaviour of evaluating the
    bijector's log-Jacobian at the physical parameters x (``tf/model.py:160``);
    ``False`` evaluates it at the unconstrained z, as the JAX substrate does
    (``jax/model.py:77``)."""

    def __init__(self, prior, observed_image, background_rms, exp_time, fldj_of_x=True):
        super().__init__(prior)
        obs = observed_image.detach().cpu().numpy() if torch.is_tensor(observed_image) else observed_image
        self.observed_numpy = np.asarray(obs, dtype=np.float32)
        self.background_rms_value = float(background_rms)
        self.exp_time_value = float(exp_time)
        err = np.sqrt(np.float32(background_rms) ** 2 +
                      np.clip(self.observed_numpy, 0, np.inf) / np.float32(exp_time)).astype(np.float32)
        self.err_numpy = err
        self.observed_image = torch.as_tensor(self.observed_numpy)
        self.err_map = torch.as_tensor(err)
        self.fldj_of_x = fldj_of_x
        example = prior.sample(seed=0)
        self.pack_bij = dist.Pack(example)
        self.unconstraining_bij = prior.experimental_default_event_space_bijector()
        self.bij = dist.Chain([self.unconstraining_bij, self.pack_bij])

    def log_prob(self, simulator, z):
        z = torch.as_tensor(z)
        if z.device.type != "cuda":
            z = z.to(torch.device("cuda", torch.cuda.current_device()))
        if z.dim() == 1:
            z = z[None]
        plan = simulator.lstsq_plan(self.observed_numpy, self.err_numpy, key=("backward", id(self)))
        x = self.bij.forward(z)
        xflat = torch.stack([v.reshape(-1) for v in dist.flatten(x)], dim=1).to(torch.float32)
        logL, chi2 = _LstsqLogL.apply(xflat, simulator, plan)
        at = x if self.fldj_of_x else self.pack_bij.forward(z)
        log_prior = self.prior.log_prob(x) + self.unconstraining_bij.forward_log_det_jacobian(at)
        return logL + log_prior, chi2
