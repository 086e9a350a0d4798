"""``LensSimulator`` of the CUDA substrate (``gigalens/tf/simulator.py:10-165``).

``simulate`` runs the fused forward kernel (ray tracing, light, PSF and
supersample binning in one launch, ``gl_forward``).  The coordinate grid,
PSF sub-kernels and observed data live in a device plan built once per
simulator (and once per probabilistic model attached to it).
"""
import ctypes
from typing import Dict

import numpy as np
import torch

from .. import _native as N
from . import autotune
from .. import simulator as _sim
from ._plan import ModelLayout, Plan


class LensSimulator(_sim.LensSimulatorInterface):
    def __init__(self, phys_model, sim_config: _sim.SimulatorConfig, bs: int):
        super().__init__(phys_model, sim_config, bs)
        self.supersample = int(sim_config.supersample or 1)
        self.layout = ModelLayout(phys_model)
        self.numPix = int(sim_config.num_pix)
        self._plan = None
        self._prob_plans: Dict[int, Plan] = {}

    # plans ----------------------------------------------------------
    def plan(self) -> Plan:
        if self._plan is None:
            self._plan = Plan(self.layout, [dict(sim_config=self.sim_config)])
        return self._plan

    def prob_plan(self, prob_model) -> Plan:
        """Plan with the model's observed image, noise model and prior."""
        key = id(prob_model)
        p = self._prob_plans.get(key)
        if p is None:
            p = Plan(self.layout, [dict(sim_config=self.sim_config, observed=prob_model.observed_numpy,
                                        background_rms=prob_model.background_rms_value,
                                        exp_time=prob_model.exp_time_value)],
                     prior=prob_model.prior)
            self._prob_plans[key] = p
        return p

    # API ------------------------------------------------------------
    def simulate(self, params, no_deflection=False):
        """Simulated images ``(bs, N, N)`` (squeezed like ``tf.squeeze`` when bs == 1)."""
        if no_deflection:
            raise NotImplementedError("no_deflection is not supported by the fused kernel")
        plan = self.plan()
        x = self.layout.flatten_params(params)
        bs = x.shape[0]
        img = torch.empty((bs, plan.max_pix), dtype=torch.float32, device=x.device)
        N.call("gl_forward", plan.handle, N.ptr(x), None, bs, None, None, N.ptr(img), None, N.stream_ptr())
        img = img.reshape(bs, self.numPix, self.numPix)
        return img.squeeze()

    def simulate_flat(self, x: torch.Tensor) -> torch.Tensor:
        """Images ``(bs, N, N)`` for flat physical parameters ``x`` ``(bs, d)``."""
        plan = self.plan()
        x = x.to(torch.float32).contiguous()
        bs = x.shape[0]
        img = torch.empty((bs, plan.max_pix), dtype=torch.float32, device=x.device)
        N.call("gl_forward", plan.handle, N.ptr(x), None, bs, None, None, N.ptr(img), None, N.stream_ptr())
        return img.reshape(bs, self.numPix, self.numPix)

    # least squares -----------------------------------------------------
    def lstsq_plan(self, observed_image, err_map, prior=None, key=None) -> Plan:
        """Plan of the linear-amplitude path for this observation and noise map."""
        obs = observed_image.detach().cpu().numpy() if torch.is_tensor(observed_image) else observed_image
        err = err_map.detach().cpu().numpy() if torch.is_tensor(err_map) else err_map
        k = key if key is not None else (id(observed_image), id(err_map))
        hit = self._lstsq_plans.get(k) if hasattr(self, "_lstsq_plans") else None
        if hit is not None and hit[1] is observed_image and hit[2] is err_map:
            return hit[0]
        if not hasattr(self, "_lstsq_plans"):
            self._lstsq_plans = {}
        p = Plan(self.layout, [dict(sim_config=self.sim_config, observed=np.asarray(obs, np.float32),
                                    err_map=None if err is None else np.asarray(err, np.float32))],
                 prior=prior)
        self._lstsq_plans[k] = (p, observed_image, err_map)
        return p

    def run_lstsq(self, plan: Plan, x: torch.Tensor, want_image=True, want_loglik=False):
        """Run the least-squares kernels on flat physical parameters ``x``."""
        x = x.to(torch.float32).contiguous()
        bs = x.shape[0]
        autotune.ensure_lstsq(plan, x)   # before the workspace query: the tuning sets its size
        nbytes = ctypes.c_size_t(0)
        D = ctypes.c_int(0)
        N.call("gl_lstsq_workspace", plan.handle, bs, ctypes.byref(nbytes), ctypes.byref(D))
        work = torch.empty(max(int(nbytes.value), 1), dtype=torch.uint8, device=x.device)
        coeffs = torch.empty((bs, D.value), dtype=torch.float32, device=x.device)
        img = torch.empty((bs, plan.max_pix), dtype=torch.float32, device=x.device) if want_image else None
        logL = torch.empty(bs, dtype=torch.float32, device=x.device) if want_loglik else None
        chi2 = torch.empty(bs, dtype=torch.float32, device=x.device) if want_loglik else None
        N.call("gl_lstsq", plan.handle, N.ptr(x), None, bs, N.ptr(work), nbytes.value, N.ptr(coeffs), N.ptr(img),
               N.ptr(logL), N.ptr(chi2), N.stream_ptr())
        return dict(coeffs=coeffs, img=img, logL=logL, chi2=chi2, work=work, D=D.value)

    def lstsq_loglik_grad(self, plan: Plan, x: torch.Tensor, coeffs: torch.Tensor) -> torch.Tensor:
        """d logL / dx of the least-squares likelihood (data-based noise) at the
        coefficients ``gl_lstsq`` returned for ``x`` (``gl_lstsq_grad``)."""
        x = x.to(torch.float32).contiguous()
        coeffs = coeffs.to(torch.float32).contiguous()
        grad = torch.empty_like(x)
        N.call("gl_lstsq_grad", plan.handle, N.ptr(x), None, x.shape[0], N.ptr(coeffs), None, None, N.ptr(grad),
               N.stream_ptr())
        return grad

    def lstsq_simulate(self, params, observed_image, err_map, return_stacked=False, return_coeffs=False,
                       no_deflection=False):
        """``tf/simulator.py:99-165``: images with the linear amplitudes solved by
        weighted least squares (pinv, rcond 1e-6)."""
        if no_deflection:
            raise NotImplementedError("no_deflection is not supported")
        plan = self.lstsq_plan(observed_image, err_map)
        x = self.layout.flatten_params(params)
        r = self.run_lstsq(plan, x, want_image=not (return_stacked or return_coeffs))
        bs, n = x.shape[0], self.numPix
        if return_stacked:
            X = r["work"][: bs * r["D"] * plan.max_pix * 4].view(torch.float32)
            return X.reshape(bs, r["D"], n, n).permute(0, 2, 3, 1).squeeze()
        if return_coeffs:
            return r["coeffs"]
        return r["img"].reshape(bs, n, n).squeeze()
