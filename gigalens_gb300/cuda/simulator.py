"""``LensSimulator`` of the CUDA substrate (``gigalens/tf/simulator.py:10-165``).

``simulate`` runs the fused forward kernel (ray tracing, light, PSF and
supersample binning in one launch, ``gl_forward``).  The coordinate grid,
PSF sub-kernels and observed data live in a device plan built once per
simulator (and once per probabilistic model attached to it).
"""
from typing import Dict

import torch

from .. import _native as N
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

    def lstsq_simulate(self, params, observed_image, err_map, return_stacked=False, return_coeffs=False,
                       no_deflection=False):
        raise NotImplementedError("lstsq_simulate is provided by the least-squares kernels")
