"""The MAP -> SVI -> HMC modelling sequence contract, ``gigalens/inference.py:10-109``."""
from abc import ABC, abstractmethod
from typing import Any, Optional, Union

import numpy as np

from . import model as _model
from . import simulator as _simulator


class ModellingSequenceInterface(ABC):
    """Multi-start MAP, then variational inference, then Hamiltonian Monte Carlo."""

    def __init__(self, phys_model: _model.PhysicalModel, prob_model: _model.ProbabilisticModel,
                 sim_config: _simulator.SimulatorConfig):
        self.phys_model = phys_model
        self.prob_model = prob_model
        self.sim_config = sim_config

    @abstractmethod
    def MAP(self, optimizer, start: Optional[Any], n_samples: int, num_steps: int, seed: Optional[Any]):
        """Returns the unconstrained parameters of all samples after ``num_steps`` steps."""

    @abstractmethod
    def SVI(self, optimizer, start, n_vi: int, num_steps: int, init_scales: Union[float, np.ndarray], seed: Any):
        """Fits a full-covariance Gaussian to the unconstrained posterior."""

    @abstractmethod
    def HMC(self, q_z, init_eps: float, init_l: int, n_hmc: int, num_burnin_steps: int, num_results: int,
            max_leapfrog_steps: int, seed: Any):
        """Draws posterior chains in unconstrained space."""
