"""Physical and probabilistic model containers, restating ``gigalens/model.py:7-58``."""
from abc import ABC, abstractmethod
from typing import List

from . import profile


class PhysicalModel:
    """The lensing system: ``lenses`` (mass), ``lens_light`` and ``source_light``."""

    def __init__(self, lenses: List[profile.MassProfile], lens_light: List[profile.LightProfile],
                 source_light: List[profile.LightProfile]):
        self.lenses = lenses
        self.lens_light = lens_light
        self.source_light = source_light


class ProbabilisticModel(ABC):
    """Prior plus a bijector that unconstrains physical parameters."""

    def __init__(self, prior, bij=None, *args):
        self.prior = prior
        self.bij = bij

    @abstractmethod
    def log_prob(self, simulator, z):
        """Unconstrained log posterior density of ``z`` (includes the Jacobian)."""
