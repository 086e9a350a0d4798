"""Abstract profile API, restating ``gigalens/profile.py:5-77``.

Difference from the reference: ``params`` is a per-instance list.  The
reference appends to the class-level ``_params`` list in
``LightProfile.__init__`` (``profile.py:35-39``), so every new
``use_lstsq=True`` instance grows the shared list; here each instance gets
its own copy.  ``params`` is informational in both implementations.
"""
from abc import ABC, abstractmethod
from typing import List


class Parameterized(ABC):
    """A parameterized profile: ``name`` and the list of parameter ``params``."""

    _name: str
    _params: List[str]

    def __init__(self, *args, **kwargs):
        self.name = self._name
        self.params = list(self._params)

    def __str__(self):
        return self.name


class LightProfile(Parameterized, ABC):
    """A light profile; ``use_lstsq`` solves the amplitude linearly."""

    def __init__(self, use_lstsq=False, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self._use_lstsq = use_lstsq
        self.depth = 1
        if self._use_lstsq:
            self.params.append("amp")

    @property
    def use_lstsq(self):
        return self._use_lstsq

    @use_lstsq.setter
    def use_lstsq(self, use_lstsq: bool):
        if use_lstsq and not self._use_lstsq:
            self.params.append("amp")
        elif not use_lstsq and self._use_lstsq:
            self.params.pop()
        self._use_lstsq = use_lstsq

    @abstractmethod
    def light(self, x, y, **kwargs):
        pass


class MassProfile(Parameterized, ABC):
    """A mass profile: ``deriv(x, y, **params) -> (alpha_x, alpha_y)``."""

    @abstractmethod
    def deriv(self, x, y, **kwargs):
        pass
