"""Prior distributions and bijectors: the subset of TensorFlow Probability the
reference's users write priors with (``tests/conftest.py:21-73``,
``tf-demo.ipynb`` cell 2) and the reference's models consume
(``tf/model.py:38-51``), restated in PyTorch.

Covered: ``Normal``, ``LogNormal``, ``Uniform``, ``TruncatedNormal``,
``JointDistributionNamed`` (dict of leaves), ``JointDistributionSequential``
(list of parts), their ``experimental_default_event_space_bijector()``
(Identity / Exp / Sigmoid(low, high) per leaf), ``Chain``, and the
``tf.nest`` flatten order (lists in order, dict keys sorted).

Semantics restated from TFP's documented behaviour (TFP >= 0.15 is not
importable here, so these are not pinned against it):
  * Normal(loc, scale).log_prob = -((x-loc)/scale)^2/2 - log(scale) - log(2 pi)/2
  * LogNormal = exp of Normal: log_prob(x) = Normal.log_prob(log x) - log x
  * Uniform(low, high).log_prob = -log(high-low) on [low, high), -inf outside
  * TruncatedNormal = Normal renormalised to [low, high], -inf outside
  * default bijectors: Normal -> Identity, LogNormal -> Exp,
    Uniform / TruncatedNormal -> Sigmoid(low, high) with
    forward(z) = low + (high-low) sigmoid(z) and
    log|det J| = log(high-low) - softplus(-z) - softplus(z)
Sampling uses a torch.Generator seeded from ``seed``; TFP's random streams
are not reproduced.
"""
import math
from typing import Any, List

import numpy as np
import torch

from . import _native

LOG_2PI = math.log(2.0 * math.pi)


# ----------------------------------------------------------------- nest
def flatten(struct) -> List[Any]:
    """Leaves in ``tf.nest.flatten`` order (lists/tuples in order, dict keys sorted)."""
    if isinstance(struct, dict):
        out = []
        for k in sorted(struct.keys()):
            out.extend(flatten(struct[k]))
        return out
    if isinstance(struct, (list, tuple)):
        out = []
        for v in struct:
            out.extend(flatten(v))
        return out
    return [struct]


def pack_sequence_as(structure, flat):
    """Inverse of ``flatten``: fill ``structure``'s shape with ``flat``."""
    it = iter(flat)

    def build(s):
        if isinstance(s, dict):
            return {k: build(s[k]) for k in sorted(s.keys())}
        if isinstance(s, (list, tuple)):
            return type(s)(build(v) for v in s) if isinstance(s, tuple) else [build(v) for v in s]
        return next(it)

    out = build(structure)
    return out


def map_structure(fn, *structs):
    leaves = [flatten(s) for s in structs]
    return pack_sequence_as(structs[0], [fn(*xs) for xs in zip(*leaves)])


def _gen(seed):
    g = torch.Generator()
    g.manual_seed(int(seed) if seed is not None else int(torch.randint(0, 2 ** 31 - 1, ()).item()))
    return g


def _shape(sample_shape):
    if sample_shape is None:
        return ()
    if isinstance(sample_shape, int):
        return (sample_shape,)
    return tuple(sample_shape)


# ----------------------------------------------------------------- bijectors
class Bijector:
    def forward(self, x):
        raise NotImplementedError

    def inverse(self, y):
        raise NotImplementedError

    def forward_log_det_jacobian(self, x):
        raise NotImplementedError


class Identity(Bijector):
    def forward(self, x):
        return x

    def inverse(self, y):
        return y

    def forward_log_det_jacobian(self, x):
        return torch.zeros_like(torch.as_tensor(x))


class Exp(Bijector):
    def forward(self, x):
        return torch.exp(x)

    def inverse(self, y):
        return torch.log(y)

    def forward_log_det_jacobian(self, x):
        return torch.as_tensor(x)


class Sigmoid(Bijector):
    """``low + (high - low) * sigmoid(x)``."""

    def __init__(self, low, high):
        self.low, self.high = float(low), float(high)

    def forward(self, x):
        return self.low + (self.high - self.low) * torch.sigmoid(x)

    def inverse(self, y):
        return torch.log(y - self.low) - torch.log(self.high - y)

    def forward_log_det_jacobian(self, x):
        F = torch.nn.functional
        return math.log(self.high - self.low) - F.softplus(-x) - F.softplus(x)


class JointMap(Bijector):
    """Applies a structure of bijectors leafwise; the log-det sums over leaves."""

    def __init__(self, bijectors):
        self.bijectors = bijectors

    def forward(self, x):
        return map_structure(lambda b, v: b.forward(v), self.bijectors, x)

    def inverse(self, y):
        return map_structure(lambda b, v: b.inverse(v), self.bijectors, y)

    def forward_log_det_jacobian(self, x):
        terms = [b.forward_log_det_jacobian(v) for b, v in zip(flatten(self.bijectors), flatten(x))]
        return sum(terms)


class Pack(Bijector):
    """``(bs, d)`` tensor <-> structure of ``(bs,)`` leaves (``tf/model.py:42-49``)."""

    def __init__(self, example):
        self.example = example
        self.size = len(flatten(example))

    def forward(self, z):
        z = torch.as_tensor(z)
        return pack_sequence_as(self.example, [z[..., i] for i in range(self.size)])

    def inverse(self, x):
        return torch.stack([torch.as_tensor(v) for v in flatten(x)], dim=-1)

    def forward_log_det_jacobian(self, z):
        return torch.zeros(torch.as_tensor(z).shape[:-1])


class Chain(Bijector):
    """``Chain([A, B]).forward(x) = A.forward(B.forward(x))`` (TFP order)."""

    def __init__(self, bijectors):
        self.bijectors = list(bijectors)

    def forward(self, x):
        for b in reversed(self.bijectors):
            x = b.forward(x)
        return x

    def inverse(self, y):
        for b in self.bijectors:
            y = b.inverse(y)
        return y

    def forward_log_det_jacobian(self, x):
        total = 0
        for b in reversed(self.bijectors):
            total = total + b.forward_log_det_jacobian(x)
            x = b.forward(x)
        return total


# ----------------------------------------------------------------- leaves
class Distribution:
    def sample(self, sample_shape=(), seed=None, generator=None):
        raise NotImplementedError

    def log_prob(self, x):
        raise NotImplementedError

    def experimental_default_event_space_bijector(self):
        raise NotImplementedError

    def gl_leaf(self):
        """(dist code, a, b, c, d) for the C ABI's gl_prior_leaf."""
        raise NotImplementedError


class Normal(Distribution):
    def __init__(self, loc, scale):
        self.loc, self.scale = float(loc), float(scale)

    def sample(self, sample_shape=(), seed=None, generator=None):
        g = generator if generator is not None else _gen(seed)
        return (self.loc + self.scale * torch.randn(_shape(sample_shape), generator=g,
                                                    dtype=torch.float64)).float()

    def log_prob(self, x):
        x = torch.as_tensor(x)
        u = (x - self.loc) / self.scale
        return -0.5 * u * u - math.log(self.scale) - 0.5 * LOG_2PI

    def experimental_default_event_space_bijector(self):
        return Identity()

    def gl_leaf(self):
        return (_native.GL_DIST_NORMAL, self.loc, self.scale, 0.0, 0.0)


class LogNormal(Distribution):
    def __init__(self, loc, scale):
        self.loc, self.scale = float(loc), float(scale)

    def sample(self, sample_shape=(), seed=None, generator=None):
        g = generator if generator is not None else _gen(seed)
        n = self.loc + self.scale * torch.randn(_shape(sample_shape), generator=g, dtype=torch.float64)
        return torch.exp(n).float()

    def log_prob(self, x):
        x = torch.as_tensor(x)
        y = torch.log(x)
        u = (y - self.loc) / self.scale
        return -0.5 * u * u - math.log(self.scale) - 0.5 * LOG_2PI - y

    def experimental_default_event_space_bijector(self):
        return Exp()

    def gl_leaf(self):
        return (_native.GL_DIST_LOGNORMAL, self.loc, self.scale, 0.0, 0.0)


class Uniform(Distribution):
    def __init__(self, low=0.0, high=1.0):
        self.low, self.high = float(low), float(high)

    def sample(self, sample_shape=(), seed=None, generator=None):
        g = generator if generator is not None else _gen(seed)
        u = torch.rand(_shape(sample_shape), generator=g, dtype=torch.float64)
        return (self.low + (self.high - self.low) * u).float()

    def log_prob(self, x):
        x = torch.as_tensor(x)
        inside = (x >= self.low) & (x < self.high)
        val = torch.full_like(x, -math.log(self.high - self.low))
        return torch.where(inside, val, torch.full_like(x, -math.inf))

    def experimental_default_event_space_bijector(self):
        return Sigmoid(self.low, self.high)

    def gl_leaf(self):
        return (_native.GL_DIST_UNIFORM, self.low, self.high, 0.0, 0.0)


def _ndtr(x):
    return 0.5 * math.erfc(-x / math.sqrt(2.0))


class TruncatedNormal(Distribution):
    def __init__(self, loc, scale, low, high):
        self.loc, self.scale, self.low, self.high = float(loc), float(scale), float(low), float(high)
        a = (self.low - self.loc) / self.scale
        b = (self.high - self.loc) / self.scale
        self._Fa, self._Fb = _ndtr(a), _ndtr(b)
        self._logZ = math.log(self._Fb - self._Fa)

    def sample(self, sample_shape=(), seed=None, generator=None):
        g = generator if generator is not None else _gen(seed)
        u = torch.rand(_shape(sample_shape), generator=g, dtype=torch.float64)
        p = self._Fa + (self._Fb - self._Fa) * u
        x = self.loc + self.scale * torch.special.ndtri(p)
        return x.clamp(self.low, self.high).float()

    def log_prob(self, x):
        x = torch.as_tensor(x)
        u = (x - self.loc) / self.scale
        lp = -0.5 * u * u - math.log(self.scale) - 0.5 * LOG_2PI - self._logZ
        inside = (x >= self.low) & (x <= self.high)
        return torch.where(inside, lp, torch.full_like(lp, -math.inf))

    def experimental_default_event_space_bijector(self):
        return Sigmoid(self.low, self.high)

    def gl_leaf(self):
        return (_native.GL_DIST_TRUNCNORMAL, self.loc, self.scale, self.low, self.high)


# ----------------------------------------------------------------- joints
class _Joint(Distribution):
    parts: Any

    def structure(self):
        """``parts`` with nested joint distributions replaced by their parts."""
        def expand(s):
            if isinstance(s, _Joint):
                return s.structure()
            if isinstance(s, dict):
                return {k: expand(v) for k, v in s.items()}
            if isinstance(s, (list, tuple)):
                return [expand(v) for v in s]
            return s
        return expand(self.parts)

    def leaves(self):
        return flatten(self.structure())

    def sample(self, sample_shape=(), seed=None, generator=None):
        g = generator if generator is not None else _gen(seed)
        return pack_sequence_as(self.structure(), [d.sample(sample_shape, generator=g) for d in self.leaves()])

    def log_prob(self, x):
        terms = [d.log_prob(v) for d, v in zip(self.leaves(), flatten(x))]
        return sum(terms)

    def experimental_default_event_space_bijector(self):
        return JointMap(pack_sequence_as(self.structure(),
                                         [d.experimental_default_event_space_bijector() for d in self.leaves()]))


class JointDistributionNamed(_Joint):
    """A dict of leaf distributions (independent)."""

    def __init__(self, model: dict):
        self.parts = dict(model)


class JointDistributionSequential(_Joint):
    """A list of parts (independent; callables of earlier parts are not supported)."""

    def __init__(self, model: list):
        for m in model:
            if callable(m) and not isinstance(m, Distribution):
                raise NotImplementedError("dependent JointDistributionSequential parts are not supported")
        self.parts = list(model)


def prior_leaves(prior) -> List[Distribution]:
    """Leaf distributions of a prior in flatten order."""
    if isinstance(prior, _Joint):
        return prior.leaves()
    return flatten(prior)
