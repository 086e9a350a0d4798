"""Keras-compatible optimizer objects for the modelling sequence.

The reference drives MAP and SVI with ``tf.keras.optimizers.Adam`` and
``tf.keras.optimizers.schedules.PolynomialDecay`` (``tf-demo.ipynb`` cells
12 and 14, ``tf/inference.py:34``).  These classes keep those constructor
signatures; MAP applies the update with the fused ``gl_adam_step`` kernel
(device-side step counter and schedule, so it can replay from a CUDA graph).
"""
import math

import torch

from .. import _native as N


class PolynomialDecay:
    """``lr(s) = (lr0 - end) (1 - min(s, decay_steps)/decay_steps)^power + end``."""

    def __init__(self, initial_learning_rate, decay_steps, end_learning_rate=0.0001, power=1.0, cycle=False):
        if cycle:
            raise NotImplementedError("cycle=True is not supported")
        self.initial_learning_rate = float(initial_learning_rate)
        self.decay_steps = float(decay_steps)
        self.end_learning_rate = float(end_learning_rate)
        self.power = float(power)

    def __call__(self, step):
        s = min(float(step), self.decay_steps)
        return (self.initial_learning_rate - self.end_learning_rate) * (1 - s / self.decay_steps) ** self.power \
            + self.end_learning_rate


class schedules:  # noqa: N801  (mirrors tf.keras.optimizers.schedules)
    PolynomialDecay = PolynomialDecay


class Adam:
    """Adam with Keras defaults (``epsilon=1e-7``) and Keras' update form."""

    def __init__(self, learning_rate=0.001, beta_1=0.9, beta_2=0.999, epsilon=1e-7):
        self.learning_rate = learning_rate
        self.beta_1 = float(beta_1)
        self.beta_2 = float(beta_2)
        self.epsilon = float(epsilon)

    def cfg(self):
        c = N.gl_adam_cfg()
        lr = self.learning_rate
        if isinstance(lr, PolynomialDecay):
            c.schedule = N.GL_LR_POLYNOMIAL
            c.lr0, c.lr_end, c.decay_steps, c.power = (lr.initial_learning_rate, lr.end_learning_rate,
                                                       lr.decay_steps, lr.power)
        elif callable(lr):
            raise NotImplementedError("learning-rate callables other than PolynomialDecay are not supported")
        else:
            c.schedule = N.GL_LR_CONSTANT
            c.lr0 = float(lr)
        c.beta1, c.beta2, c.eps = self.beta_1, self.beta_2, self.epsilon
        return c

    def lr_at(self, step):
        lr = self.learning_rate
        return lr(step) if callable(lr) else float(lr)


class AdamState:
    """Moments and the device step counter for one variable."""

    def __init__(self, var: torch.Tensor, opt: Adam):
        self.var = var
        self.m = torch.zeros_like(var)
        self.v = torch.zeros_like(var)
        self.step = torch.zeros(1, dtype=torch.int32, device=var.device)
        self.opt = opt
        self._cfg = opt.cfg()

    def apply(self, grad: torch.Tensor, grad_scale: float = 1.0, stream=None):
        N.call("gl_adam_step", N.ptr(self.var), N.ptr(self.m), N.ptr(self.v), N.ptr(grad), self.var.numel(),
               float(grad_scale), self._cfg, N.ptr(self.step), N.stream_ptr(stream))
