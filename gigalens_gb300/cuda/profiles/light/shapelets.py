"""Shapelet light profile (``gigalens/tf/profiles/light/shapelets.py:11-85``).

``interpolate=False`` evaluates the basis functions exactly from the Hermite
recursion.  ``interpolate=True`` (the reference's default) reproduces the
reference's tables: the 1-D functions phi_n(t) exp(-t^2/2) sampled at 6000
points on [-5, 5] (float32), linearly interpolated as
``tfp.math.interp_regular_1d_grid`` and 0 outside [-5, 5].  The two modes
agree inside [-5, 5] to the reference's own test tolerance
(``tests/test_profiles.py:35-47``, rtol 1e-5 / atol 1e-4); outside it the
tabulated basis is cut to zero, which for n >= 3 drops values of up to 0.06 %
(n = 3) to 8 % (n = 8) of the function's peak.
"""
import torch

from .... import _native as N
from .... import profile
from .. import _eval


class Shapelets(profile.LightProfile):
    _name = "SHAPELETS"
    _params = ["beta", "center_x", "center_y"]

    def __init__(self, n_max, use_lstsq=False, interpolate=True):
        super().__init__(use_lstsq=False)
        self._use_lstsq = use_lstsq
        self.n_max = int(n_max)
        self.n_layers = (self.n_max + 1) * (self.n_max + 2) // 2
        self.interpolate = interpolate
        width = len(str(self.n_layers))
        self._amp_names = ["amp" + str(i).zfill(width) for i in range(self.n_layers)]
        self.params = list(self._params) + list(self._amp_names)
        self.N1, self.N2 = [], []
        n1 = n2 = 0
        for _ in range(self.n_layers):
            self.N1.append(n1)
            self.N2.append(n2)
            if n1 == 0:
                n1, n2 = n2 + 1, 0
            else:
                n1, n2 = n1 - 1, n2 + 1
        self.depth = self.n_layers

    @property
    def niter(self):
        return self.n_max

    def light(self, x, y, center_x, center_y, beta, **amp):
        dev = _eval._dev()
        tensors = [_eval.as_cuda(x, dev), _eval.as_cuda(y, dev), _eval.as_cuda(beta, dev),
                   _eval.as_cuda(center_x, dev), _eval.as_cuda(center_y, dev)]
        amps = None
        if not self.use_lstsq:
            amps = [_eval.as_cuda(amp[k], dev) for k in self._amp_names]
            tensors += amps
        shape = torch.broadcast_shapes(*[t.shape for t in tensors])
        flat = [t.expand(shape).reshape(-1) for t in tensors]
        n = flat[0].numel()
        xs, ys = flat[0].contiguous(), flat[1].contiguous()
        prm = torch.stack(flat[2:5], 0).contiguous()
        if self.use_lstsq:
            out = torch.empty((self.n_layers, n), dtype=torch.float32, device=dev)
            a = None
        else:
            a = torch.stack(flat[5:], 0).contiguous()
            out = torch.empty(n, dtype=torch.float32, device=dev)
        N.call("gl_shapelets_eval", self.n_max, int(bool(self.interpolate)), N.ptr(xs), N.ptr(ys), n, N.ptr(prm),
               N.ptr(a), N.ptr(out), N.stream_ptr())
        if self.use_lstsq:
            return out.reshape(self.n_layers, *shape)
        return out.reshape(shape)
