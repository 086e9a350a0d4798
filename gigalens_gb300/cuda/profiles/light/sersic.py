"""Sersic light profiles (``gigalens/tf/profiles/light/sersic.py:9-72``)."""
import torch

from .... import profile
from .. import _eval


class Sersic(profile.LightProfile):
    """Spherical Sersic: ``Ie exp(-b_n ((R/R_sersic)^(1/n) - 1))``, b_n = 1.9992 n - 0.3271."""

    _name = "SERSIC"
    _params = ["R_sersic", "n_sersic", "center_x", "center_y"]

    def light(self, x, y, R_sersic, n_sersic, center_x, center_y, Ie=None):
        Ie = torch.ones_like(torch.as_tensor(R_sersic, dtype=torch.float32)) if self.use_lstsq else Ie
        out = _eval.evaluate("SERSIC", x, y, dict(R_sersic=R_sersic, n_sersic=n_sersic, center_x=center_x,
                                                  center_y=center_y, Ie=Ie))
        return out[None] if self.use_lstsq else out


class SersicEllipse(Sersic):
    """Elliptical Sersic with complex ellipticity (e1, e2)."""

    _name = "SERSIC_ELLIPSE"
    _params = ["R_sersic", "n_sersic", "e1", "e2", "center_x", "center_y"]

    def light(self, x, y, R_sersic, n_sersic, e1, e2, center_x, center_y, Ie=None):
        Ie = torch.ones_like(torch.as_tensor(R_sersic, dtype=torch.float32)) if self.use_lstsq else Ie
        out = _eval.evaluate("SERSIC_ELLIPSE", x, y, dict(R_sersic=R_sersic, n_sersic=n_sersic, e1=e1, e2=e2,
                                                          center_x=center_x, center_y=center_y, Ie=Ie))
        return out[None] if self.use_lstsq else out


class CoreSersic(Sersic):
    """Core-Sersic light (``tf/profiles/light/sersic.py:75-121``) with the
    reference's expression kept as written:
    ``Ie (1 + (Rb/R)^alpha)^(gamma/alpha) exp(-bn (R^alpha + Rb^alpha) / R_sersic^alpha / (alpha n) - 1)``
    (the reference's ``R_sersic ** alpha ** 1.0`` is ``R_sersic ** alpha``)."""

    _name = "CORE_SERSIC"
    _params = ["R_sersic", "n_sersic", "Rb", "alpha", "gamma", "e1", "e2", "center_x", "center_y"]

    def light(self, x, y, R_sersic, n_sersic, Rb, alpha, gamma, e1, e2, center_x, center_y, Ie=None):
        Ie = torch.ones_like(torch.as_tensor(R_sersic, dtype=torch.float32)) if self.use_lstsq else Ie
        out = _eval.evaluate("CORE_SERSIC", x, y, dict(R_sersic=R_sersic, n_sersic=n_sersic, Rb=Rb, alpha=alpha,
                                                       gamma=gamma, e1=e1, e2=e2, center_x=center_x,
                                                       center_y=center_y, Ie=Ie))
        return out[None] if self.use_lstsq else out
