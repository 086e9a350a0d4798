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
