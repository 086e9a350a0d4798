"""Singular isothermal ellipsoid (``gigalens/tf/profiles/mass/sie.py:9-50``)."""
from .... import profile
from .. import _eval


class SIE(profile.MassProfile):
    _name = "SIE"
    s_scale = 1e-4
    _params = ["theta_E", "e1", "e2", "center_x", "center_y"]

    def deriv(self, x, y, theta_E, e1, e2, center_x, center_y):
        return _eval.evaluate("SIE", x, y, dict(theta_E=theta_E, e1=e1, e2=e2, center_x=center_x,
                                                center_y=center_y))
