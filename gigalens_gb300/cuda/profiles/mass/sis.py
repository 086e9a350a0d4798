"""Singular isothermal sphere (``gigalens/tf/profiles/mass/sis.py:9-18``)."""
from .... import profile
from .. import _eval


class SIS(profile.MassProfile):
    _name = "SIS"
    _params = ["theta_E", "center_x", "center_y"]

    def deriv(self, x, y, theta_E, center_x, center_y):
        return _eval.evaluate("SIS", x, y, dict(theta_E=theta_E, center_x=center_x, center_y=center_y))
