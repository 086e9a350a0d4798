"""Truncated NFW profile (``gigalens/tf/profiles/mass/tnfw.py:10-58``)."""
from .... import profile
from .. import _eval


class TNFW(profile.MassProfile):
    """Truncated NFW deflection with scale radius ``Rs``, deflection at the scale
    radius ``alpha_Rs`` and truncation radius ``r_trunc`` (``R`` clamped to
    ``0.001 Rs`` as in the reference)."""

    _name = "TNFW"
    _params = ["Rs", "alpha_Rs", "r_trunc", "center_x", "center_y"]

    def deriv(self, x, y, Rs, alpha_Rs, r_trunc, center_x, center_y):
        return _eval.evaluate("TNFW", x, y, dict(Rs=Rs, alpha_Rs=alpha_Rs, r_trunc=r_trunc, center_x=center_x,
                                                 center_y=center_y))
