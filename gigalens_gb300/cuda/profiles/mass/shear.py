"""External shear (``gigalens/tf/profiles/mass/shear.py:6-14``)."""
from .... import profile
from .. import _eval


class Shear(profile.MassProfile):
    _name = "SHEAR"
    _params = ["gamma1", "gamma2"]

    def deriv(self, x, y, gamma1, gamma2):
        return _eval.evaluate("SHEAR", x, y, dict(gamma1=gamma1, gamma2=gamma2))
