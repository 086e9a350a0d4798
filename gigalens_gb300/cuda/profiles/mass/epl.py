"""Elliptical power law (``gigalens/tf/profiles/mass/epl.py:9-68``)."""
from .... import profile
from .. import _eval


class EPL(profile.MassProfile):
    """Elliptical power law, iterative series (Tessore & Metcalf 2015).

    ``niter`` caps the series; the number of terms actually summed follows the
    reference's rule over the whole batch of ellipticities.
    """

    _name = "EPL"
    _params = ["theta_E", "gamma", "e1", "e2", "center_x", "center_y"]

    def __init__(self, niter=50):
        super().__init__()
        self.niter = niter

    def deriv(self, x, y, theta_E, gamma, e1, e2, center_x, center_y):
        return _eval.evaluate("EPL", x, y, dict(theta_E=theta_E, gamma=gamma, e1=e1, e2=e2,
                                                center_x=center_x, center_y=center_y), self.niter)
