from . import epl, shear, sie, sis, tnfw  # noqa: F401
