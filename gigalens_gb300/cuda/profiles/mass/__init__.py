from . import epl, shear, sie, sis  # noqa: F401
