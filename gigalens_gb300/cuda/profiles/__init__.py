from . import light, mass  # noqa: F401
