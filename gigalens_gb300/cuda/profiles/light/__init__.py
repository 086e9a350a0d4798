from . import sersic  # noqa: F401
