"""GB300-native batched MIRK boundary-value solver (host side)."""
from . import problems  # noqa: F401
