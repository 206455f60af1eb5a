"""GB300 AVBD rigid-body time-step: Python host side of the C ABI in include/avbdg.h."""

from . import capi, scenes  # noqa: F401
