"""GB300-native radiation-transfer engine for the Helios radiation plugin.

Product code: libhrt.so (CUDA, sm_103a; sources in csrc/, C ABI in include/hrt.h),
its ctypes binding (_hrt), the host-side mirror of the reference's Context /
RadiationModel API (radiation) and seeded synthetic scenes (scenes).
"""
from . import scenes  # noqa: F401

__all__ = ["scenes", "load"]


def load():
    """Load libhrt.so; raises ImportError if it has not been built."""
    from . import _hrt

    return _hrt.load()
