"""exptool_gb300: GB300-native (sm_103a) basis-function-expansion dynamics.

Drop-in GPU implementations of exptool's spherical Sturm-Liouville and
cylindrical EOF coefficient accumulation, potential/force evaluation and
leapfrog orbit integration (``exptool_gb300.basis.spheresl``,
``exptool_gb300.basis.eof``, ``exptool_gb300.basis.potential``,
``exptool_gb300.utils.integrate``, ``exptool_gb300.orbits.orbit``), backed by
the CUDA library ``lib/libexptool_gb300.so`` (C ABI: include/exptool_gb300.h).
"""
__version__ = "0.1.0"


def library():
    """Load (building if needed) the CUDA library; returns the ctypes handle."""
    from . import _lib
    return _lib.load()
