"""GB300-native time-integration path of FrictionQPotSpringBlock.

Drop-in for the reference's Python module on the time-integration path:

    import frictionqpotspringblock_gb300 as FrictionQPotSpringBlock
    system = FrictionQPotSpringBlock.Line1d.System_Cuspy_Laplace(...)

Every call goes through the C ABI of libfqsb.so (include/fqsb.h) to FP64
kernels for sm_103a; there is no CPU fallback.
"""

from . import Line1d, Line2d, Particles, detail  # noqa: F401
from ._capi import FrictionError  # noqa: F401

__version__ = "0.1.0"


def version():
    return __version__
