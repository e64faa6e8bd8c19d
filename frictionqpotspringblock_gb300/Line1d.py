"""Line1d systems: particles on a periodic ring with nearest-neighbour Laplace interactions.

Mirrors the reference's Line1d submodule (python/main.cpp:480-765,
include/FrictionQPotSpringBlock/Line1d.h:112-421) for the potentials on the
time-integration path: Cuspy, SemiSmooth and Smooth with Laplace1d interactions.
"""

from . import _capi as C
from ._system import System


def version_dependencies():
    """Versions of this implementation and of what it is built on (Line1d.h:34-37)."""
    return [
        "frictionqpotspringblock_gb300=" + C.lib().fqsb_version().decode().split()[1],
        "cuda=13.0",
    ]


def version_compiler():
    return ["nvcc=13.0", "arch=sm_103a"]


class System_Cuspy_Laplace(System):
    """Cuspy potential + Laplace1d interactions (main.cpp:488-529, Line1d.h:112-162)."""

    _potential = C.CUSPY
    _interactions = C.LAPLACE1D
    _rank = 1
    _name = "Line1d.System_Cuspy_Laplace"

    def __init__(self, m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                 offset=-100.0, nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                         offset=offset, nchunk=nchunk, **kwargs)


class System_SemiSmooth_Laplace(System):
    """SemiSmooth potential + Laplace1d interactions (main.cpp:679-722, Line1d.h:336-377)."""

    _potential = C.SEMISMOOTH
    _interactions = C.LAPLACE1D
    _rank = 1
    _name = "Line1d.System_SemiSmooth_Laplace"

    def __init__(self, m, eta, mu, kappa, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                 offset=-100.0, nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                         offset=offset, nchunk=nchunk, kappa=kappa, **kwargs)


class System_Smooth_Laplace(System):
    """Smooth potential + Laplace1d interactions (main.cpp:724-765, Line1d.h:379-422)."""

    _potential = C.SMOOTH
    _interactions = C.LAPLACE1D
    _rank = 1
    _name = "Line1d.System_Smooth_Laplace"

    def __init__(self, m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                 offset=-100.0, nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                         offset=offset, nchunk=nchunk, **kwargs)
