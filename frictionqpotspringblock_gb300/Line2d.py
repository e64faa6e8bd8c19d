"""Line2d systems: a periodic rows x cols grid with 5-point Laplace interactions.

Mirrors the reference's Line2d submodule for System_Cuspy_Laplace
(python/main.cpp:915-960, include/FrictionQPotSpringBlock/Line2d.h:77-116);
particle p = i * cols + j uses pcg32(seed + p) (Line2d.h:28-34).
"""

from . import _capi as C
from ._system import System
from .Line1d import version_compiler, version_dependencies  # noqa: F401


class System_Cuspy_Laplace(System):
    """Cuspy potential + Laplace2d interactions."""

    _potential = C.CUSPY
    _interactions = C.LAPLACE2D
    _rank = 2
    _name = "Line2d.System_Cuspy_Laplace"

    def __init__(self, m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                 offset=-100.0, nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                         offset=offset, nchunk=nchunk, **kwargs)


class System_Cuspy_QuarticGradient(System):
    """Cuspy potential + QuarticGradient2d interactions (main.cpp:963-1005, Line2d.h:122-167,
    detail.h:658-751)."""

    _potential = C.CUSPY
    _interactions = C.QUARTICGRADIENT2D
    _rank = 2
    _name = "Line2d.System_Cuspy_QuarticGradient"

    def __init__(self, m, eta, mu, k2, k4, k_frame, dt, shape, seed, distribution, parameters, offset=-100.0,
                 nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, 0.0, k_frame, dt, shape, seed, distribution, parameters, offset=offset,
                         nchunk=nchunk, interaction_parameters=(k2, k4), **kwargs)
