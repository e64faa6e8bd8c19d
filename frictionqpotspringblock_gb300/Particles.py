"""Particles systems: independent particles (no interactions).

Mirrors the reference's Particles submodule for System_Cuspy, System_SemiSmooth
and System_Smooth (python/main.cpp:290-470, include/FrictionQPotSpringBlock/Particles.h:93-311).
They run through the same fused step as Line1d with the interaction term off.
"""

from . import _capi as C
from ._system import System
from .Line1d import _RandomForcing, version_compiler, version_dependencies  # noqa: F401


class System_Cuspy(System):
    _potential = C.CUSPY
    _interactions = C.INTERACTIONS_NONE
    _rank = 1
    _name = "Particles.System_Cuspy"

    def __init__(self, m, eta, mu, k_frame, dt, shape, seed, distribution, parameters, offset=-100.0, nchunk=5000,
                 **kwargs):
        super().__init__(m, eta, mu, 0.0, k_frame, dt, shape, seed, distribution, parameters, offset=offset,
                         nchunk=nchunk, **kwargs)


class System_SemiSmooth(System):
    _potential = C.SEMISMOOTH
    _interactions = C.INTERACTIONS_NONE
    _rank = 1
    _name = "Particles.System_SemiSmooth"

    def __init__(self, m, eta, mu, kappa, k_frame, dt, shape, seed, distribution, parameters, offset=-100.0,
                 nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, 0.0, k_frame, dt, shape, seed, distribution, parameters, offset=offset,
                         nchunk=nchunk, kappa=kappa, **kwargs)


class System_Smooth(System):
    _potential = C.SMOOTH
    _interactions = C.INTERACTIONS_NONE
    _rank = 1
    _name = "Particles.System_Smooth"

    def __init__(self, m, eta, mu, k_frame, dt, shape, seed, distribution, parameters, offset=-100.0, nchunk=5000,
                 **kwargs):
        super().__init__(m, eta, mu, 0.0, k_frame, dt, shape, seed, distribution, parameters, offset=offset,
                         nchunk=nchunk, **kwargs)


class System_Cuspy_RandomForcing(_RandomForcing, System):
    """Independent Cuspy particles with a random normal force each (main.cpp:335-384, Particles.h:161-227)."""

    _potential = C.CUSPY
    _interactions = C.INTERACTIONS_NONE
    _rank = 1
    _name = "Particles.System_Cuspy_RandomForcing"

    def __init__(self, m, eta, mu, k_frame, dt, mean, stddev, seed_forcing, dinc_init, dinc, shape, seed,
                 distribution, parameters, offset=-100.0, nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, 0.0, k_frame, dt, shape, seed, distribution, parameters, offset=offset,
                         nchunk=nchunk, **kwargs)
        self._attach_random_forcing(mean, stddev, seed_forcing, dinc_init, dinc)
