"""Line1d systems: particles on a periodic ring with nearest-neighbour Laplace interactions.

Mirrors the reference's Line1d submodule (python/main.cpp:480-765,
include/FrictionQPotSpringBlock/Line1d.h:112-421) for the potentials on the
time-integration path: Cuspy, SemiSmooth and Smooth with Laplace1d interactions.
"""

from . import _capi as C
from ._system import System, _Hidden


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


class System_Cuspy_Quartic(System):
    """Cuspy potential + Quartic1d interactions (main.cpp:768-810, Line1d.h:428-481, detail.h:757-805)."""

    _potential = C.CUSPY
    _interactions = C.QUARTIC1D
    _rank = 1
    _name = "Line1d.System_Cuspy_Quartic"

    def __init__(self, m, eta, mu, a1, a2, k_frame, dt, shape, seed, distribution, parameters, offset=-100.0,
                 nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, 0.0, k_frame, dt, shape, seed, distribution, parameters, offset=offset,
                         nchunk=nchunk, interaction_parameters=(a1, a2), **kwargs)


class System_Cuspy_QuarticGradient(System):
    """Cuspy potential + QuarticGradient1d interactions (main.cpp:813-855, Line1d.h:562-615,
    detail.h:616-653)."""

    _potential = C.CUSPY
    _interactions = C.QUARTICGRADIENT1D
    _rank = 1
    _name = "Line1d.System_Cuspy_QuarticGradient"

    def __init__(self, m, eta, mu, k2, k4, k_frame, dt, shape, seed, distribution, parameters, offset=-100.0,
                 nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, 0.0, k_frame, dt, shape, seed, distribution, parameters, offset=offset,
                         nchunk=nchunk, interaction_parameters=(k2, k4), **kwargs)


class System_Cuspy_LongRange(System):
    """Cuspy potential + LongRange1d interactions, all pairs decaying as 1 / d^(1 + alpha)
    (main.cpp:857-897, Line1d.h:617-675, detail.h:812-868)."""

    _potential = C.CUSPY
    _interactions = C.LONGRANGE1D
    _rank = 1
    _name = "Line1d.System_Cuspy_LongRange"

    def __init__(self, m, eta, mu, k_interactions, alpha, k_frame, dt, shape, seed, distribution, parameters,
                 offset=-100.0, nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                         offset=offset, nchunk=nchunk, interaction_parameters=(alpha, 0.0), **kwargs)


class System_Cuspy_Laplace_Nopassing(System):
    """Cuspy + Laplace1d minimised with the no-passing rule, no dynamics (main.cpp:532-568, Line1d.h:173-238).

    m = 1; minimise() runs the overdamped no-passing fixed point (detail.h:1694-1753); the time-stepping
    members are absent as in the reference (its binding omits mySystemNdDynamics)."""

    _potential = C.CUSPY
    _interactions = C.LAPLACE1D
    _rank = 1
    _name = "Line1d.System_Cuspy_Laplace_Nopassing"

    timeStep = _Hidden()
    timeSteps = _Hidden()
    timeStepsUntilEvent = _Hidden()
    flowSteps = _Hidden()

    def __init__(self, mu, k_interactions, k_frame, shape, seed, distribution, parameters, offset=-100.0,
                 nchunk=5000, eta=0.0, dt=0.0, **kwargs):
        super().__init__(1.0, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                         offset=offset, nchunk=nchunk, **kwargs)

    def minimise(self, tol=1e-5, niter_tol=10, max_iter=int(1e9), time_activity=False, max_iter_is_error=True) -> int:
        if time_activity:
            raise RuntimeError("assertion failed (!time_activity)")
        out = C.ctypes.c_uint64()
        C.check(self._h, C.lib().fqsb_minimise_nopassing(self._h, float(tol), int(niter_tol), int(max_iter),
                                                          int(bool(max_iter_is_error)), C.ctypes.byref(out)))
        return out.value


class _RandomForcing:
    """Members of the RandomForcing systems: `external` (mySystemNdExternal, main.cpp:205-208); the
    athermal members are absent as in the reference (its bindings omit mySystemNdAthermal)."""

    external = property(lambda s: s._external, doc="Class adding external force")
    minimise = _Hidden()
    minimise_truncate = _Hidden()
    eventDrivenStep = _Hidden()
    quasistaticActivityFirst = _Hidden()
    quasistaticActivityLast = _Hidden()


class System_Cuspy_Laplace_RandomForcing(_RandomForcing, System):
    """Cuspy + Laplace1d with a random normal force per particle, redrawn every `dinc` increments (first
    at `dinc_init`) from one pcg32 stream (main.cpp:570-621, Line1d.h:264-330, detail.h:881-1000)."""

    _potential = C.CUSPY
    _interactions = C.LAPLACE1D
    _rank = 1
    _name = "Line1d.System_Cuspy_Laplace_RandomForcing"

    def __init__(self, m, eta, mu, k_interactions, k_frame, dt, mean, stddev, seed_forcing, dinc_init, dinc, shape,
                 seed, distribution, parameters, offset=-100.0, nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                         offset=offset, nchunk=nchunk, **kwargs)
        self._attach_random_forcing(mean, stddev, seed_forcing, dinc_init, dinc)


class System_Cuspy_Quartic_RandomForcing(_RandomForcing, System):
    """Cuspy + Quartic1d with a random normal force per particle (main.cpp:623-676, Line1d.h:486-556)."""

    _potential = C.CUSPY
    _interactions = C.QUARTIC1D
    _rank = 1
    _name = "Line1d.System_Cuspy_Quartic_RandomForcing"

    def __init__(self, m, eta, mu, a1, a2, k_frame, dt, mean, stddev, seed_forcing, dinc_init, dinc, shape, seed,
                 distribution, parameters, offset=-100.0, nchunk=5000, **kwargs):
        super().__init__(m, eta, mu, 0.0, k_frame, dt, shape, seed, distribution, parameters, offset=offset,
                         nchunk=nchunk, interaction_parameters=(a1, a2), **kwargs)
        self._attach_random_forcing(mean, stddev, seed_forcing, dinc_init, dinc)
