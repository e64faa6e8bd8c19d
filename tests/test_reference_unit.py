"""The reference's unit tests for Line1d, Particles and Line2d (tests/test_Line1d.py,
tests/test_Particles.py, tests/test_Line2d.py), run against two backends with the reference's class
and member names: the oracle on the CPU, and the GPU classes of frictionqpotspringblock_gb300
(marker `gpu`).  The reference draws its random parameters unseeded; here they come from a seeded
generator.  Checks are the reference's (np.allclose / assertAlmostEqual)."""

import types

import numpy as np
import pytest

from oracle import oracle as O


class _OracleExternal:
    """`system.external` on an oracle system (RandomNormalForcing's state / f_thermal / next)."""

    def __init__(self, s):
        self._s = s

    state = property(lambda e: e._s.thermal_state, lambda e, v: setattr(e._s, "thermal_state", v))
    f_thermal = property(lambda e: e._s.f_thermal, lambda e, v: setattr(e._s, "f_thermal", v))
    next = property(lambda e: e._s.thermal_next, lambda e, v: setattr(e._s, "thermal_next", v))


def _oracle_api():
    def forcing(make):
        def build(mean, stddev, seed_forcing, dinc_init, dinc, **kw):
            s = make(**kw)
            O.attach_random_forcing(s, mean, stddev, seed_forcing, dinc_init, dinc)
            s.external = _OracleExternal(s)
            return s

        return build

    line1d = types.SimpleNamespace(
        System_Cuspy_Laplace=lambda **kw: O.line1d("Cuspy", **kw),
        System_SemiSmooth_Laplace=lambda **kw: O.line1d("SemiSmooth", **kw),
        System_Smooth_Laplace=lambda **kw: O.line1d("Smooth", **kw),
        System_Cuspy_LongRange=O.line1d_longrange,
        System_Cuspy_Laplace_RandomForcing=forcing(lambda **kw: O.line1d("Cuspy", **kw)),
        System_Cuspy_Laplace_Nopassing=O.line1d_nopassing,
        System_Cuspy_Quartic=O.line1d_quartic,
        System_Cuspy_QuarticGradient=O.line1d_quartic_gradient,
    )
    particles = types.SimpleNamespace(
        System_Cuspy=lambda **kw: O.particles("Cuspy", **kw),
        System_SemiSmooth=lambda **kw: O.particles("SemiSmooth", **kw),
        System_Smooth=lambda **kw: O.particles("Smooth", **kw),
        System_Cuspy_RandomForcing=forcing(lambda **kw: O.particles("Cuspy", **kw)),
    )
    line2d = types.SimpleNamespace(System_Cuspy_Laplace=O.line2d)
    return types.SimpleNamespace(Line1d=line1d, Particles=particles, Line2d=line2d)


@pytest.fixture(params=["oracle", pytest.param("gpu", marks=pytest.mark.gpu)])
def FQ(request):
    if request.param == "oracle":
        return _oracle_api()
    return pytest.importorskip("frictionqpotspringblock_gb300")


# the reference's common test system: unit wells centred on 0 (delta distribution, offset -49.5)
UNIT = dict(dt=1.0, shape=[3], seed=0, distribution="delta", parameters=[1.0], offset=-49.5, nchunk=100)


def unit(**kw):
    par = dict(UNIT)
    par.update(kw)
    return par


def _check_at_minimum(system):
    """By construction u = 0 is a local minimum of every potential (test_Line1d.py:74-86)."""
    assert system.residual < 1e-5
    for name in ("f", "f_potential", "f_frame", "f_interactions", "f_damping"):
        assert np.allclose(getattr(system, name), 0.0), name
    assert np.all(system.chunk.index_at_align + 1 == np.argmax(system.chunk.data[0, :] > 0))
    assert np.all(system.chunk.right_of_align > 0)
    assert np.all(system.chunk.left_of_align <= 0)


def test_init_line1d(FQ):
    """test_Line1d.py:25-86: every Line1d class starts at rest in the middle of its wells."""
    rng = np.random.default_rng(1)
    N = 5
    eta, mu, k_interactions, k_frame = (float(x) for x in rng.random(4))
    par = unit(m=1.0, eta=eta, mu=mu, k_interactions=k_interactions, k_frame=k_frame, shape=[N])
    rand = dict(mean=0, stddev=1, seed_forcing=0, dinc_init=np.ones(N, dtype=int), dinc=np.ones(N, dtype=int))
    systems = [
        FQ.Line1d.System_Cuspy_Laplace(**par),
        FQ.Line1d.System_SemiSmooth_Laplace(kappa=1, **par),
        FQ.Line1d.System_Smooth_Laplace(**par),
        FQ.Line1d.System_Cuspy_LongRange(alpha=1, **par),
        FQ.Line1d.System_Cuspy_Laplace_RandomForcing(**par, **rand),
    ]
    nopassing = dict(par)
    nopassing.pop("m")
    systems.append(FQ.Line1d.System_Cuspy_Laplace_Nopassing(**nopassing))
    quartic = dict(par)
    quartic.pop("k_interactions")
    systems.append(FQ.Line1d.System_Cuspy_Quartic(a1=1, a2=1, **quartic))
    systems.append(FQ.Line1d.System_Cuspy_QuarticGradient(k2=1, k4=1, **quartic))
    for system in systems:
        _check_at_minimum(system)


def test_init_particles(FQ):
    """test_Particles.py:25-75."""
    rng = np.random.default_rng(2)
    N = 5
    eta, mu, k_frame = (float(x) for x in rng.random(3))
    par = unit(m=1, eta=eta, mu=mu, k_frame=k_frame, shape=[N])
    rand = dict(mean=0, stddev=1, seed_forcing=0, dinc_init=np.ones(N, dtype=int), dinc=np.ones(N, dtype=int))
    systems = [
        FQ.Particles.System_Cuspy(**par),
        FQ.Particles.System_SemiSmooth(kappa=1, **par),
        FQ.Particles.System_Smooth(**par),
        FQ.Particles.System_Cuspy_RandomForcing(**par, **rand),
    ]
    for system in systems:
        _check_at_minimum(system)


@pytest.mark.parametrize("module", ["Line1d", "Particles"])
def test_forces(FQ, module):
    """test_Line1d.py:89-176 and test_Particles.py:78-153: each force component after moving one
    particle and giving one a velocity, twice (the second time across a well boundary)."""
    rng = np.random.default_rng(3)
    N = 5
    eta, mu, k_interactions, k_frame = (float(x) for x in rng.random(4))
    par = unit(m=1.0, eta=eta, mu=mu, k_frame=k_frame, shape=[N])
    if module == "Line1d":
        system = FQ.Line1d.System_Cuspy_Laplace(k_interactions=k_interactions, **par)
    else:
        k_interactions = 0.0
        system = FQ.Particles.System_Cuspy(**par)
    _check_at_minimum(system)

    def check(f_potential, f_interactions, f_frame, f_damping):
        assert np.all(system.chunk.right_of_align > system.u)
        assert np.all(system.chunk.left_of_align <= system.u)
        assert np.allclose(system.f_potential, f_potential)
        assert np.allclose(system.f_frame, f_frame)
        assert np.allclose(system.f_interactions, f_interactions)
        assert np.allclose(system.f_damping, f_damping)
        assert np.allclose(system.f, f_potential + f_frame + f_interactions + f_damping)

    du, dv = np.zeros(N), np.zeros(N)
    du[0], dv[2] = rng.random(2)
    system.u += du
    system.v += dv
    umin = np.floor(du[0] + 0.5)
    check(mu * np.array([umin - du[0], 0, 0, 0, 0]),
          k_interactions * np.array([-2 * du[0], du[0], 0, 0, du[0]]),
          k_frame * np.array([-du[0], 0, 0, 0, 0]),
          eta * np.array([0, 0, -dv[2], 0, 0]))

    du, dv = np.zeros(N), np.zeros(N)
    du[1], dv[3] = 2.0 * rng.random(2)
    system.u += du
    system.v += dv
    u, v = system.u, system.v
    lap = np.roll(u, 1) - 2 * u + np.roll(u, -1)
    lap[3] = 0.0
    check(mu * np.array([np.floor(u[0] + 0.5) - u[0], np.floor(u[1] + 0.5) - u[1], 0, 0, 0]),
          k_interactions * lap,
          k_frame * np.array([-u[0], -u[1], 0, 0, 0]),
          eta * np.array([0, 0, -v[2], -v[3], 0]))


EVENT_SYSTEMS = {
    "Line1d": lambda FQ: FQ.Line1d.System_Cuspy_Laplace(**unit(m=1.0, eta=1.0, mu=1.0, k_interactions=1.0,
                                                                 k_frame=0.1)),
    "Particles": lambda FQ: FQ.Particles.System_Cuspy(**unit(m=1.0, eta=1.0, mu=1.0, k_frame=0.1)),
    "LongRange": lambda FQ: FQ.Line1d.System_Cuspy_LongRange(**unit(m=1.0, eta=1.0, mu=1.0, k_interactions=1.0,
                                                                      k_frame=0.1, alpha=1)),
}


@pytest.mark.parametrize("which", list(EVENT_SYSTEMS))
def test_event_driven_step(FQ, which):
    """test_Line1d.py:178-219, test_Particles.py:155-195, test_Line1d.py:520-563: alternate
    eventDrivenStep(0.2, kick=False / True) walks all particles to just before / just after the well
    edges at 0.5 and 1.5; the frame follows with u_frame = u (1 + k_frame) / k_frame."""
    system = EVENT_SYSTEMS[which](FQ)
    N = 3
    assert system.residual < 1e-5
    walk = ((0.5 - 0.1, False), (0.5 + 0.1, True), (1.5 - 0.1, False), (1.5 + 0.1, True))
    for k, (target, kick) in enumerate(walk):
        i_n = system.chunk.index_at_align
        system.eventDrivenStep(0.2, kick)
        if k == 0:
            assert system.residual < 1e-5
        assert np.allclose(system.u, target * np.ones(N))
        assert np.all(system.chunk.index_at_align == i_n) == (not kick)
        assert system.u_frame == pytest.approx(target * (1.0 + 0.1) / 0.1, abs=1e-7)


@pytest.mark.parametrize("module", ["Line1d", "Particles"])
def test_trigger(FQ, module):
    """test_Line1d.py:221-248 and test_Particles.py:197-223: trigger moves particle 0 just past its
    well edge; minimise_truncate stops after the first plastic event."""
    if module == "Line1d":
        system = FQ.Line1d.System_Cuspy_Laplace(**unit(m=1.0, eta=1.0, mu=1.0, k_interactions=1.0, k_frame=0.1))
    else:
        system = FQ.Particles.System_Cuspy(**unit(m=1.0, eta=1.0, mu=1.0, k_frame=0.1))
    N = 3
    i_n = system.chunk.index_at_align.copy()
    system.trigger(0, 0.2)
    u = np.zeros(N)
    u[0] = 0.5 + 0.1
    assert np.allclose(system.u, u)
    ret = system.minimise_truncate(i_n=i_n, A_truncate=1)
    assert np.sum(system.chunk.index_at_align != i_n) >= 1
    assert ret > 0
    assert system.residual > 1e-5


@pytest.mark.parametrize("module", ["Line1d", "Particles"])
def test_advance_to_fixed_force(FQ, module):
    """test_Line1d.py:250-275 and test_Particles.py:225-249."""
    if module == "Line1d":
        system = FQ.Line1d.System_Cuspy_Laplace(**unit(m=1.0, eta=1.0, mu=1.0, k_interactions=1.0, k_frame=0.1))
    else:
        system = FQ.Particles.System_Cuspy(**unit(m=1.0, eta=1.0, mu=1.0, k_frame=0.1))
    assert system.residual < 1e-5
    system.advanceToFixedForce(0.1)
    assert np.mean(system.f_frame) == pytest.approx(0.1, abs=1e-7)
    assert system.residual < 1e-5
    system.advanceToFixedForce(0.0)
    assert np.mean(system.f_frame) == pytest.approx(0.0, abs=1e-7)
    assert np.allclose(system.u, 0.0)
    assert np.allclose(system.u_frame, 0.0)


@pytest.mark.parametrize("module", ["Line1d", "Particles"])
def test_semismooth_event_driven_step(FQ, module):
    """test_Line1d.py:344-399 and test_Particles.py:317-372: the SemiSmooth potential's event-driven
    steps end just inside / outside the parabola's junction points (mu xi + kappa y) / (mu + kappa), in
    both directions."""
    mu, kappa, eps = 1, 0.1, 0.001
    if module == "Line1d":
        system = FQ.Line1d.System_SemiSmooth_Laplace(**unit(m=1.0, eta=1.0, mu=mu, kappa=kappa, k_interactions=1.0,
                                                            k_frame=0.1))
    else:
        system = FQ.Particles.System_SemiSmooth(**unit(m=1.0, eta=1.0, mu=mu, kappa=kappa, k_frame=0.1))
    assert system.residual < 1e-5
    u0 = system.u.copy()
    uf0 = system.u_frame
    left = system.chunk.left_of_align
    right = system.chunk.right_of_align
    mid = 0.5 * (left + right)
    upper = (mu * mid + kappa * right) / (mu + kappa)
    lower = (mu * mid + kappa * left) / (mu + kappa)

    assert system.maxUniformDisplacement() == pytest.approx(np.min(upper - system.u), abs=1e-7)
    system.eventDrivenStep(eps=eps, kick=False)
    assert system.residual < 1e-5
    assert np.allclose(system.u, upper - 0.5 * eps)
    assert system.maxUniformDisplacement() == pytest.approx(0.5 * eps, abs=1e-7)
    system.eventDrivenStep(eps=eps, kick=True)
    assert system.residual > 1e-5
    assert np.allclose(system.u, upper + 0.5 * eps)
    assert system.maxUniformDisplacement() == pytest.approx(0, abs=1e-7)

    system.u = u0
    system.u_frame = uf0
    assert system.maxUniformDisplacement(-1) == pytest.approx(np.min(system.u - lower), abs=1e-7)
    system.eventDrivenStep(eps=eps, kick=False, direction=-1)
    assert system.residual < 1e-5
    assert np.allclose(system.u, lower + 0.5 * eps)
    assert system.maxUniformDisplacement(-1) == pytest.approx(0.5 * eps, abs=1e-7)
    system.eventDrivenStep(eps=eps, kick=True, direction=-1)
    assert system.residual > 1e-5
    assert np.allclose(system.u, lower - 0.5 * eps)
    assert system.maxUniformDisplacement() == pytest.approx(0, abs=1e-7)


def test_line2d_interactions(FQ):
    """test_Line2d.py:21-57: the periodic 5-point Laplacian of a unit displacement, rolled over the grid."""
    rows, cols = 5, 4
    k_interactions = float(np.random.default_rng(5).random())
    system = FQ.Line2d.System_Cuspy_Laplace(**unit(m=1, eta=1, mu=1, k_interactions=k_interactions, k_frame=0.1,
                                                   shape=[rows, cols]))
    assert system.residual < 1e-5
    assert list(system.shape) == [rows, cols]
    assert system.size == rows * cols
    f0 = np.array([[-4, 1, 0, 1], [1, 0, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0], [1, 0, 0, 0]]) * k_interactions
    u0 = np.zeros((rows, cols))
    u0[0, 0] = 1.0
    for i in range(rows):
        for j in range(cols):
            x = np.roll(np.roll(u0, i, axis=0), j, axis=1)
            system.u = x
            assert np.allclose(system.f_interactions, np.roll(np.roll(f0, i, axis=0), j, axis=1))
            assert np.allclose(system.u, x)
