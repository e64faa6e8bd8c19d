"""RandomNormalForcing on the GPU (Line1d.System_Cuspy_Laplace_RandomForcing,
Line1d.System_Cuspy_Quartic_RandomForcing, Particles.System_Cuspy_RandomForcing): the reference's unit
tests, its golden trajectory, and bit-for-bit parity with the oracle (thermal draws numbered by the
device-side scan over the flat index, the thermal term in every force sum of the step, the external
members state / f_thermal / next)."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

GOLDEN = __import__("pathlib").Path(__file__).parent / "golden"
FIELDS = ["u", "v", "a", "f", "f_potential", "f_interactions", "f_frame", "f_damping"]
EXACT = dict(sum_mode=O.SUM_PAIRWISE, math_mode=O.MATH_PORTABLE)


def make_pair(kind, n, mean=0.0, stddev=0.3, seed_forcing=5, dinc_init=None, dinc=None, **kw):
    rng = np.random.default_rng(n)
    if dinc_init is None:
        dinc_init = rng.integers(0, 12, n)
    if dinc is None:
        dinc = rng.integers(1, 9, n)
    par = dict(m=1.0, eta=kw.get("eta", 0.3), mu=1.0, k_frame=kw.get("k_frame", 1.0 / n), dt=0.1,
               seed=kw.get("seed", 11), distribution="weibull", parameters=[2.0, 1.0, 1e-5],
               offset=kw.get("offset", -20.0), nchunk=kw.get("nchunk", 200))
    th = dict(mean=mean, stddev=stddev, seed_forcing=seed_forcing, dinc_init=dinc_init, dinc=dinc)
    if kind == "Laplace1d":
        gpu = fqsb.Line1d.System_Cuspy_Laplace_RandomForcing(k_interactions=1.0, shape=[n], **par, **th)
        ref = O.line1d("Cuspy", k_interactions=1.0, shape=[n], **par, **EXACT)
    elif kind == "Quartic1d":
        gpu = fqsb.Line1d.System_Cuspy_Quartic_RandomForcing(a1=0.8, a2=0.6, shape=[n], **par, **th)
        ref = O.line1d_quartic(a1=0.8, a2=0.6, shape=[n], **par, **EXACT)
    else:
        gpu = fqsb.Particles.System_Cuspy_RandomForcing(shape=[n], **par, **th)
        ref = O.particles("Cuspy", shape=[n], **par, **EXACT)
    O.attach_random_forcing(ref, **th)
    return gpu, ref


def assert_same(gpu, ref):
    for name in FIELDS:
        g, r = getattr(gpu, name), getattr(ref, name)
        assert np.array_equal(g, r), (name, np.max(np.abs(g - r)))
    assert np.array_equal(gpu.external.f_thermal, ref.f_thermal)
    assert np.array_equal(gpu.external.next, ref.thermal_next)
    assert gpu.external.state == ref.thermal_state
    assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align)
    assert gpu.inc == ref.inc
    assert gpu.u_frame == ref.u_frame
    assert gpu.residual == ref.residual


@pytest.mark.parametrize("cls", ["Line1d", "Particles"])
def test_reference_unit_test(cls):
    """tests/test_Line1d.py:565-600 and tests/test_Particles.py:374-412: with dinc_init = dinc = 1 each
    `inc += 1` redraws every particle's force from the one stream, in particle order."""
    N = 10
    par = dict(m=1, eta=1, mu=1, k_frame=0.1, dt=1, mean=0, stddev=1, seed_forcing=0,
               dinc_init=np.ones(N, dtype=int), dinc=np.ones(N, dtype=int), shape=[N], seed=0,
               distribution="delta", parameters=[1.0], offset=-49.5, nchunk=100)
    if cls == "Line1d":
        system = fqsb.Line1d.System_Cuspy_Laplace_RandomForcing(k_interactions=1, **par)
    else:
        system = fqsb.Particles.System_Cuspy_RandomForcing(**par)
    assert system.residual < 1e-5
    assert np.all(system.external.f_thermal == 0)
    # the stream drawn by hand: pcg32(0) on the default stream, mean + stddev sqrt(2) erfinv(2 r - 1)
    from scipy.special import erfinv

    state, inc = O.pcg32_seed(0)
    r = []
    states = []
    for _ in range(2 * N):
        states.append(state)
        old = state
        state = (old * 0x5851F42D4C957F2D + inc) & ((1 << 64) - 1)
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        r.append((((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF) * 2.0 ** -32)
    expect = np.sqrt(2.0) * erfinv(2 * np.array(r) - 1)
    system.inc += 1
    system.refresh()
    assert system.residual > 1e-5
    assert np.allclose(system.external.f_thermal, expect[:N])
    assert np.array_equal(system.external.next, 2 * np.ones(N))
    assert system.external.state == states[N]
    system.inc += 1
    system.refresh()
    assert np.allclose(system.external.f_thermal, expect[N:])
    assert system.external.state == state
    assert repr(system.external) == "<FrictionQPotSpringBlock.detail.RandomNormalForcing_1>"


def test_athermal_members_absent():
    """The RandomForcing bindings omit mySystemNdAthermal (main.cpp:614-616)."""
    system, _ = make_pair("Laplace1d", 16)
    for name in ("minimise", "minimise_truncate", "eventDrivenStep", "quasistaticActivityFirst"):
        assert not hasattr(system, name)
    assert hasattr(system, "timeStepsUntilEvent") and hasattr(system, "flowSteps")
    assert hasattr(system, "trigger") and hasattr(system, "external")


# 1000 / 5000: one and several tiles of the draw, one particle per thread in the step; 2^18 + 77:
# ragged last tile, two particles per thread (each of the six thermal step kernels is run)
@pytest.mark.parametrize("kind,n", [("Laplace1d", n) for n in (7, 1000, 5000, 2 ** 18 + 77)] +
                         [("Quartic1d", n) for n in (1000, 2 ** 18 + 77)] +
                         [("Particles", n) for n in (1000, 2 ** 18 + 77)])
def test_parity(kind, n):
    big = n > 10000
    dinc = None
    if big:
        # keep the oracle's draws to a few hundred thousand (erfinv is not cheap on the CPU)
        rng = np.random.default_rng(1)
        dinc = rng.integers(20, 60, n)
    gpu, ref = make_pair(kind, n, dinc=dinc)
    assert_same(gpu, ref)
    rng = np.random.default_rng(n + 1)
    u0 = rng.normal(0.0, 0.4, n)
    gpu.u = u0
    ref.u = u0
    assert_same(gpu, ref)
    nsteps = 40 if big else 200
    gpu.timeSteps(nsteps)
    ref.timeSteps(nsteps)
    assert_same(gpu, ref)
    gpu.flowSteps(nsteps, 0.2)
    ref.flowSteps(nsteps, 0.2)
    assert_same(gpu, ref)


def test_every_particle_every_step():
    """dinc = 1 for all: every step draws N values, the stream advances by N per step."""
    gpu, ref = make_pair("Laplace1d", 3000, dinc_init=np.zeros(3000, dtype=int), dinc=np.ones(3000, dtype=int))
    assert_same(gpu, ref)
    for _ in range(3):
        gpu.timeSteps(7)
        ref.timeSteps(7)
        assert_same(gpu, ref)


def test_host_driven_iteration(monkeypatch):
    """The same draws through the kernel-by-kernel form of the run loop (FQSB_NO_GRAPH=1)."""
    monkeypatch.setenv("FQSB_NO_GRAPH", "1")
    gpu, ref = make_pair("Laplace1d", 5000)
    gpu.flowSteps(150, 0.1)
    ref.flowSteps(150, 0.1)
    assert_same(gpu, ref)


def test_time_steps_until_event():
    gpu, ref = make_pair("Laplace1d", 2000, stddev=0.05, dinc=np.full(2000, 5))
    gpu.u_frame = 0.3
    ref.u_frame = 0.3
    assert_same(gpu, ref)
    n_gpu = gpu.timeStepsUntilEvent(max_iter=5000)
    n_ref = ref.timeStepsUntilEvent(max_iter=5000)
    assert n_gpu == n_ref
    assert_same(gpu, ref)


def test_external_setters():
    """set_state / set_next / set_f_thermal (detail.h:956-995): f keeps its value until the next force
    update; the next steps use the new forces, state and increments."""
    gpu, ref = make_pair("Laplace1d", 1500)
    gpu.timeSteps(30)
    ref.timeSteps(30)
    rng = np.random.default_rng(3)
    f_th = rng.normal(0.0, 1.0, 1500)
    nxt = ref.thermal_next + rng.integers(0, 3, 1500)
    for s in (gpu.external,):
        s.f_thermal = f_th
        s.next = nxt
        s.state = 0x9E3779B97F4A7C15
    ref.f_thermal = f_th
    ref.thermal_next = nxt
    ref.thermal_state = 0x9E3779B97F4A7C15
    assert_same(gpu, ref)
    gpu.u_frame = gpu.u_frame + 0.01  # set_u_frame: computeForce with the new f_thermal
    ref.u_frame = ref.u_frame + 0.01
    assert_same(gpu, ref)
    gpu.timeSteps(40)
    ref.timeSteps(40)
    assert_same(gpu, ref)
    with pytest.raises(RuntimeError):
        gpu.external.f_thermal = np.zeros(3)


def test_set_inc_and_refresh_draw():
    """set_inc and refresh call updated_inc (detail.h:1241-1247, 1310-1315)."""
    gpu, ref = make_pair("Laplace1d", 800)
    for inc in (3, 3, 20, 21):
        gpu.inc = inc
        ref.inc = inc
        assert_same(gpu, ref)
        gpu.refresh()
        ref.refresh()
        assert_same(gpu, ref)
    gpu.timeSteps(25)
    ref.timeSteps(25)
    assert_same(gpu, ref)


def test_trigger_then_draw():
    """After trigger the forces are not updated (detail.h:1972-1977); a draw at set_inc recomputes f
    from them and the new thermal forces."""
    gpu, ref = make_pair("Laplace1d", 600, dinc_init=np.ones(600, dtype=int), dinc=np.ones(600, dtype=int))
    gpu.trigger(17, 0.1)
    ref.trigger(17, 0.1)
    assert_same(gpu, ref)
    gpu.inc = gpu.inc + 1
    ref.inc = ref.inc + 1
    assert_same(gpu, ref)
    gpu.timeSteps(10)
    ref.timeSteps(10)
    assert_same(gpu, ref)


def test_golden_prefix():
    """examples/Line1d_System_Cuspy_Laplace_RandomForcing.py + .h5 (outputs of flowSteps(1000) at finite
    temperature), the first outputs, as np.isclose like the reference's example."""
    golden = np.load(GOLDEN / "Line1d_System_Cuspy_Laplace_RandomForcing.npz")
    N = 1000
    common = dict(m=1.0, eta=2.0 * np.sqrt(3.0) / 10.0, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1,
                  shape=[N], seed=0, distribution="random", parameters=[2.0], offset=-50)
    athermal = fqsb.Line1d.System_Cuspy_Laplace(**common)
    athermal.minimise()
    system = fqsb.Line1d.System_Cuspy_Laplace_RandomForcing(mean=0.0, stddev=0.05, seed_forcing=0,
                                                            dinc_init=O.pcg32_randint(0, N, 100),
                                                            dinc=100 * np.ones(N, dtype=np.int64), **common)
    system.u = athermal.u
    for k in range(20):
        system.flowSteps(1000, 5e-2)
        assert np.isclose(system.u_frame, golden["frame"][k]), k
        assert np.isclose(np.mean(system.f_frame), golden["f_frame"][k]), k
        assert np.isclose(system.temperature, golden["t_insta"][k]), k


def test_unsupported():
    """RandomNormalForcing is built for the reference's three RandomForcing classes (Cuspy with Laplace1d,
    Quartic1d or no interactions): other systems refuse it; a second attach is refused."""
    import ctypes

    from frictionqpotspringblock_gb300 import _capi as C

    s = fqsb.Line1d.System_SemiSmooth_Laplace(m=1, eta=1, mu=1, kappa=1, k_interactions=1, k_frame=0.1, dt=0.1,
                                              shape=[64], seed=0, distribution="delta", parameters=[1.0],
                                              offset=-49.5, nchunk=100)
    di = np.ones(64, dtype=np.int64)
    p = di.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    assert C.lib().fqsb_set_random_forcing(s._h, 0.0, 1.0, 0, p, p) == C.ERR_UNSUPPORTED
    gpu, _ = make_pair("Laplace1d", 64)
    assert C.lib().fqsb_set_random_forcing(gpu._h, 0.0, 1.0, 0, p, p) == C.ERR_INVALID
    # the adjoint refuses thermal systems
    sched = np.zeros(4)
    loss = ctypes.c_double()
    assert C.lib().fqsb_adjoint_forward(gpu._h, sched.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 4, 2, 1,
                                        ctypes.byref(loss)) == C.ERR_UNSUPPORTED
