"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

The oracle runs with the device's reduction order (pairwise tree over the flat
particle index) and the device's deterministic elementary functions, so the
comparison is bit for bit: u, v, a, all forces, well indices, yield positions,
chunk windows, increments and returned values must be identical.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

KINDS = {
    "Line1d_Cuspy": (lambda **p: fqsb.Line1d.System_Cuspy_Laplace(**p), lambda **p: O.line1d("Cuspy", **p), 1),
    "Line1d_SemiSmooth": (lambda **p: fqsb.Line1d.System_SemiSmooth_Laplace(kappa=0.5, **p),
                          lambda **p: O.line1d("SemiSmooth", kappa=0.5, **p), 1),
    "Line1d_Smooth": (lambda **p: fqsb.Line1d.System_Smooth_Laplace(**p), lambda **p: O.line1d("Smooth", **p), 1),
    "Line2d_Cuspy": (lambda **p: fqsb.Line2d.System_Cuspy_Laplace(**p), lambda **p: O.line2d(**p), 2),
    "Particles_Cuspy": (lambda **p: fqsb.Particles.System_Cuspy(**{k: v for k, v in p.items() if k != "k_interactions"}),
                        lambda **p: O.particles("Cuspy", **{k: v for k, v in p.items() if k != "k_interactions"}), 1),
}


def make_pair(kind, shape, distribution="weibull", parameters=(2.0, 1.0, 1e-5), offset=-20.0, nchunk=200, **kw):
    gpu_f, ref_f, rank = KINDS[kind]
    if rank == 2 and len(shape) == 1:
        shape = [shape[0] // 8, 8]
    par = dict(m=kw.get("m", 1.0), eta=kw.get("eta", 0.1), mu=kw.get("mu", 1.0),
               k_interactions=kw.get("k_interactions", 1.0), k_frame=kw.get("k_frame", 1.0 / np.prod(shape)),
               dt=kw.get("dt", 0.1), shape=list(shape), seed=kw.get("seed", 3), distribution=distribution,
               parameters=list(parameters), offset=offset, nchunk=nchunk)
    gpu = gpu_f(**par)
    ref = ref_f(**par, sum_mode=O.SUM_PAIRWISE, math_mode=O.MATH_PORTABLE)
    return gpu, ref


FIELDS = ["u", "v", "a", "f", "f_potential", "f_interactions", "f_frame", "f_damping"]


def assert_same(gpu, ref, chunk=True):
    for name in FIELDS:
        g, r = getattr(gpu, name), getattr(ref, name)
        assert np.array_equal(g, r), (name, np.max(np.abs(g - r)))
    assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align)
    assert np.array_equal(gpu.chunk.chunk_index_at_align, ref.chunk.chunk_index_at_align)
    assert np.array_equal(gpu.chunk.left_of_align, ref.chunk.left_of_align)
    assert np.array_equal(gpu.chunk.right_of_align, ref.chunk.right_of_align)
    assert gpu.inc == ref.inc
    assert gpu.u_frame == ref.u_frame
    assert gpu.residual == ref.residual
    assert gpu.temperature == ref.temperature
    if chunk:
        assert np.array_equal(gpu.chunk.start, ref.chunk.start)
        assert np.array_equal(gpu.chunk.data, ref.chunk.data)


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("distribution,parameters", [("weibull", (2.0, 1.0, 1e-5)), ("random", (2.0,)),
                                                      ("delta", (1.0,)), ("exponential", (1.0, 0.01)),
                                                      ("weibull", (1.5, 0.8, 1e-3))])
def test_construction(kind, distribution, parameters):
    gpu, ref = make_pair(kind, [200], distribution, parameters, offset=-30.0)
    assert_same(gpu, ref)


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("n", [1, 7, 96, 1000, 5000])
def test_time_steps(kind, n):
    if kind.startswith("Line2d") and n < 16:
        pytest.skip("grid needs 8 columns")
    gpu, ref = make_pair(kind, [n], m=1.3, eta=0.2, mu=0.9, k_interactions=1.1)
    rng = np.random.default_rng(n)
    u0 = rng.normal(0.0, 2.0, gpu.size).reshape(gpu.shape)
    v0 = rng.normal(0.0, 0.1, gpu.size).reshape(gpu.shape)
    gpu.u = u0
    ref.u = u0
    gpu.v = v0
    ref.v = v0
    assert_same(gpu, ref)
    gpu.timeStep()
    ref.timeStep()
    assert_same(gpu, ref)
    gpu.timeSteps(137)
    ref.timeSteps(137)
    assert_same(gpu, ref)


@pytest.mark.parametrize("kind", ["Line1d_Cuspy", "Line2d_Cuspy", "Line1d_SemiSmooth"])
def test_flow_steps(kind):
    gpu, ref = make_pair(kind, [512])
    gpu.flowSteps(300, 0.05)
    ref.flowSteps(300, 0.05)
    assert_same(gpu, ref)
    gpu.u_frame = gpu.u_frame + 0.5
    ref.u_frame = ref.u_frame + 0.5
    assert_same(gpu, ref)


@pytest.mark.parametrize("kind", list(KINDS))
def test_quasistatic_cycles(kind):
    """eventDrivenStep + minimise (the reference's examples/*.py protocol), with activity timing."""
    gpu, ref = make_pair(kind, [256], k_frame=1e-2)
    if kind.endswith("Smooth") and not kind.endswith("SemiSmooth"):
        for _ in range(3):
            gpu.u_frame = gpu.u_frame + 0.3
            ref.u_frame = ref.u_frame + 0.3
            assert gpu.minimise(time_activity=True) == ref.minimise(time_activity=True)
            assert gpu.quasistaticActivityFirst == ref.quasistaticActivityFirst
            assert gpu.quasistaticActivityLast == ref.quasistaticActivityLast
            assert_same(gpu, ref)
        return
    for step in range(12):
        if step == 0:
            gpu.u_frame = 0.0
            ref.u_frame = 0.0
        else:
            assert gpu.eventDrivenStep(1e-3, step % 2 == 0) == ref.eventDrivenStep(1e-3, step % 2 == 0)
        if step % 2 == 0:
            assert gpu.minimise(time_activity=True) == ref.minimise(time_activity=True) == 0
            assert gpu.quasistaticActivityFirst == ref.quasistaticActivityFirst
            assert gpu.quasistaticActivityLast == ref.quasistaticActivityLast
        assert_same(gpu, ref)


@pytest.mark.parametrize("direction", [1, -1])
def test_event_driven_direction(direction):
    gpu, ref = make_pair("Line1d_Cuspy", [300])
    for kick in [False, True, False, True]:
        assert gpu.maxUniformDisplacement(direction) == ref.maxUniformDisplacement(direction)
        assert gpu.eventDrivenStep(1e-4, kick, direction) == ref.eventDrivenStep(1e-4, kick, direction)
        assert_same(gpu, ref)
    assert gpu.minimise() == ref.minimise()
    assert_same(gpu, ref)


def test_time_steps_until_event():
    gpu, ref = make_pair("Line1d_Cuspy", [400], k_frame=1e-2)
    gpu.eventDrivenStep(1e-3, True)
    ref.eventDrivenStep(1e-3, True)
    a = gpu.timeStepsUntilEvent()
    b = ref.timeStepsUntilEvent()
    assert a == b
    assert_same(gpu, ref)
    assert gpu.timeStepsUntilEvent() == ref.timeStepsUntilEvent()
    assert_same(gpu, ref)


def test_trigger_and_truncate():
    """Reference test_Line1d.py:221-248 pattern, compared with the oracle."""
    gpu, ref = make_pair("Line1d_Cuspy", [64], k_frame=0.1)
    i_n = gpu.chunk.index_at_align.copy()
    gpu.trigger(5, 0.2)
    ref.trigger(5, 0.2)
    assert_same(gpu, ref)  # forces stay those before the trigger
    gpu.u_frame = 0.01
    ref.u_frame = 0.01
    assert_same(gpu, ref)
    gpu.v = np.full(gpu.shape, 1e-3)
    ref.v = np.full(ref.shape, 1e-3)
    assert_same(gpu, ref)
    a = gpu.minimise_truncate(i_n=i_n, A_truncate=1)
    b = ref.minimise_truncate(i_n=i_n, A_truncate=1)
    assert a == b > 0
    assert gpu.quasistaticActivityFirst == ref.quasistaticActivityFirst
    assert_same(gpu, ref)
    a = gpu.minimise_truncate(i_n=i_n, S_truncate=3)
    b = ref.minimise_truncate(i_n=i_n, S_truncate=3)
    assert a == b
    assert_same(gpu, ref)


def test_advance_to_fixed_force():
    gpu, ref = make_pair("Line1d_Cuspy", [128], k_frame=0.1)
    gpu.minimise()
    ref.minimise()
    gpu.advanceToFixedForce(0.05, allow_plastic=True)
    ref.advanceToFixedForce(0.05, allow_plastic=True)
    assert_same(gpu, ref)
    with pytest.raises(RuntimeError, match="assertion failed"):
        gpu.advanceToFixedForce(50.0)


def test_errors():
    gpu, ref = make_pair("Line1d_Cuspy", [64])
    gpu.u_frame = 5.0
    with pytest.raises(RuntimeError, match="No convergence found"):
        gpu.minimise(max_iter=5)
    assert gpu.minimise(max_iter=5, max_iter_is_error=False) == 6
    smooth, _ = make_pair("Line1d_Smooth", [64])
    with pytest.raises(RuntimeError, match="Operation not possible"):
        smooth.maxUniformDisplacement()
    u = gpu.u
    u[3] = np.nan
    gpu.u = u
    with pytest.raises(RuntimeError, match="NaN entries found"):
        gpu.timeSteps(3)


def test_regeneration_sweep():
    """Reference test_Line1d.py:277-341 pattern: sweep u over >1000 wells forward and back with a
    100-position chunk, restore the chunk from (state_at(start), data[..., 0], start)."""
    gpu, ref = make_pair("Line1d_Cuspy", [3], "weibull", (2.0, 1.1, 1e-3), offset=-50.0, nchunk=100,
                         mu=0.7, k_frame=0.1, eta=1.0, dt=1.0)
    du = np.array([5.0, 7.0, 10.0])
    saved = None
    for repeat in range(3):
        if repeat >= 1:
            st, val, start, u = saved
            gpu.chunk.restore(state=st, value=val, index=start)
            ref.chunk.restore(state=st, value=val, index=start)
            gpu.u = u
            ref.u = u
        for i in list(range(1500)) + list(range(1500))[::-1]:
            gpu.u = i * du
            ref.u = i * du
            assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align), (repeat, i)
            assert np.array_equal(gpu.chunk.left_of_align, ref.chunk.left_of_align)
            assert np.array_equal(gpu.chunk.right_of_align, ref.chunk.right_of_align)
            assert np.array_equal(gpu.f_potential, ref.f_potential)
            if (repeat == 0 and i == 500) or (repeat == 1 and i == 1000):
                start = gpu.chunk.start.copy()
                assert np.array_equal(start, ref.chunk.start)
                st = gpu.chunk.state_at(start)
                assert np.array_equal(st, ref.chunk.state_at(start))
                saved = (st, gpu.chunk.data[..., 0].copy(), start, gpu.u.copy())
        assert_same(gpu, ref)


@pytest.mark.parametrize("which,nstep", [("Line1d_Cuspy_Laplace", 40), ("Line1d_SemiSmooth_Laplace", 60),
                                         ("Line2d_Cuspy_Laplace", 20), ("Particles_Cuspy", 60)])
def test_golden_prefix_gpu(which, nstep):
    """The reference's historic golden trajectories, run on the GPU."""
    import pathlib

    golden = np.load(pathlib.Path(__file__).parent / "golden" / (which + ".npz"))
    common = dict(m=1.0, eta=2.0 * np.sqrt(3.0) / 10.0, mu=1.0, dt=0.1, seed=0, distribution="random",
                  parameters=[2.0], offset=-50)
    if which == "Line1d_Cuspy_Laplace":
        s = fqsb.Line1d.System_Cuspy_Laplace(shape=[1000], k_interactions=1.0, k_frame=1.0 / 1000, **common)
    elif which == "Line1d_SemiSmooth_Laplace":
        s = fqsb.Line1d.System_SemiSmooth_Laplace(shape=[1000], k_interactions=1.0, kappa=1.0, k_frame=1.0 / 1000,
                                                  **common)
    elif which == "Line2d_Cuspy_Laplace":
        s = fqsb.Line2d.System_Cuspy_Laplace(shape=[50, 50], k_interactions=1.0, k_frame=1.0 / 2500, **common)
    else:
        s = fqsb.Particles.System_Cuspy(shape=[1000], k_frame=1.0 / 1000, **common)
    for step in range(nstep):
        i_n = np.copy(s.chunk.index_at_align)
        if step == 0:
            s.u_frame = 0.0
        else:
            s.eventDrivenStep(1e-3, step % 2 == 0)
        if step % 2 == 0:
            assert s.minimise() == 0
        assert np.isclose(s.u_frame, golden["frame"][step]), step
        assert np.isclose(np.mean(s.f_frame), golden["f_frame"][step]), step
        assert np.sum(s.chunk.index_at_align - i_n) == golden["S"][step], step


def test_full_size_yields_sampled():
    """N = 2^22, nchunk = 2000 (the large-N throughput workload): for sampled particles the current
    well (index, left and right yield) equals the oracle's canonical sequence, after construction
    and after a random displacement; a second construction and run are identical (determinism)."""
    N = 2 ** 22
    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1, shape=[N], seed=1,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-1000.0, nchunk=2000)
    s = fqsb.Line1d.System_Cuspy_Laplace(**par)
    rng = np.random.default_rng(5)
    sample = [int(p) for p in rng.integers(0, N, 32)] + [0, N - 1]
    u0 = rng.normal(0.0, 30.0, N)
    for step in range(2):
        idx, left, right = s.chunk.index_at_align, s.chunk.left_of_align, s.chunk.right_of_align
        for p in sample:
            ref = O.sequence(1, p, "weibull", [2.0, 1.0, 1e-5], -1000.0, 2000, int(idx[p]), 2)
            assert left[p] == ref[0] and right[p] == ref[1], p
        s.u = u0
    s.timeSteps(20)
    u1, i1 = s.u, s.chunk.index_at_align
    del s
    s2 = fqsb.Line1d.System_Cuspy_Laplace(**par)
    s2.u = u0
    s2.timeSteps(20)
    assert np.array_equal(s2.u, u1)
    assert np.array_equal(s2.chunk.index_at_align, i1)


@pytest.mark.parametrize("kind", ["Line1d_Cuspy", "Line2d_Cuspy", "Particles_Cuspy", "Line1d_SemiSmooth",
                                  "Line1d_Smooth"])
def test_regeneration_inside_steps(kind):
    """Particles slide across many wells inside minimise / flowSteps with a 40-position chunk, so chunk
    windows move during the fused steps (the run graph's regeneration branch) -- compared with the oracle."""
    gpu, ref = make_pair(kind, [128], nchunk=40, offset=-5.0, k_frame=0.5, eta=0.5)
    for du in [12.0, 15.0, -20.0]:
        gpu.u_frame = gpu.u_frame + du
        ref.u_frame = ref.u_frame + du
        assert gpu.minimise(time_activity=True, max_iter=200000) == ref.minimise(time_activity=True, max_iter=200000)
        assert gpu.quasistaticActivityFirst == ref.quasistaticActivityFirst
        assert gpu.quasistaticActivityLast == ref.quasistaticActivityLast
        assert_same(gpu, ref)
    gpu.flowSteps(3000, 0.2)
    ref.flowSteps(3000, 0.2)
    assert_same(gpu, ref)
    assert np.max(np.abs(gpu.chunk.start)) > 20  # the windows did move


def test_regeneration_inside_steps_large():
    """Same at 1d N = 2^17 (many CTAs; several pending CTAs per step)."""
    gpu, ref = make_pair("Line1d_Cuspy", [2 ** 17], nchunk=40, offset=-5.0, k_frame=0.5, eta=0.5)
    gpu.flowSteps(800, 0.5)
    ref.flowSteps(800, 0.5)
    assert_same(gpu, ref)
    assert np.max(gpu.chunk.start) > 0


def test_large_ring_two_per_thread():
    """1d N = 2^18: the launch shape with two particles per thread (N >= 2 * 152 * 512), the one the
    large-N throughput workload runs; flow with window regeneration, a frame jump and minimise."""
    gpu, ref = make_pair("Line1d_Cuspy", [2 ** 18], nchunk=40, offset=-5.0)
    gpu.flowSteps(400, 0.5)
    ref.flowSteps(400, 0.5)
    assert_same(gpu, ref)
    gpu.u_frame = gpu.u_frame + 0.5
    ref.u_frame = ref.u_frame + 0.5
    assert gpu.minimise(max_iter=3000, max_iter_is_error=False) == ref.minimise(max_iter=3000, max_iter_is_error=False)
    assert_same(gpu, ref)
