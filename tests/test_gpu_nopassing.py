"""Line1d.System_Cuspy_Laplace_Nopassing on the GPU against the oracle and the reference's golden file.

The reference minimises this class with the overdamped no-passing fixed point
(include/FrictionQPotSpringBlock/detail.h:1694-1753) and checks it with
examples/Line1d_Cuspy_Laplace_Nopassing.py against a stored .h5 trajectory.  The GPU path must
give the oracle's numbers bit for bit (pairwise sums, as the device) and reproduce the golden file.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

GOLDEN = __import__("pathlib").Path(__file__).parent / "golden"
FIELDS = ["u", "v", "a", "f", "f_potential", "f_interactions", "f_frame", "f_damping"]


def make_pair(n, **kw):
    par = dict(mu=kw.get("mu", 1.0), k_interactions=kw.get("k_interactions", 1.0), k_frame=kw.get("k_frame", 1.0 / n),
               shape=[n], seed=kw.get("seed", 0), distribution=kw.get("distribution", "random"),
               parameters=kw.get("parameters", [2.0]), offset=kw.get("offset", -50.0), nchunk=kw.get("nchunk", 5000))
    gpu = fqsb.Line1d.System_Cuspy_Laplace_Nopassing(**par)
    ref = O.line1d_nopassing(**par, sum_mode=O.SUM_PAIRWISE, math_mode=O.MATH_PORTABLE)
    return gpu, ref


def assert_same(gpu, ref):
    for name in FIELDS:
        g, r = getattr(gpu, name), getattr(ref, name)
        assert np.array_equal(g, r), (name, np.max(np.abs(g - r)))
    assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align)
    assert np.array_equal(gpu.chunk.start, ref.chunk.start)
    assert gpu.inc == ref.inc
    assert gpu.u_frame == ref.u_frame
    assert gpu.residual == ref.residual


def test_golden_protocol():
    """examples/Line1d_Cuspy_Laplace_Nopassing.py, 1000 steps, against the .h5 file; bit-exact with the
    oracle along the way."""
    golden = np.load(GOLDEN / "Line1d_Cuspy_Laplace_Nopassing.npz")
    gpu, ref = make_pair(1000)
    for step in range(1000):
        i_n = np.copy(gpu.chunk.index_at_align)
        if step == 0:
            gpu.u_frame = 0.0
            ref.u_frame = 0.0
        else:
            gpu.eventDrivenStep(1e-3, step % 2 == 0)
            ref.eventDrivenStep(1e-3, step % 2 == 0)
        if step % 2 == 0:
            assert gpu.minimise(**MAXIT) == 0
            assert ref.minimise_nopassing(**MAXIT) == 0
        assert np.isclose(gpu.u_frame, golden["frame"][step]), step
        assert np.isclose(np.mean(gpu.f_frame), golden["f_frame"][step]), step
        assert np.sum(gpu.chunk.index_at_align - i_n) == golden["S"][step], step
        if step % 50 == 0:
            assert_same(gpu, ref)
    assert_same(gpu, ref)


# Every call below is bounded: from a rough configuration (e.g. random positions) the reference's
# Jacobi fixed point can oscillate between wells and never meet the tolerance, so an unbounded
# minimise would run forever on the reference as here.
MAXIT = dict(max_iter=100000, max_iter_is_error=False)


@pytest.mark.parametrize("n", [2, 3, 64, 1000, 5000, 2 ** 17])
def test_quasistatic_steps(n):
    gpu, ref = make_pair(n, distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-20.0, nchunk=200)
    for du in (0.0, 0.3, 2.5, 0.7):
        gpu.u_frame = gpu.u_frame + du
        ref.u_frame = ref.u_frame + du
        assert gpu.minimise(**MAXIT) == ref.minimise_nopassing(**MAXIT) == 0
        assert_same(gpu, ref)
        assert gpu.eventDrivenStep(1e-3, True) == ref.eventDrivenStep(1e-3, True)
        assert gpu.minimise(**MAXIT) == ref.minimise_nopassing(**MAXIT) == 0
        assert_same(gpu, ref)


def test_window_moves_inside_the_sweep():
    """A small chunk window: the no-passing updates move windows inside the fixed-point loop."""
    gpu, ref = make_pair(4096, nchunk=40, offset=-5.0, k_frame=0.5, k_interactions=0.7, mu=1.3)
    for du in (3.0, 11.0, 30.0):
        gpu.u_frame = gpu.u_frame + du
        ref.u_frame = ref.u_frame + du
        assert gpu.minimise(**MAXIT) == ref.minimise_nopassing(**MAXIT) == 0
        assert_same(gpu, ref)
    assert np.max(gpu.chunk.start) > 0


def test_not_converged_keeps_the_sweep_forces():
    gpu, ref = make_pair(1000, offset=-20.0, nchunk=200)
    gpu.u_frame = 5.0
    ref.u_frame = 5.0
    with pytest.raises(RuntimeError, match="No convergence found"):
        gpu.minimise(max_iter=2)
    gpu2, ref2 = make_pair(1000, offset=-20.0, nchunk=200)
    gpu2.u_frame = 5.0
    ref2.u_frame = 5.0
    assert gpu2.minimise(max_iter=3, max_iter_is_error=False) == ref2.minimise_nopassing(
        max_iter=3, max_iter_is_error=False) == 4
    assert_same(gpu2, ref2)
    assert gpu2.minimise(**MAXIT) == ref2.minimise_nopassing(**MAXIT) == 0
    assert_same(gpu2, ref2)


def test_interface():
    gpu, _ = make_pair(16)
    for name in ("timeStep", "timeSteps", "timeStepsUntilEvent", "flowSteps"):
        assert not hasattr(gpu, name)
    with pytest.raises(RuntimeError):
        gpu.minimise(time_activity=True)
    assert repr(gpu) == "<FrictionQPotSpringBlock.Line1d.System_Cuspy_Laplace_Nopassing>"
    one = fqsb.Line1d.System_Cuspy_Laplace_Nopassing(mu=1.0, k_interactions=1.0, k_frame=1.0, shape=[1], seed=0,
                                                       distribution="random", parameters=[2.0], offset=-50.0)
    with pytest.raises(RuntimeError, match="N >= 2"):
        one.minimise()
