"""Line1d.System_Cuspy_LongRange on the GPU: the reference's own tests, the golden trajectory of
examples/Line1d_Cuspy_Laplace_LongRange.py, and bit-for-bit parity with the oracle (sequential
all-pairs sums in the reference's order) through dynamics, minimise and event-driven steps."""

import numpy as np
import pytest

from oracle import oracle as O

from test_oracle_longrange import COMMON, check_event_driven, check_interactions

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

GOLDEN = __import__("pathlib").Path(__file__).parent / "golden"
FIELDS = ["u", "v", "a", "f", "f_potential", "f_interactions", "f_frame", "f_damping"]
MAXIT = dict(max_iter=20000, max_iter_is_error=False)


def gpu_make(N, k, alpha):
    return fqsb.Line1d.System_Cuspy_LongRange(k_interactions=k, alpha=alpha, shape=[N], **COMMON)


def test_interactions():
    check_interactions(gpu_make)


def test_event_driven():
    check_event_driven(gpu_make)


def make_pair(n, alpha):
    par = dict(m=1.0, eta=0.3, mu=1.0, k_interactions=0.8, alpha=alpha, k_frame=1.0 / n, dt=0.1, shape=[n], seed=9,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-20.0, nchunk=200)
    return fqsb.Line1d.System_Cuspy_LongRange(**par), O.line1d_longrange(**par, sum_mode=O.SUM_PAIRWISE,
                                                                         math_mode=O.MATH_PORTABLE)


def assert_same(gpu, ref):
    for name in FIELDS:
        g, r = getattr(gpu, name), getattr(ref, name)
        assert np.array_equal(g, r), (name, np.max(np.abs(g - r)))
    assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align)
    assert gpu.inc == ref.inc
    assert gpu.u_frame == ref.u_frame
    assert gpu.residual == ref.residual


@pytest.mark.parametrize("n", [2, 3, 10, 257, 1000, 2500])
@pytest.mark.parametrize("alpha", [1.0, 0.7])
def test_parity(n, alpha):
    gpu, ref = make_pair(n, alpha)
    u0 = np.random.default_rng(n).normal(0.0, 0.3, n)
    gpu.u = u0
    ref.u = u0
    assert_same(gpu, ref)
    gpu.timeSteps(100)
    ref.timeSteps(100)
    assert_same(gpu, ref)
    assert gpu.minimise(**MAXIT) == ref.minimise(**MAXIT)
    assert_same(gpu, ref)
    assert gpu.eventDrivenStep(1e-4, True) == ref.eventDrivenStep(1e-4, True)
    assert gpu.minimise(**MAXIT) == ref.minimise(**MAXIT)
    assert_same(gpu, ref)
    gpu.flowSteps(100, 0.3)
    ref.flowSteps(100, 0.3)
    assert_same(gpu, ref)


def test_host_driven_launches(monkeypatch):
    monkeypatch.setenv("FQSB_NO_GRAPH", "1")
    gpu, ref = make_pair(1500, 1.0)
    gpu.u_frame = 3.0
    ref.u_frame = 3.0
    assert gpu.minimise(**MAXIT) == ref.minimise(**MAXIT)
    assert_same(gpu, ref)


def test_golden_prefix():
    golden = np.load(GOLDEN / "Line1d_Cuspy_Laplace_LongRange.npz")
    par = dict(m=1.0, eta=2.0 * np.sqrt(3.0) / 10.0, mu=1.0, k_interactions=1.0, alpha=1, k_frame=1.0 / 1000, dt=0.1,
               shape=[1000], seed=0, distribution="random", parameters=[2.0], offset=-50)
    gpu = fqsb.Line1d.System_Cuspy_LongRange(**par)
    ref = O.line1d_longrange(**par, sum_mode=O.SUM_PAIRWISE, math_mode=O.MATH_PORTABLE)
    for step in range(30):
        i_n = np.copy(gpu.chunk.index_at_align)
        if step == 0:
            gpu.u_frame = 0.0
            ref.u_frame = 0.0
        else:
            gpu.eventDrivenStep(1e-3, step % 2 == 0)
            ref.eventDrivenStep(1e-3, step % 2 == 0)
        if step % 2 == 0:
            assert gpu.minimise(max_iter=1000000) == 0
            assert ref.minimise(max_iter=1000000) == 0
        assert np.isclose(gpu.u_frame, golden["frame"][step]), step
        assert np.isclose(np.mean(gpu.f_frame), golden["f_frame"][step]), step
        assert np.sum(gpu.chunk.index_at_align - i_n) == golden["S"][step], step
    assert_same(gpu, ref)
