"""Quartic / QuarticGradient interactions on the GPU: the reference's interaction tests, the golden
trajectory of Line1d_Cuspy_Quartic, and bit-for-bit parity with the oracle through dynamics,
minimise and event-driven steps (one-cluster path for small rings, graph path for large rings and
for the 2d grid)."""

import numpy as np
import pytest

from oracle import oracle as O

from test_oracle_quartic import CHECKS, COMMON

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

GOLDEN = __import__("pathlib").Path(__file__).parent / "golden"
FIELDS = ["u", "v", "a", "f", "f_potential", "f_interactions", "f_frame", "f_damping"]

GPU = {
    "Quartic1d": lambda shape, a, b, **kw: fqsb.Line1d.System_Cuspy_Quartic(a1=a, a2=b, shape=shape, **kw),
    "QuarticGradient1d": lambda shape, a, b, **kw: fqsb.Line1d.System_Cuspy_QuarticGradient(k2=a, k4=b, shape=shape,
                                                                                            **kw),
    "QuarticGradient2d": lambda shape, a, b, **kw: fqsb.Line2d.System_Cuspy_QuarticGradient(k2=a, k4=b, shape=shape,
                                                                                            **kw),
}
REF = {
    "Quartic1d": lambda shape, a, b, **kw: O.line1d_quartic(a1=a, a2=b, shape=shape, **kw),
    "QuarticGradient1d": lambda shape, a, b, **kw: O.line1d_quartic_gradient(k2=a, k4=b, shape=shape, **kw),
    "QuarticGradient2d": lambda shape, a, b, **kw: O.line2d_quartic_gradient(k2=a, k4=b, shape=shape, **kw),
}
MAXIT = dict(max_iter=20000, max_iter_is_error=False)


@pytest.mark.parametrize("kind,check", CHECKS)
def test_interactions(kind, check):
    """tests/test_Line1d.py:402-476 and tests/test_Line2d.py:60-173 on the GPU classes."""
    check(lambda shape, a, b: GPU[kind](shape, a, b, **COMMON))


def make_pair(kind, shape, a, b, **kw):
    par = dict(m=1.0, eta=kw.get("eta", 0.2), mu=1.0, k_frame=kw.get("k_frame", 1.0 / int(np.prod(shape))), dt=0.1,
               seed=kw.get("seed", 7), distribution="weibull", parameters=[2.0, 1.0, 1e-5],
               offset=kw.get("offset", -20.0), nchunk=kw.get("nchunk", 200))
    return GPU[kind](shape, a, b, **par), REF[kind](shape, a, b, **par, sum_mode=O.SUM_PAIRWISE,
                                                     math_mode=O.MATH_PORTABLE)


def assert_same(gpu, ref):
    for name in FIELDS:
        g, r = getattr(gpu, name), getattr(ref, name)
        assert np.array_equal(g, r), (name, np.max(np.abs(g - r)))
    assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align)
    assert np.array_equal(gpu.chunk.start, ref.chunk.start)
    assert gpu.inc == ref.inc
    assert gpu.u_frame == ref.u_frame
    assert gpu.residual == ref.residual


# 160000 particles: the large-ring launch shape with two particles per thread; 2^17: one per thread
CASES = [("Quartic1d", [n]) for n in (7, 1000, 5000, 2 ** 17, 160000)] + \
        [("QuarticGradient1d", [n]) for n in (7, 1000, 5000, 2 ** 17, 160000)] + \
        [("QuarticGradient2d", s) for s in ([3, 5], [16, 24], [37, 45], [64, 96], [256, 320])]


@pytest.mark.parametrize("kind,shape", CASES)
def test_parity(kind, shape):
    gpu, ref = make_pair(kind, shape, 0.8, 0.6)
    rng = np.random.default_rng(int(np.prod(shape)))
    u0 = rng.normal(0.0, 0.4, gpu.size).reshape(gpu.shape)
    gpu.u = u0
    ref.u = u0
    assert_same(gpu, ref)
    gpu.timeSteps(150)
    ref.timeSteps(150)
    assert_same(gpu, ref)
    if gpu.size > 50000:
        # large systems: dynamics only (the oracle's minimise at this size takes minutes)
        gpu.flowSteps(100, 0.2)
        ref.flowSteps(100, 0.2)
        assert_same(gpu, ref)
        return
    assert gpu.minimise(**MAXIT) == ref.minimise(**MAXIT)
    assert_same(gpu, ref)
    for kick in (False, True):
        assert gpu.eventDrivenStep(1e-4, kick) == ref.eventDrivenStep(1e-4, kick)
        assert gpu.minimise(**MAXIT) == ref.minimise(**MAXIT)
        assert_same(gpu, ref)
    gpu.flowSteps(200, 0.2)
    ref.flowSteps(200, 0.2)
    assert_same(gpu, ref)


@pytest.mark.parametrize("n", [64, 4096])
def test_parity_graph_path(monkeypatch, n):
    """Small rings through the CUDA-graph path (FQSB_NO_SMALL=1) as well."""
    monkeypatch.setenv("FQSB_NO_SMALL", "1")
    for kind in ("Quartic1d", "QuarticGradient1d"):
        gpu, ref = make_pair(kind, [n], 1.1, 0.3)
        gpu.u_frame = 2.0
        ref.u_frame = 2.0
        assert gpu.minimise(**MAXIT) == ref.minimise(**MAXIT)
        assert_same(gpu, ref)
        gpu.flowSteps(300, 0.3)
        ref.flowSteps(300, 0.3)
        assert_same(gpu, ref)


def test_golden_prefix():
    """examples/Line1d_Cuspy_Quartic.py against the .h5 file (100 steps), bit-exact with the oracle."""
    golden = np.load(GOLDEN / "Line1d_Cuspy_Quartic.npz")
    par = dict(m=1.0, eta=2.0 * np.sqrt(3.0) / 10.0, mu=1.0, a1=1.0, a2=1.0, k_frame=1.0 / 1000, dt=0.1,
               shape=[1000], seed=0, distribution="random", parameters=[2.0], offset=-50)
    gpu = fqsb.Line1d.System_Cuspy_Quartic(**par)
    ref = O.line1d_quartic(**par, sum_mode=O.SUM_PAIRWISE, math_mode=O.MATH_PORTABLE)
    for step in range(100):
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


def test_interface():
    gpu = GPU["Quartic1d"]([8], 1.0, 1.0, **COMMON)
    assert repr(gpu) == "<FrictionQPotSpringBlock.Line1d.System_Cuspy_Quartic>"
    with pytest.raises(RuntimeError):
        gpu.adjoint_forward(np.zeros(10), K=5, last=5)
