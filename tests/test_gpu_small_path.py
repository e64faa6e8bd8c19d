"""The one-cluster run kernel of small systems against the graph path, bit for bit.

Line1d / Particles systems with N <= 8192 run each timeSteps / flowSteps / minimise /
timeStepsUntilEvent as one launch of one thread-block cluster (state in registers, halos through
distributed shared memory); larger systems, Line2d and trajectory recording use the CUDA graph.
FQSB_NO_SMALL=1 at construction forces the graph path, so the same protocol can run both ways.
The oracle parity tests cover each path against the CPU restatement as well."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

FIELDS = ["u", "v", "a", "f", "f_potential", "f_interactions", "f_frame", "f_damping"]

MAKE = {
    "Line1d_Cuspy": lambda **p: fqsb.Line1d.System_Cuspy_Laplace(**p),
    "Line1d_SemiSmooth": lambda **p: fqsb.Line1d.System_SemiSmooth_Laplace(kappa=0.5, **p),
    "Line1d_Smooth": lambda **p: fqsb.Line1d.System_Smooth_Laplace(**p),
    "Particles_Cuspy": lambda **p: fqsb.Particles.System_Cuspy(**{k: v for k, v in p.items() if k != "k_interactions"}),
}


def make_both(monkeypatch, kind, n, **kw):
    par = dict(m=1.0, eta=kw.get("eta", 0.1), mu=1.0, k_interactions=1.0, k_frame=kw.get("k_frame", 1.0 / n),
               dt=0.1, shape=[n], seed=5, distribution="weibull", parameters=[2.0, 1.0, 1e-5],
               offset=kw.get("offset", -20.0), nchunk=kw.get("nchunk", 200))
    monkeypatch.delenv("FQSB_NO_SMALL", raising=False)
    small = MAKE[kind](**par)
    monkeypatch.setenv("FQSB_NO_SMALL", "1")
    graph = MAKE[kind](**par)
    monkeypatch.delenv("FQSB_NO_SMALL", raising=False)
    return small, graph


def assert_same(a, b):
    for name in FIELDS:
        x, y = getattr(a, name), getattr(b, name)
        assert np.array_equal(x, y), (name, np.max(np.abs(x - y)))
    assert np.array_equal(a.chunk.index_at_align, b.chunk.index_at_align)
    assert np.array_equal(a.chunk.start, b.chunk.start)
    assert a.inc == b.inc
    assert a.u_frame == b.u_frame
    assert a.residual == b.residual


@pytest.mark.parametrize("kind", list(MAKE))
@pytest.mark.parametrize("n", [1, 33, 1024, 5000, 8192])
def test_flow_event_minimise(monkeypatch, kind, n):
    small, graph = make_both(monkeypatch, kind, n)
    rng = np.random.default_rng(n)
    u0 = rng.normal(0.0, 0.5, n)
    for s in (small, graph):
        s.u = u0
    small.flowSteps(300, 0.3)
    graph.flowSteps(300, 0.3)
    assert_same(small, graph)
    for kick in (False, True):
        if kind.endswith("Smooth") and not kind.endswith("SemiSmooth"):
            # no event-driven step for the Smooth potential (maxUniformDisplacement is not defined)
            small.u_frame = small.u_frame + 0.01
            graph.u_frame = graph.u_frame + 0.01
        else:
            small.eventDrivenStep(1e-4, kick)
            graph.eventDrivenStep(1e-4, kick)
        assert small.minimise(max_iter=20000, max_iter_is_error=False) == \
            graph.minimise(max_iter=20000, max_iter_is_error=False)
        assert_same(small, graph)
    small.u_frame = small.u_frame + 0.05
    graph.u_frame = graph.u_frame + 0.05
    assert small.timeStepsUntilEvent(max_iter=5000) == graph.timeStepsUntilEvent(max_iter=5000)
    assert_same(small, graph)
    small.u_frame = small.u_frame + 0.05
    graph.u_frame = graph.u_frame + 0.05
    assert small.minimise(time_activity=True, max_iter=20000, max_iter_is_error=False) == \
        graph.minimise(time_activity=True, max_iter=20000, max_iter_is_error=False)
    assert small.quasistaticActivityFirst == graph.quasistaticActivityFirst
    assert small.quasistaticActivityLast == graph.quasistaticActivityLast
    assert_same(small, graph)


@pytest.mark.parametrize("n", [64, 4096])
def test_window_moves_and_truncate(monkeypatch, n):
    """Small chunk windows so that windows move inside the run; minimise_truncate on activity."""
    small, graph = make_both(monkeypatch, "Line1d_Cuspy", n, nchunk=40, offset=-5.0, k_frame=0.5, eta=0.5)
    small.flowSteps(800, 0.5)
    graph.flowSteps(800, 0.5)
    assert_same(small, graph)
    assert np.max(small.chunk.start) > 0
    i_n = small.chunk.index_at_align.copy()
    small.u_frame = small.u_frame + 1.0
    graph.u_frame = graph.u_frame + 1.0
    assert small.minimise_truncate(i_n=i_n, A_truncate=max(1, n // 8)) == \
        graph.minimise_truncate(i_n=i_n, A_truncate=max(1, n // 8))
    assert_same(small, graph)


def test_nan_reported(monkeypatch):
    small, _ = make_both(monkeypatch, "Line1d_Cuspy", 100)
    u = small.u
    u[3] = np.nan
    small.u = u
    with pytest.raises(RuntimeError, match="NaN entries found"):
        small.timeSteps(5)


@pytest.mark.parametrize("kind", ["Line1d_Cuspy", "Particles_Cuspy"])
@pytest.mark.parametrize("n", [64, 1024, 8192])
def test_short_runs_with_window_moves(monkeypatch, kind, n):
    """The one-cluster kernel takes one time step past the end of every run before it learns that the
    run is over, and then restores the state from before that step.  Runs of 1 to 5 steps with fast
    particles and 40-position chunk windows (a window move every few wells) make that extra step move
    windows often; the restored windows, wells and state must equal the graph path's."""
    small, graph = make_both(monkeypatch, kind, n, nchunk=40, offset=-5.0)
    rng = np.random.default_rng(n + 1)
    v0 = np.abs(rng.normal(3.0, 1.0, n))
    for s in (small, graph):
        s.v = v0
    moved = 0
    for k in range(60):
        start = small.chunk.start.copy()
        nsteps = 1 + k % 5
        small.timeSteps(nsteps)
        graph.timeSteps(nsteps)
        assert_same(small, graph)
        assert np.array_equal(small.chunk.data, graph.chunk.data), k
        moved += int(np.sum(small.chunk.start != start))
    assert moved > 0


@pytest.mark.parametrize("n", [64, 1024])
def test_window_moves_across_restore(monkeypatch, n):
    """The one-cluster kernel copies the new slots of a forward window move from a next-window buffer
    filled before the run.  chunk.restore with shifted values starts other sequences at the same
    window positions, so the buffers must be refilled; the windows moved in the runs before and after
    it must equal the graph path's, whose moves draw every value."""
    small, graph = make_both(monkeypatch, "Line1d_Cuspy", n, nchunk=40, offset=-5.0, k_frame=0.5, eta=0.5)
    for s in (small, graph):
        s.flowSteps(800, 0.5)
    assert_same(small, graph)
    assert np.array_equal(small.chunk.data, graph.chunk.data)
    start = small.chunk.start.copy()
    assert np.max(start) > 0
    state = small.chunk.state_at(start)
    value = small.chunk.data[..., 0] + 0.25
    for s in (small, graph):
        s.chunk.restore(state=state, value=value, index=start)
        s.flowSteps(800, 0.5)
    assert_same(small, graph)
    assert np.array_equal(small.chunk.data, graph.chunk.data)
    assert np.max(small.chunk.start - start) > 0
