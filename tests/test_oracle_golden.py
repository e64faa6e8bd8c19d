"""The oracle against the reference's historic golden trajectories.

The reference's examples/{Line1d_Cuspy_Laplace,Line2d_Cuspy_Laplace,
Line1d_SemiSmooth_Laplace,Particles_Cuspy,Line1d_Cuspy_Laplace_Nopassing,
Line1d_Cuspy_Quartic,Line1d_Cuspy_Laplace_LongRange}.py run an event-driven quasistatic
protocol and assert np.allclose on the frame position and the mean frame force,
and exact equality of the avalanche size S, against stored .h5 files
(examples/Line1d_Cuspy_Laplace.py:35-67).  The same protocol runs here through
the CPU oracle against fixtures extracted from those files
(tests/golden/make_golden.py).  Passing pins the pcg32 stream and seeding, the
"random" transform, the cumulative-sum chunk with forward regeneration and the
integrator.
"""

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = __import__("pathlib").Path(__file__).parent / "golden"


def make(which, sum_mode, math_mode=O.MATH_LIBM):
    common = dict(m=1.0, eta=2.0 * np.sqrt(3.0) / 10.0, mu=1.0, dt=0.1, seed=0, distribution="random",
                  parameters=[2.0], offset=-50, sum_mode=sum_mode, math_mode=math_mode)
    if which == "Line1d_Cuspy_Laplace":
        return O.line1d("Cuspy", shape=[1000], k_interactions=1.0, k_frame=1.0 / 1000, **common)
    if which == "Line1d_SemiSmooth_Laplace":
        return O.line1d("SemiSmooth", shape=[1000], k_interactions=1.0, k_frame=1.0 / 1000, kappa=1.0, **common)
    if which == "Line2d_Cuspy_Laplace":
        return O.line2d(shape=[50, 50], k_interactions=1.0, k_frame=1.0 / 2500, **common)
    if which == "Line1d_Cuspy_Laplace_LongRange":
        # examples/Line1d_Cuspy_Laplace_LongRange.py:17-30
        return O.line1d_longrange(shape=[1000], k_interactions=1.0, alpha=1, k_frame=1.0 / 1000, **common)
    if which == "Line1d_Cuspy_Quartic":
        # examples/Line1d_Cuspy_Quartic.py:17-31
        return O.line1d_quartic(shape=[1000], a1=1.0, a2=1.0, k_frame=1.0 / 1000, **common)
    if which == "Line1d_Cuspy_Laplace_Nopassing":
        # examples/Line1d_Cuspy_Laplace_Nopassing.py:17-26 (m = 1, eta = dt = 0)
        return O.line1d_nopassing(mu=1.0, k_interactions=1.0, k_frame=1.0 / 1000, shape=[1000], seed=0,
                                  distribution="random", parameters=[2.0], offset=-50, sum_mode=sum_mode,
                                  math_mode=math_mode)
    return O.particles("Cuspy", shape=[1000], k_frame=1.0 / 1000, **common)


def run_protocol(system, golden, nstep, minimise="minimise"):
    for step in range(nstep):
        i_n = np.copy(system.chunk.index_at_align)
        if step == 0:
            system.u_frame = 0.0
        else:
            system.eventDrivenStep(1e-3, step % 2 == 0)
        if step % 2 == 0:
            assert getattr(system, minimise)() == 0
        assert np.isclose(system.u_frame, golden["frame"][step]), step
        assert np.isclose(np.mean(system.f_frame), golden["f_frame"][step]), step
        assert np.sum(system.chunk.index_at_align - i_n) == golden["S"][step], step


CASES = [
    ("Line1d_Cuspy_Laplace", 160),
    ("Line1d_SemiSmooth_Laplace", 300),
    ("Line2d_Cuspy_Laplace", 60),
    ("Particles_Cuspy", 300),
    ("Line1d_Cuspy_Laplace_Nopassing", 1000),
    ("Line1d_Cuspy_Quartic", 100),
    ("Line1d_Cuspy_Laplace_LongRange", 8),
]


def minimiser(which):
    return "minimise_nopassing" if which.endswith("Nopassing") else "minimise"


@pytest.mark.parametrize("which,nstep", CASES)
@pytest.mark.parametrize("sum_mode", [O.SUM_SEQUENTIAL, O.SUM_PAIRWISE])
def test_golden_prefix(which, nstep, sum_mode):
    golden = np.load(GOLDEN / (which + ".npz"))
    run_protocol(make(which, sum_mode), golden, nstep, minimiser(which))


@pytest.mark.slow
@pytest.mark.parametrize("which", [c[0] for c in CASES])
def test_golden_full(which):
    golden = np.load(GOLDEN / (which + ".npz"))
    run_protocol(make(which, O.SUM_SEQUENTIAL), golden, len(golden["S"]), minimiser(which))


def test_golden_regenerates_chunk():
    """The Line1d golden crosses ~16k wells per particle with nchunk=5000: forward regeneration is pinned."""
    golden = np.load(GOLDEN / "Line1d_Cuspy_Laplace.npz")
    assert golden["S"].sum() / 1000 > 5000
