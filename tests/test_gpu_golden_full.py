"""The reference's historic golden trajectories, run in full on the GPU.

Each of the reference's examples/*.py runs a protocol and asserts np.allclose on the frame position and
the mean frame force and exact equality of the avalanche size S against a stored .h5 file
(examples/Line1d_Cuspy_Laplace.py:35-67).  The same protocols run here through the CUDA path over their
whole length (1000 or 2000 event-driven steps, 200 for the all-pairs LongRange1d file, 500 outputs of
flowSteps(1000) for the thermal file), with the same assertions, against fixtures extracted from those
files (tests/golden/make_golden.py).  The "random" distribution of these files uses no elementary
function, so the GPU's yield positions equal the reference's bit for bit here.
"""

import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

GOLDEN = pathlib.Path(__file__).parent / "golden"
COMMON = dict(m=1.0, eta=2.0 * np.sqrt(3.0) / 10.0, mu=1.0, dt=0.1, seed=0, distribution="random",
              parameters=[2.0], offset=-50)


def make(which):
    """The systems of examples/<which>.py (e.g. examples/Line1d_Cuspy_Laplace.py:17-30)."""
    if which == "Line1d_Cuspy_Laplace":
        return fqsb.Line1d.System_Cuspy_Laplace(shape=[1000], k_interactions=1.0, k_frame=1.0 / 1000, **COMMON)
    if which == "Line1d_SemiSmooth_Laplace":
        return fqsb.Line1d.System_SemiSmooth_Laplace(shape=[1000], k_interactions=1.0, kappa=1.0, k_frame=1.0 / 1000,
                                                     **COMMON)
    if which == "Line2d_Cuspy_Laplace":
        return fqsb.Line2d.System_Cuspy_Laplace(shape=[50, 50], k_interactions=1.0, k_frame=1.0 / 2500, **COMMON)
    if which == "Line1d_Cuspy_Quartic":
        return fqsb.Line1d.System_Cuspy_Quartic(shape=[1000], a1=1.0, a2=1.0, k_frame=1.0 / 1000, **COMMON)
    if which == "Line1d_Cuspy_Laplace_LongRange":
        return fqsb.Line1d.System_Cuspy_LongRange(shape=[1000], k_interactions=1.0, alpha=1, k_frame=1.0 / 1000,
                                                  **COMMON)
    return fqsb.Particles.System_Cuspy(shape=[1000], k_frame=1.0 / 1000, **COMMON)


@pytest.mark.timeout(900)
@pytest.mark.parametrize("which", ["Line1d_Cuspy_Laplace", "Line1d_SemiSmooth_Laplace", "Line2d_Cuspy_Laplace",
                                   "Particles_Cuspy", "Line1d_Cuspy_Quartic", "Line1d_Cuspy_Laplace_LongRange"])
def test_golden_full(which):
    golden = np.load(GOLDEN / (which + ".npz"))
    system = make(which)
    for step in range(len(golden["S"])):
        i_n = np.copy(system.chunk.index_at_align)
        if step == 0:
            system.u_frame = 0.0
        else:
            system.eventDrivenStep(1e-3, step % 2 == 0)
        if step % 2 == 0:
            assert system.minimise() == 0, step
        assert np.isclose(system.u_frame, golden["frame"][step]), step
        assert np.isclose(np.mean(system.f_frame), golden["f_frame"][step]), step
        assert np.sum(system.chunk.index_at_align - i_n) == golden["S"][step], step


@pytest.mark.timeout(900)
def test_golden_full_random_forcing():
    """examples/Line1d_System_Cuspy_Laplace_RandomForcing.py + .h5: all 500 outputs of flowSteps(1000) at
    finite temperature (frame position, mean frame force, instantaneous temperature)."""
    from oracle import oracle as O  # the reference's seeding of dinc_init (prrng randint), restated

    golden = np.load(GOLDEN / "Line1d_System_Cuspy_Laplace_RandomForcing.npz")
    N = 1000
    common = dict(COMMON, k_interactions=1.0, k_frame=1.0 / N, shape=[N])
    athermal = fqsb.Line1d.System_Cuspy_Laplace(**common)
    athermal.minimise()
    system = fqsb.Line1d.System_Cuspy_Laplace_RandomForcing(mean=0.0, stddev=0.05, seed_forcing=0,
                                                            dinc_init=O.pcg32_randint(0, N, 100),
                                                            dinc=100 * np.ones(N, dtype=np.int64), **common)
    system.u = athermal.u
    for k in range(len(golden["frame"])):
        system.flowSteps(1000, 5e-2)
        assert np.isclose(system.u_frame, golden["frame"][k]), k
        assert np.isclose(np.mean(system.f_frame), golden["f_frame"][k]), k
        assert np.isclose(system.temperature, golden["t_insta"][k]), k
