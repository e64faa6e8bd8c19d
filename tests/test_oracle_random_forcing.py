"""RandomNormalForcing (System_Cuspy_Laplace_RandomForcing) of the oracle.

The reference draws every particle's thermal force from one pcg32 stream (prrng's pcg32(seed), the
default PCG stream), in particle order, every `dinc` increments, with prrng's normal transform, and
the example draws `dinc_init` with prrng.pcg32(0).randint.  prrng is not in the reference tree; the
oracle restates pcg32's default-stream seeding, the PCG bounded draw for randint and the normal
quantile mean + stddev sqrt(2) erfinv(2 r - 1), r = u32 2^-32.  The golden trajectory
examples/Line1d_System_Cuspy_Laplace_RandomForcing.py + .h5 (500 outputs of flowSteps(1000) at finite
temperature: frame position, mean frame force, instantaneous temperature, np.allclose) pins the choice
(the other candidate streams and randint forms miss the first output by ~20% in temperature)."""

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = __import__("pathlib").Path(__file__).parent / "golden"


def test_reference_unit_test():
    """tests/test_Line1d.py:565-600: with dinc_init = dinc = 1 every increment redraws all forces."""
    N = 10
    system = O.line1d_random_forcing(m=1, eta=1, mu=1, k_interactions=1, k_frame=0.1, dt=1, mean=0, stddev=1,
                                     seed_forcing=0, dinc_init=np.ones(N, dtype=int), dinc=np.ones(N, dtype=int),
                                     shape=[N], seed=0, distribution="delta", parameters=[1.0], offset=-49.5,
                                     nchunk=100)
    assert system.residual < 1e-5
    # the same stream, drawn by hand: mean + stddev sqrt(2) erfinv(2 r - 1)
    from scipy.special import erfinv

    state, inc = O.pcg32_seed(0)
    r = []
    M = (1 << 64) - 1
    for _ in range(2 * N):
        old = state
        state = (old * 0x5851F42D4C957F2D + inc) & M
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        r.append((((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF) * 2.0 ** -32)
    r = np.array(r)
    expect = np.sqrt(2.0) * erfinv(2 * r - 1)
    system.inc = system.inc + 1
    system.refresh()
    assert system.residual > 1e-5
    assert np.allclose(system.f_thermal, expect[:N])
    system.inc = system.inc + 1
    system.refresh()
    assert np.allclose(system.f_thermal, expect[N:])


def run_golden(nout):
    golden = np.load(GOLDEN / "Line1d_System_Cuspy_Laplace_RandomForcing.npz")
    N = 1000
    common = dict(m=1.0, eta=2.0 * np.sqrt(3.0) / 10.0, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1,
                  shape=[N], seed=0, distribution="random", parameters=[2.0], offset=-50, sum_mode=O.SUM_SEQUENTIAL,
                  math_mode=O.MATH_LIBM)
    athermal = O.line1d("Cuspy", **common)
    athermal.minimise()
    system = O.line1d_random_forcing(mean=0.0, stddev=0.05, seed_forcing=0, dinc_init=O.pcg32_randint(0, N, 100),
                                     dinc=100 * np.ones(N, dtype=np.int64), **common)
    system.u = athermal.u
    for k in range(nout):
        system.flowSteps(1000, 5e-2)
        assert np.isclose(system.u_frame, golden["frame"][k]), k
        assert np.isclose(np.mean(system.f_frame), golden["f_frame"][k]), k
        assert np.isclose(system.temperature, golden["t_insta"][k]), k


def test_golden_prefix():
    run_golden(25)


@pytest.mark.slow
def test_golden_full():
    run_golden(500)


def _advance(state, delta, inc):
    """pcg32 jump-ahead by delta steps (Brown 1994), as the device draw kernels do it."""
    M = (1 << 64) - 1
    cm, cp, am, ap = 0x5851F42D4C957F2D, inc, 1, 0
    while delta > 0:
        if delta & 1:
            am, ap = (am * cm) & M, (ap * cm + cp) & M
        cp, cm = ((cm + 1) * cp) & M, (cm * cm) & M
        delta >>= 1
    return (am * state + ap) & M


def test_draw_numbering_by_scan():
    """The device numbers a step's draws by an exclusive scan of the drawing particles over the flat
    index (1024-particle tiles) and jumps the stream to each particle's draw: the oracle's sequential
    loop (detail.h:935-940) must give the same state, increments and forces."""
    N = 2500
    rng = np.random.default_rng(4)
    dinc_init, dinc = rng.integers(0, 6, N), rng.integers(1, 5, N)
    ref = O.line1d("Cuspy", m=1.0, eta=0.3, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1, seed=3,
                   distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-20.0, nchunk=100, shape=[N])
    O.attach_random_forcing(ref, 0.1, 0.2, 9, dinc_init, dinc)
    state, inc = O.pcg32_seed(9)
    nxt = dinc_init.astype(np.int64)
    f = np.zeros(N)
    sc = 0.2 * np.sqrt(2.0)
    for step in range(6):
        if step:
            ref.timeStep()
        draw = step >= nxt
        tiles = np.add.reduceat(draw.astype(np.int64), np.arange(0, N, 1024))
        offset = np.concatenate([[0], np.cumsum(tiles)[:-1]])
        rank = np.repeat(offset, 1024)[:N] + (np.cumsum(draw) - draw - np.repeat(np.cumsum(tiles) - tiles, 1024)[:N])
        for p in np.flatnonzero(draw):
            old = _advance(state, int(rank[p]), inc)
            xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
            rot = old >> 59
            r = (((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF) * 2.0 ** -32
            f[p] = 0.1 + sc * O.math("erfinv", 2.0 * r - 1.0)
        nxt = nxt + np.where(draw, dinc, 0)
        state = _advance(state, int(draw.sum()), inc)
        assert np.array_equal(f, ref.f_thermal), step
        assert np.array_equal(nxt, ref.thermal_next), step
        assert state == ref.thermal_state, step


def test_set_f_thermal_keeps_f():
    """set_f_thermal changes f_thermal only; f follows at the next computeForce (here set_u_frame)."""
    N = 50
    s = O.line1d_random_forcing(m=1, eta=1, mu=1, k_interactions=1, k_frame=0.1, dt=1, mean=0, stddev=1,
                                seed_forcing=0, dinc_init=np.zeros(N, dtype=int), dinc=np.ones(N, dtype=int),
                                shape=[N], seed=0, distribution="delta", parameters=[1.0], offset=-49.5, nchunk=100)
    f0 = s.f.copy()
    s.f_thermal = np.full(N, 2.0)
    assert np.array_equal(s.f, f0)
    s.u_frame = s.u_frame
    assert np.array_equal(s.f, ((s.f_frame + s.f_potential) + s.f_interactions) + s.f_damping + 2.0)
