"""LongRange1d of the oracle against the reference's own tests (tests/test_Line1d.py:479-563) and the
golden trajectory of examples/Line1d_Cuspy_Laplace_LongRange.py (in test_oracle_golden.py)."""

import numpy as np

from oracle import oracle as O

COMMON = dict(m=1.0, eta=1.0, mu=1.0, k_frame=0.1, dt=1.0, seed=0, distribution="delta", parameters=[1.0],
              offset=-49.5, nchunk=100)


def check_interactions(make):
    N, k = 10, 0.12
    system = make(N, k, 1.0)
    dp = np.arange(N)
    dn = np.arange(N)[::-1] + 1
    d = np.where(dp < dn, dp, dn)
    x = np.zeros(N)
    x[0] = 1
    system.u = x
    f = np.zeros_like(x)
    for j in range(1, N):
        f[j] = k * (x[0] - x[j]) / (d[j] ** 2)
    f[0] = -np.sum(f)
    for i in range(N):
        system.u = np.roll(x, i)
        assert np.allclose(np.roll(f, i), system.f_interactions)


def check_event_driven(make):
    N = 3
    system = make(N, 1.0, 1.0)
    assert system.residual < 1e-5
    i_n = system.chunk.index_at_align
    system.eventDrivenStep(0.2, False)
    assert system.residual < 1e-5
    assert np.allclose(system.u, (0.5 - 0.1) * np.ones(N))
    assert np.all(system.chunk.index_at_align == i_n)
    assert np.isclose(system.u_frame, (0.5 - 0.1) * (1.0 + 0.1) / 0.1)
    i_n = system.chunk.index_at_align
    system.eventDrivenStep(0.2, True)
    assert np.allclose(system.u, (0.5 + 0.1) * np.ones(N))
    assert not np.all(system.chunk.index_at_align == i_n)
    assert np.isclose(system.u_frame, (0.5 + 0.1) * (1.0 + 0.1) / 0.1)
    i_n = system.chunk.index_at_align
    system.eventDrivenStep(0.2, False)
    assert np.allclose(system.u, (1.5 - 0.1) * np.ones(N))
    assert np.all(system.chunk.index_at_align == i_n)
    i_n = system.chunk.index_at_align
    system.eventDrivenStep(0.2, True)
    assert np.allclose(system.u, (1.5 + 0.1) * np.ones(N))
    assert not np.all(system.chunk.index_at_align == i_n)
    assert np.isclose(system.u_frame, (1.5 + 0.1) * (1.0 + 0.1) / 0.1)


def oracle_make(N, k, alpha):
    return O.line1d_longrange(k_interactions=k, alpha=alpha, shape=[N], **COMMON)


def test_interactions():
    check_interactions(oracle_make)


def test_event_driven():
    check_event_driven(oracle_make)
