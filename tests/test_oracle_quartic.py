"""The Quartic interactions of the oracle against the reference's own interaction tests.

tests/test_Line1d.py:402-476 (System_Cuspy_Quartic, System_Cuspy_QuarticGradient) and
tests/test_Line2d.py:60-173 (Line2d System_Cuspy_QuarticGradient) displace one particle of a ring /
grid at rest in its well and compare f_interactions with the analytic stencil (np.allclose), for every
position of the displaced particle.  The golden trajectory of Line1d_Cuspy_Quartic is in
test_oracle_golden.py."""

import numpy as np
import pytest

from oracle import oracle as O

COMMON = dict(m=1.0, eta=1.0, mu=1.0, k_frame=0.1, dt=1.0, seed=0, distribution="delta", parameters=[1.0],
              offset=-49.5, nchunk=100)


def factories():
    """(builder(kind, shape, a, b, sum_mode), name) pairs, so the GPU tests can reuse the same checks."""
    return {
        "Quartic1d": lambda shape, a, b, **kw: O.line1d_quartic(a1=a, a2=b, shape=shape, **COMMON, **kw),
        "QuarticGradient1d": lambda shape, a, b, **kw: O.line1d_quartic_gradient(k2=a, k4=b, shape=shape, **COMMON,
                                                                                 **kw),
        "QuarticGradient2d": lambda shape, a, b, **kw: O.line2d_quartic_gradient(k2=a, k4=b, shape=shape, **COMMON,
                                                                                 **kw),
    }


def check_quartic1d(make):
    N = 10
    rng = np.random.default_rng(1)
    a1, a2, du = (float(x) for x in rng.random(3))
    system = make([N], a1, a2)
    assert system.residual < 1e-5
    u0 = np.array([du, 0, 0, 0, 0, 0, 0, 0, 0, 0])
    laplace = np.array([-2 * du, du, 0, 0, 0, 0, 0, 0, 0, du])
    du_p = np.array([-du, 0, 0, 0, 0, 0, 0, 0, 0, du])
    du_n = np.array([-du, du, 0, 0, 0, 0, 0, 0, 0, 0])
    f0 = a1 * laplace + a2 * (du_p**3 + du_n**3)
    for i in range(N):
        u = np.roll(u0, i)
        system.u = u
        assert np.allclose(system.f_interactions, np.roll(f0, i))
        assert np.allclose(system.u, u)


def check_quartic_gradient1d(make):
    N = 10
    rng = np.random.default_rng(2)
    k2, k4, du = (float(x) for x in rng.random(3))
    system = make([N], k2, k4)
    assert system.residual < 1e-5
    u0 = np.array([du, 0, 0, 0, 0, 0, 0, 0, 0, 0])
    laplace = np.array([-2 * du, du, 0, 0, 0, 0, 0, 0, 0, du])
    gradient = np.array([0, 0.5 * du, 0, 0, 0, 0, 0, 0, 0, 0.5 * du])
    f0 = k2 * laplace + k4 * laplace * gradient**2
    for i in range(N):
        u = np.roll(u0, i)
        system.u = u
        assert np.allclose(system.f_interactions, np.roll(f0, i))


def check_quartic_gradient2d_basic(make):
    rows, cols, k2 = 5, 4, 0.12
    system = make([rows, cols], k2, 0.0)
    assert system.residual < 1e-5
    f0 = np.array([[-4, 1, 0, 1], [1, 0, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0], [1, 0, 0, 0]]) * k2
    u0 = np.array([[1, 0, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0]], dtype=float)
    for i in range(rows):
        for j in range(cols):
            x = np.roll(np.roll(u0, i, axis=0), j, axis=1)
            system.u = x
            assert np.allclose(system.f_interactions, np.roll(np.roll(f0, i, axis=0), j, axis=1))
            assert np.allclose(system.u, x)


def check_quartic_gradient2d(make):
    rows, cols, k2, k4 = 5, 5, 0.12, 0.34
    system = make([rows, cols], k2, k4)
    assert system.residual < 1e-5
    u0 = np.zeros((5, 5))
    u0[2, 2] = 1
    d2udx2 = np.zeros((5, 5))
    d2udx2[2, 1:4] = [1, -2, 1]
    d2udy2 = d2udx2.T
    dudx = np.zeros((5, 5))
    dudx[2, 1:4] = [0.5, 0, -0.5]
    dudy = dudx.T
    d2udxdy = np.zeros((5, 5))
    f0 = (d2udx2 + d2udy2) * (k2 + k4 / 3) + 2 / 3 * k4 * (
        dudx**2 * d2udx2 + dudy**2 * d2udy2 + 2 * dudx * dudy * d2udxdy
    )
    for i in range(rows):
        for j in range(cols):
            x = np.roll(np.roll(u0, i, axis=0), j, axis=1)
            system.u = x
            assert np.allclose(system.f_interactions, np.roll(np.roll(f0, i, axis=0), j, axis=1))


CHECKS = [
    ("Quartic1d", check_quartic1d),
    ("QuarticGradient1d", check_quartic_gradient1d),
    ("QuarticGradient2d", check_quartic_gradient2d_basic),
    ("QuarticGradient2d", check_quartic_gradient2d),
]


@pytest.mark.parametrize("kind,check", CHECKS)
def test_interactions_oracle(kind, check):
    check(factories()[kind])
