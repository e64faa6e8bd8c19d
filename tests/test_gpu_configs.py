"""The benchmark configurations at their own sizes, on the GPU.

* The 2048 x 2048 Line2d System_Cuspy_Laplace grid (eta = 0.2, 500 yield positions per site, pcg32
  seed 2): construction, one quasistatic cycle and a regeneration sweep against the CPU oracle (its
  OpenMP build, same results as the single-threaded one), bit for bit.
* The 4096-realisation batch: a random slice of 256 realisations of the real size list (N_j
  log-uniform in [256, 65536], seeds 1000 + j), two quasistatic cycles in the batched form against
  looping the plain path, bit for bit.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")
from frictionqpotspringblock_gb300 import _capi  # noqa: E402
from frictionqpotspringblock_gb300 import batch as B  # noqa: E402

FIELDS = ["u", "v", "a", "f", "f_potential", "f_interactions", "f_frame", "f_damping"]


def assert_fields(gpu, ref):
    for name in FIELDS:
        g, r = getattr(gpu, name), getattr(ref, name)
        assert np.array_equal(g, r), (name, float(np.max(np.abs(g - r))))
    assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align)
    assert np.array_equal(gpu.chunk.left_of_align, ref.chunk.left_of_align)
    assert np.array_equal(gpu.chunk.right_of_align, ref.chunk.right_of_align)
    assert gpu.inc == ref.inc
    assert gpu.u_frame == ref.u_frame
    assert gpu.residual == ref.residual


@pytest.mark.timeout(1800)
def test_line2d_2048():
    side = 2048
    n = side * side
    par = dict(m=1.0, eta=0.2, mu=1.0, k_interactions=1.0, k_frame=1.0 / n, dt=0.1, shape=[side, side], seed=2,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-100.0, nchunk=500)
    gpu = fqsb.Line2d.System_Cuspy_Laplace(**par)
    ref = O.line2d(**par, sum_mode=O.SUM_PAIRWISE, math_mode=O.MATH_PORTABLE, threads=True)
    assert_fields(gpu, ref)
    rng = np.random.default_rng(2)
    sample = [int(p) for p in rng.integers(0, n, 24)] + [0, n - 1]
    # one quasistatic cycle (eventDrivenStep(1e-5, False), eventDrivenStep(1e-5, True), minimise)
    for kick in (False, True):
        assert gpu.eventDrivenStep(1e-5, kick) == ref.eventDrivenStep(1e-5, kick)
    assert gpu.minimise(max_iter=20000, max_iter_is_error=False) == ref.minimise(max_iter=20000,
                                                                                   max_iter_is_error=False)
    assert_fields(gpu, ref)
    # regeneration sweep: every site crosses ~680 wells forward, then back
    u = gpu.u
    for shift in (600.0, 0.0):
        gpu.u = u + shift
        ref.u = u + shift
        assert_fields(gpu, ref)
        idx, left = gpu.chunk.index_at_align.ravel(), gpu.chunk.left_of_align.ravel()
        for p in sample:
            y = O.sequence(2, p, "weibull", [2.0, 1.0, 1e-5], -100.0, 500, int(idx[p]), 1)
            assert left[p] == y[0], (shift, p)


@pytest.mark.timeout(1800)
def test_batched_slice_of_4096():
    sizes = B.log_uniform_sizes(4096, 256, 65536, seed=3)
    pick = np.sort(np.random.default_rng(5).choice(4096, 256, replace=False))
    sz = sizes[pick]
    seeds = 1000 + pick
    common = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, dt=0.1, distribution="weibull",
                  parameters=[2.0, 1.0, 1e-5], offset=-100.0)
    b = B.Line1d_System_Cuspy_Laplace(sz, seeds, 1.0 / sz, nchunk=1000, window=64, **common)
    ncycles = 2
    out = b.quasistatic(ncycles, 1e-5)
    assert np.all(out["status"] == 0)
    for j in range(len(sz)):
        s = fqsb.Line1d.System_Cuspy_Laplace(k_frame=1.0 / float(sz[j]), shape=[int(sz[j])], seed=int(seeds[j]),
                                             nchunk=1000, **common)
        for c in range(ncycles):
            i_n = s.chunk.index_at_align
            s.eventDrivenStep(1e-5, False)
            s.eventDrivenStep(1e-5, True)
            assert s.minimise() == 0
            assert out["u_frame"][j, c] == s.u_frame, (j, c)
            assert out["f_frame"][j, c] == s._scalar(_capi.SCALAR_MEAN_F_FRAME), (j, c)
            assert out["S"][j, c] == int(np.sum(s.chunk.index_at_align - i_n)), (j, c)
            assert out["inc"][j, c] == s.inc, (j, c)
        assert np.array_equal(b.index_at_align(j), s.chunk.index_at_align), j
        assert np.array_equal(b.field(j, "u"), s.u), j
        del s
