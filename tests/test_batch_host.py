"""Host-side pieces of the batched form (no GPU): the realisation-size stream and its statistics."""

import numpy as np

from frictionqpotspringblock_gb300 import batch as B
from oracle import oracle as O


def test_pcg32_uniform_matches_oracle_stream():
    u = B.pcg32_uniform(3, 50)
    ref = O.pcg32_stream(3, 0, 50).astype(np.float64) * 2.0 ** -32
    assert np.array_equal(u, ref)


def test_log_uniform_sizes_statistics():
    s = B.log_uniform_sizes(4096, 256, 65536, seed=3)
    assert s.min() >= 256 and s.max() <= 65536
    # E[N] = (65536 - 256) / ln(256) = 11773: the 4096 realisations hold ~4.8e7 particles
    assert 4.3e7 < s.sum() < 5.3e7
