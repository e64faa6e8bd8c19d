"""Batched form against the plain path, realisation by realisation.

Each realisation of the batch must follow the plain path's trajectory bit for bit: the same u_frame,
mean f_frame, avalanche size S and increment after every quasistatic cycle, and the same final
positions and well indices as `Line1d.System_Cuspy_Laplace` driven by eventDrivenStep(eps, False),
eventDrivenStep(eps, True), minimise() (the plain path itself is checked against the CPU oracle in
test_gpu_parity.py).  The batch keeps a small chunk window per particle; the second case makes
particles cross many windows so the batch's regeneration branch runs.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")
from frictionqpotspringblock_gb300 import _capi  # noqa: E402
from frictionqpotspringblock_gb300 import batch as B  # noqa: E402

COMMON = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, dt=0.1, distribution="weibull",
              parameters=[2.0, 1.0, 1e-5], offset=-20.0)


def plain_cycles(n, seed, k_frame, nchunk, ncycles, eps, tol=1e-5):
    s = fqsb.Line1d.System_Cuspy_Laplace(k_frame=k_frame, shape=[n], seed=seed, nchunk=nchunk, **COMMON)
    rec = {"u_frame": [], "f_frame": [], "S": [], "inc": []}
    for _ in range(ncycles):
        i_n = s.chunk.index_at_align
        s.eventDrivenStep(eps, False)
        s.eventDrivenStep(eps, True)
        assert s.minimise(tol=tol, max_iter=2000000) == 0
        rec["u_frame"].append(s.u_frame)
        rec["f_frame"].append(s._scalar(_capi.SCALAR_MEAN_F_FRAME))
        rec["S"].append(int(np.sum(s.chunk.index_at_align - i_n)))
        rec["inc"].append(s.inc)
    return s, rec


def check_batch(sizes, nchunk, window, ncycles, eps, threads=0, ppt=0):
    seeds = 1000 + np.arange(len(sizes))
    kf = 1.0 / np.asarray(sizes, dtype=float)
    b = B.Line1d_System_Cuspy_Laplace(sizes, seeds, kf, nchunk=nchunk, window=window, threads=threads, ppt=ppt,
                                      **COMMON)
    out = b.quasistatic(ncycles, eps, max_iter=2000000)
    assert np.all(out["status"] == 0)
    for j, n in enumerate(sizes):
        s, rec = plain_cycles(int(n), int(seeds[j]), float(kf[j]), nchunk, ncycles, eps)
        assert np.array_equal(out["u_frame"][j], rec["u_frame"]), j
        assert np.array_equal(out["f_frame"][j], rec["f_frame"]), j
        assert np.array_equal(out["S"][j], rec["S"]), j
        assert np.array_equal(out["inc"][j], rec["inc"]), j
        assert np.array_equal(b.field(j, "u"), s.u), j
        assert np.array_equal(b.field(j, "v"), s.v), j
        assert np.array_equal(b.index_at_align(j), s.chunk.index_at_align), j
    return out


@pytest.mark.parametrize("threads,ppt", [(256, 1), (128, 2), (64, 1)])
def test_batch_matches_plain(threads, ppt):
    sizes = [3, 7, 64, 100, 256, 257, 511, 1000, 1500, 4096]
    check_batch(sizes, nchunk=200, window=48, ncycles=4, eps=1e-3, threads=threads, ppt=ppt)


def test_batch_regeneration():
    """eps = 0.3 kicks move every particle ~1 well per cycle; a 34-position window moves every ~2 wells."""
    out = check_batch([5, 40, 300, 700], nchunk=100, window=34, ncycles=14, eps=0.3)
    assert out["S"].sum() > 0


def test_batch_uneven_many():
    sizes = B.log_uniform_sizes(64, 8, 2048, seed=3)
    check_batch(list(sizes[:12]), nchunk=300, window=64, ncycles=3, eps=1e-3)
    b = B.Line1d_System_Cuspy_Laplace(sizes, 1000 + np.arange(64), 1.0 / sizes, nchunk=300, window=64, **COMMON)
    out = b.quasistatic(3, 1e-3, max_iter=2000000)
    assert np.all(out["status"] == 0)
    assert np.all(np.diff(out["inc"], axis=1) > 0)


def test_autotune_picks_a_candidate(tmp_path, monkeypatch):
    from frictionqpotspringblock_gb300 import autotune

    monkeypatch.setattr(autotune, "CACHE", tmp_path / "tune.json")
    sizes = B.log_uniform_sizes(48, 16, 1024, seed=3)

    def make(sub, threads, ppt):
        return B.Line1d_System_Cuspy_Laplace(sub, 1000 + np.arange(len(sub)), 1.0 / sub, nchunk=200, window=48,
                                             threads=threads, ppt=ppt, **COMMON)

    best = autotune.choose_tile(sizes, make, sample=16, cycles=1)
    assert tuple(best) in autotune.CANDIDATES
    assert autotune.choose_tile(sizes, make) == tuple(best)  # cached


def test_batch_host_driven(monkeypatch):
    """FQSB_NO_GRAPH=1 at creation: the batch's passes are launched one by one from the host (the form
    profilers can see); results equal the graph form's bit for bit, window moves included."""
    sizes = B.log_uniform_sizes(24, 8, 1024, seed=3)
    seeds = 1000 + np.arange(len(sizes))
    out = []
    for ng in ("0", "1"):
        monkeypatch.setenv("FQSB_NO_GRAPH", ng)
        b = B.Line1d_System_Cuspy_Laplace(sizes, seeds, 1.0 / sizes, nchunk=100, window=34, **COMMON)
        monkeypatch.delenv("FQSB_NO_GRAPH")
        out.append(b.quasistatic(6, 0.3, max_iter=2000000))
        out[-1]["u"] = np.concatenate([b.field(j, "u") for j in range(len(sizes))])
        del b
    for k in ("u_frame", "f_frame", "S", "inc", "status", "u"):
        assert np.array_equal(out[0][k], out[1][k]), k
