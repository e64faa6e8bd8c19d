"""Sharding the batched form over ranks (weak scaling, no collective on the data path), checked with
two gloo ranks on the CPU: every realisation is owned by exactly one rank, the loads are balanced, and
per-realisation results computed on the owning rank (here with the CPU oracle) gather back into the
single-rank answer."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _sizes():
    from frictionqpotspringblock_gb300 import batch as B

    return B.log_uniform_sizes(64, 16, 256, seed=3)


def _result(j, n):
    """One realisation's result: u_frame and well-index sum after one event-driven cycle (CPU oracle)."""
    from oracle import oracle as O

    s = O.line1d("Cuspy", shape=[int(n)], m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / n, dt=0.1,
                 seed=1000 + j, distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-100.0, nchunk=200)
    s.eventDrivenStep(1e-5, False)
    s.eventDrivenStep(1e-5, True)
    s.minimise()
    return s.u_frame, float(np.sum(s.chunk.index_at_align))


def _worker(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from frictionqpotspringblock_gb300 import batch as B

    sizes = _sizes()
    parts = B.partition(sizes, world)
    mine = parts[rank]
    res = np.full((len(sizes), 2), np.nan)
    for j in mine:
        res[j] = _result(int(j), int(sizes[j]))
    t = torch.from_numpy(res)
    gathered = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(gathered, t)  # only to collect the answer for the check, not part of the work
    if rank == 0:
        merged = np.full_like(res, np.nan)
        for r, g in enumerate(gathered):
            merged[parts[r]] = g.numpy()[parts[r]]
        np.save(out_path, merged)
    dist.destroy_process_group()


def test_partition_properties():
    from frictionqpotspringblock_gb300 import batch as B

    sizes = B.log_uniform_sizes(4096, 256, 65536, seed=3)
    for world in (1, 2, 3, 8):
        parts = B.partition(sizes, world)
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(len(sizes)))
        loads = np.array([sizes[p].sum() for p in parts])
        assert loads.max() - loads.min() <= sizes.max()


def test_two_gloo_ranks_match_one(tmp_path):
    out = tmp_path / "merged.npy"
    mp.start_processes(_worker, args=(2, _free_port(), str(out)), nprocs=2, join=True, start_method="spawn")
    merged = np.load(out)
    sizes = _sizes()
    ref = np.array([_result(j, int(n)) for j, n in enumerate(sizes)])
    assert np.array_equal(merged, ref)
