"""The batched form sharded over two ranks (gloo, both on cuda:0): each rank runs its part of the
realisations (batch.quasistatic_shard) as its own GPU batch with no exchange while running; the results
gathered by realisation index equal one batch of all realisations bit for bit.  The two ranks' kernels
never wait on each other (independent batches on one GPU)."""

import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")
mp = pytest.importorskip("torch.multiprocessing")

COMMON = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, dt=0.1, distribution="weibull",
              parameters=[2.0, 1.0, 1e-5], offset=-100.0, nchunk=400, window=48)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _sizes():
    from frictionqpotspringblock_gb300 import batch as B

    return B.log_uniform_sizes(96, 64, 4096, seed=3)


def _worker(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from frictionqpotspringblock_gb300 import batch as B

    sizes = _sizes()
    idx, out = B.quasistatic_shard(sizes, 1000 + np.arange(len(sizes)), 1.0 / sizes, rank, world, 2, 1e-5, **COMMON)
    gathered = [None] * world
    dist.all_gather_object(gathered, (idx, out))
    if rank == 0:
        merged = {k: np.zeros((len(sizes),) + v.shape[1:], v.dtype) for k, v in out.items()}
        seen = np.zeros(len(sizes), int)
        for i, o in gathered:
            for k in merged:
                merged[k][i] = o[k]
            seen[i] += 1
        assert np.all(seen == 1)
        np.savez(out_path, **merged)
    dist.destroy_process_group()


def test_two_ranks_match_one_batch(tmp_path):
    from frictionqpotspringblock_gb300 import batch as B

    out = tmp_path / "merged.npz"
    mp.start_processes(_worker, args=(2, _free_port(), str(out)), nprocs=2, join=True, start_method="spawn")
    merged = np.load(out)
    sizes = _sizes()
    kw = {k: v for k, v in COMMON.items()}
    b = B.Line1d_System_Cuspy_Laplace(sizes, 1000 + np.arange(len(sizes)), 1.0 / sizes, **kw)
    ref = b.quasistatic(2, 1e-5)
    for k in ("u_frame", "f_frame", "S", "inc", "status"):
        assert np.array_equal(merged[k], ref[k]), k
