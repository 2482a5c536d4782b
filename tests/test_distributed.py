"""Replica sharding across ranks, checked with world_size-2 gloo process groups on CPU."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

from ettk_gb300.distributed import gather_rows, shard


def test_shard_covers_everything():
    for n in (0, 1, 7, 200, 2001):
        for w in (1, 2, 3, 8):
            parts = [shard(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(w - 1))
            sizes = [e - s for s, e in parts]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s, e = shard(n, rank, world)
    # each rank "aligns" its share: rows carry the global pair index so the gather order is checkable
    D = np.zeros((e - s, 17, 1), np.float32)
    D[:, 0, 0] = np.arange(s, e)
    D[:, 1:, 0] = rank
    full = gather_rows(D, n, rank, world, dist)
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_gather_two_ranks(tmp_path):
    n = 11
    out = str(tmp_path / "D.npy")
    mp.spawn(_worker, args=(2, _free_port(), n, out), nprocs=2, join=True)
    D = np.load(out)
    assert D.shape == (n, 17, 1)
    assert np.array_equal(D[:, 0, 0], np.arange(n))
    s1, _ = shard(n, 1, 2)
    assert (D[:s1, 1:, 0] == 0).all() and (D[s1:, 1:, 0] == 1).all()
