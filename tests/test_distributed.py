"""Replica sharding across ranks, checked with world_size-2 gloo process groups on CPU."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

from ettk_gb300.distributed import average_across_ranks, gather_rows, shard


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


class _SpectrumStandIn:
    """Stand-in for the metric's split average on CPU: each member contributes fixed seeded half spectra
    (acc = |w| B, re = w B x, im = w B y), and finish divides as getImage does where acc > 0."""

    def __init__(self, N=8, members=10):
        rng = np.random.default_rng(3)
        self.N = N
        self.B = rng.random((members, N, N, N // 2 + 1))
        self.X = rng.standard_normal((members, N, N, N // 2 + 1))
        self.Y = rng.standard_normal((members, N, N, N // 2 + 1))

    def average_partial(self, particles, weights, matrices):
        shape = (self.N, self.N, self.N // 2 + 1)
        re, im, acc = np.zeros(shape), np.zeros(shape), np.zeros(shape)
        for p, w in zip(particles, weights):
            acc += abs(w) * self.B[p]
            re += w * self.B[p] * self.X[p]
            im += w * self.B[p] * self.Y[p]
        return re, im, acc

    def average_finish(self, re, im, acc):
        return np.where(acc > 0, re / np.where(acc > 0, acc, 1), 0) + 1j * np.where(acc > 0, im / np.where(acc > 0, acc, 1), 0)


def _avg_worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = _SpectrumStandIn()
    parts = list(range(10))
    weights = [1.0, 0.5, -0.25, 1.0, 0.0, 2.0, 1.0, 0.75, -1.0, 1.0]
    mats = [np.eye(4)] * 10
    avg = average_across_ranks(m, parts, weights, mats, rank, world, dist)
    np.save(out_path % rank, avg)
    dist.barrier()
    dist.destroy_process_group()


def test_average_across_two_ranks(tmp_path):
    """The split average: each of two gloo ranks accumulates its half of the members, the accumulators are summed
    by all_reduce, and every rank finishes the same average as one process accumulating every member."""
    out = str(tmp_path / "avg_%d.npy")
    mp.spawn(_avg_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    m = _SpectrumStandIn()
    weights = [1.0, 0.5, -0.25, 1.0, 0.0, 2.0, 1.0, 0.75, -1.0, 1.0]
    ref = m.average_finish(*m.average_partial(list(range(10)), weights, [np.eye(4)] * 10))
    for r in (0, 1):
        got = np.load(out % r)
        assert np.allclose(got, ref, rtol=1e-12, atol=0)
