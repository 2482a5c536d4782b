"""Replica sharding across ranks (one GPU per rank).

The reference distributes (reference, particle) pairs to MPI workers in bundles
(inc/em/nbfCorrelationImageMetric.h:2010-2282); pairs are independent, so here every rank aligns
a disjoint, contiguous share of the pair list on its own GPU and rank 0 gathers the result rows
(torch.distributed point-to-point of the small D rows; no collective on the data path).

Class averages are the one place with an exchange: each rank accumulates its share of the members
(getImageMPI's three half-spectrum accumulators) and one sum across ranks precedes the average
(getImage), the reduction the reference performs over MPI (inc/em/nbfWedgedAverageImage3D.h:216-356).
"""
import numpy as np


def shard(n_pairs, rank, world):
    """Contiguous [start, stop) share of n_pairs for `rank` (sizes differ by at most one)."""
    base, extra = divmod(n_pairs, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_rows(D_local, n_pairs, rank, world, dist):
    """Assemble the full D (n_pairs, cols, ncand) on rank 0 from every rank's share; returns None elsewhere."""
    cols, ncand = D_local.shape[1], D_local.shape[2]
    if rank == 0:
        D = np.empty((n_pairs, cols, ncand), np.float32)
        s, e = shard(n_pairs, 0, world)
        D[s:e] = D_local
        import torch
        for r in range(1, world):
            s, e = shard(n_pairs, r, world)
            buf = torch.empty((e - s, cols, ncand), dtype=torch.float32)
            if e > s:
                dist.recv(buf, src=r)
            D[s:e] = buf.numpy()
        return D
    import torch
    if D_local.shape[0]:
        dist.send(torch.from_numpy(np.ascontiguousarray(D_local, np.float32)), dst=0)
    return None


def average_across_ranks(metric, particles, weights, matrices, rank, world, dist):
    """Class average of members spread over the ranks: this rank's contiguous share of (particles, weights,
    matrices) accumulated by metric.average_partial, the three accumulators summed over the ranks
    (dist.all_reduce), and the average finished on every rank by metric.average_finish."""
    import torch
    s, e = shard(len(particles), rank, world)
    parts = metric.average_partial(list(particles[s:e]), list(weights[s:e]), list(matrices[s:e]))
    summed = []
    for a in parts:
        t = torch.from_numpy(np.ascontiguousarray(a, np.float64))
        if dist.get_backend() == "nccl":  # NCCL reduces device tensors
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        summed.append(t.cpu().numpy())
    return metric.average_finish(*summed)
