"""Replica sharding of alignment pairs across ranks (one GPU per rank).

The reference distributes (reference, particle) pairs to MPI workers in bundles
(inc/em/nbfCorrelationImageMetric.h:2010-2282); pairs are independent, so here every rank aligns
a disjoint, contiguous share of the pair list on its own GPU and rank 0 gathers the result rows
(torch.distributed point-to-point of the small D rows; no collective on the data path).
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
