"""Sharding a batch of reads over ranks (one GPU per rank).

Reads are independent, so a multi-GPU run gives every rank its own subset of
reads and no collective touches the data path.  The subsets balance band cells
(the work) by longest-processing-time assignment.
"""
from __future__ import annotations

import numpy as np


def owners(n_bands, world: int) -> np.ndarray:
    """Rank owning each read: reads in decreasing band count, each to the least
    loaded rank (ties to the lowest rank)."""
    n_bands = np.asarray(n_bands, dtype=np.int64)
    order = np.argsort(-n_bands, kind="stable")
    load = np.zeros(world, dtype=np.int64)
    owner = np.zeros(len(n_bands), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += int(n_bands[i])
    return owner


def shard_reads(n_bands, world: int, rank: int) -> np.ndarray:
    """Indices (ascending) of the reads rank `rank` aligns."""
    return np.nonzero(owners(n_bands, world) == rank)[0]


def load_per_rank(n_bands, world: int) -> np.ndarray:
    n_bands = np.asarray(n_bands, dtype=np.int64)
    own = owners(n_bands, world)
    return np.array([int(n_bands[own == r].sum()) for r in range(world)], dtype=np.int64)


def reduce_model_gradient(grad_model):
    """Sums the adjoint's pore-model gradient (4096 x 2 FP64, one per rank's shard)
    over the ranks of the default torch.distributed process group: the one
    collective of a sharded run, 64 KB per batch.  The per-read gradients stay
    with their shard."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(grad_model, dtype=np.float64).copy())
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()
