"""Multi-rank path on CPU: world size 2 over gloo.  Each rank aligns its shard of
a batch with the CPU oracle (the GPU library does the same per rank on its own
GPU); the gathered results must equal the single-process run, the shards must
partition the reads, and the band-cell loads must balance."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, abea

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import load_package
    load_package()
    from abea_gb300 import synth
    from abea_gb300.shard import shard_reads
    from oracle import oracle
    dist.init_process_group("gloo", rank=rank, world_size=world)
    batch = synth.make_batch("small", seed=21, lengths=np.random.default_rng(4).integers(300, 1500, 10))
    mine = shard_reads(batch.n_bands(), world, rank)
    sub = batch.subset(mine)
    pairs, counts, best = oracle.align_batch(sub, threads=1)
    from abea_gb300.types import split_pairs
    per = split_pairs(sub, pairs, counts)
    result = {int(i): (int(c), p.tobytes(), float(b)) for i, c, p, b in zip(mine, counts, per, best)}
    gathered = [None] * world
    dist.all_gather_object(gathered, result)
    t = torch.tensor([float(sub.band_cells())], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    if rank == 0:
        merged = {}
        for g in gathered:
            assert not (set(g) & set(merged)), "shards overlap"
            merged.update(g)
        np.save(os.path.join(out_dir, "merged.npy"), np.array([merged, float(t.item())], dtype=object),
                allow_pickle=True)
    dist.destroy_process_group()


def test_two_rank_sharding_matches_single_process(tmp_path, oracle_mod):
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    merged, cells = np.load(os.path.join(tmp_path, "merged.npy"), allow_pickle=True)
    from abea_gb300 import synth
    from abea_gb300.types import split_pairs
    batch = synth.make_batch("small", seed=21, lengths=np.random.default_rng(4).integers(300, 1500, 10))
    pairs, counts, best = oracle_mod.align_batch(batch, threads=2)
    per = split_pairs(batch, pairs, counts)
    assert sorted(merged) == list(range(batch.n_reads))
    assert cells == float(batch.band_cells())
    for i in range(batch.n_reads):
        c, pb, b = merged[i]
        assert c == counts[i]
        assert pb == per[i].tobytes()
        assert b == float(best[i])


def test_shards_balance_band_cells():
    from abea_gb300 import synth
    from abea_gb300.shard import load_per_rank, shard_reads
    batch = synth.make_batch("uneven", seed=3)
    nb = batch.n_bands()
    for world in (2, 4, 8):
        parts = [shard_reads(nb, world, r) for r in range(world)]
        assert sorted(np.concatenate(parts).tolist()) == list(range(batch.n_reads))
        load = load_per_rank(nb, world)
        # LPT: no rank exceeds the mean by more than the longest read
        assert load.max() <= load.mean() + nb.max()
