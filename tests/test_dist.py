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


def _adjoint_worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import load_package
    load_package()
    from abea_gb300 import synth
    from abea_gb300.shard import reduce_model_gradient, shard_reads
    from oracle import oracle
    dist.init_process_group("gloo", rank=rank, world_size=world)
    batch = synth.make_batch("small", seed=9, lengths=np.random.default_rng(6).integers(300, 1200, 8))
    gm = np.zeros((4096, 2))
    for i in shard_reads(batch.n_bands(), world, rank):
        seq = bytes(batch.read[batch.read_ptr[i]:batch.read_ptr[i] + batch.read_len[i]])
        ev = batch.events[batch.event_ptr[i]:batch.event_ptr[i] + batch.n_events[i]]
        _, _, info = oracle.align(seq, ev, batch.model, batch.scalings[i], 0)
        gm += oracle.path_adjoint(info["walk"], info["last_from"], seq, ev, batch.model, batch.scalings[i], 0,
                                  want_model=True)[3]
    total = reduce_model_gradient(gm)
    if rank == 0:
        np.save(os.path.join(out_dir, "gm.npy"), total)
    dist.destroy_process_group()


def test_two_rank_model_gradient_reduction(tmp_path, oracle_mod):
    """A sharded adjoint: each rank sums the FP64 model gradient of its reads, one
    all-reduce gives the whole batch's (equal to one process's up to the order of
    the FP64 sums)."""
    world = 2
    mp.start_processes(_adjoint_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    total = np.load(os.path.join(tmp_path, "gm.npy"))
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=9, lengths=np.random.default_rng(6).integers(300, 1200, 8))
    ref = np.zeros((4096, 2))
    for i in range(batch.n_reads):
        seq = bytes(batch.read[batch.read_ptr[i]:batch.read_ptr[i] + batch.read_len[i]])
        ev = batch.events[batch.event_ptr[i]:batch.event_ptr[i] + batch.n_events[i]]
        _, _, info = oracle_mod.align(seq, ev, batch.model, batch.scalings[i], 0)
        ref += oracle_mod.path_adjoint(info["walk"], info["last_from"], seq, ev, batch.model, batch.scalings[i], 0,
                                       want_model=True)[3]
    assert np.count_nonzero(ref) > 0
    assert np.allclose(total, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
