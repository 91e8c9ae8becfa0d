"""Serving stream (`abea_align_stream`): reads admitted in order into device
batches by footprint, two batches in flight, optional adjoint + Gauss-Newton
step + re-alignment per batch.  The results must not depend on how the reads
were cut into batches."""
import numpy as np
import pytest

from conftest import abea


def with_scalings(batch, sc):
    from abea_gb300.types import Batch
    return Batch(read=batch.read, read_ptr=batch.read_ptr, read_len=batch.read_len, events=batch.events,
                 event_ptr=batch.event_ptr, n_events=batch.n_events, scalings=np.ascontiguousarray(sc),
                 model=batch.model, meta=dict(batch.meta))


def footprint(batch):
    """Rough device bytes of the whole batch (trace dominates: 128 B per band)."""
    return int(batch.n_bands().sum()) * 160 + int(batch.n_events.sum()) * 48


def test_stream_generator_is_deterministic_and_follows_the_laws():
    from abea_gb300 import synth
    a = synth.make_stream(seed=3, total_bases=2_000_000, threads=1)
    b = synth.make_stream(seed=3, total_bases=2_000_000, threads=4)
    assert np.array_equal(a.read, b.read) and np.array_equal(a.events, b.events)
    assert a.read_len.sum() >= 2_000_000 and a.read_len.min() >= 500 and a.read_len.max() <= 200_000
    ratio = a.n_events.sum() / (a.read_len - 5).sum()
    assert abs(ratio - 1.8 * 0.95) < 0.02
    assert np.array_equal(a.event_ptr[1:], np.cumsum(a.n_events)[:-1])
    # each read's first event starts at sample 0; lengths in [3, 34]
    assert np.all(a.events["start"][a.event_ptr] == 0)
    assert a.events["length"].min() >= 3 and a.events["length"].max() <= 34
    # event means follow the read's scaled levels of its own k-mers
    i = 7
    ranks = synth.kmer_ranks(np.frombuffer(a.sequence(i), dtype=np.uint8))
    lv = a.model["level_mean"][ranks] * a.scalings["scale"][i] + a.scalings["shift"][i]
    ev = a.events["mean"][a.event_ptr[i]:a.event_ptr[i] + a.n_events[i]]
    assert abs(np.mean(ev) - np.mean(lv)) < 1.0


def test_stream_rejects_bad_arguments_without_a_device():
    if not __import__("os").path.exists(abea.LIB_PATH):
        abea.build()
    L = abea.lib()
    assert L.abea_align_stream(None, None, 0, *([None] * 13)) == -1


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
def test_stream_over_several_batches_matches_the_oracle(oracle_mod, mode):
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=21)
    ctx = abea.Context(0, mode)
    r = ctx.align_stream(batch, batch_bytes=footprint(batch) // 6)
    assert r["stats"]["n_batches"] >= 4
    assert r["stats"]["band_cells"] == batch.band_cells()
    op, oc, _ = oracle_mod.align_batch(batch)
    assert np.array_equal(r["counts"], oc)
    for x, y in zip(abea.split_pairs(batch, r["pairs"], r["counts"]), abea.split_pairs(batch, op, oc)):
        assert np.array_equal(x, y)
    assert np.all(r["latency_ms"] > 0)
    assert np.array_equal(r["scalings"], batch.scalings)
    # the same call again (device batches reused) and one batch for everything
    r2 = ctx.align_stream(batch, batch_bytes=footprint(batch) // 6)
    r3 = ctx.align_stream(batch)
    assert r3["stats"]["n_batches"] == 1
    for rr in (r2, r3):
        assert np.array_equal(rr["counts"], oc)
        for x, y in zip(abea.split_pairs(batch, rr["pairs"], rr["counts"]), abea.split_pairs(batch, op, oc)):
            assert np.array_equal(x, y)


@pytest.mark.gpu
def test_stream_with_edge_case_reads_equals_align_batch(ref_synthetic):
    """Tiny reads, reads with few events and paths over their output slot, cut
    into batches of a read or two."""
    batch = ref_synthetic[0]
    ctx = abea.Context(0, abea.MODE_BATCHED)
    pairs, counts = ctx.align_batch(batch)
    r = ctx.align_stream(batch, batch_bytes=1)  # every read is a batch of its own
    assert r["stats"]["n_batches"] == batch.n_reads
    assert np.array_equal(r["counts"], counts)
    for x, y in zip(abea.split_pairs(batch, r["pairs"], r["counts"]), abea.split_pairs(batch, pairs, counts)):
        assert np.array_equal(x, y)


@pytest.mark.gpu
def test_stream_recalibration_step_equals_one_gauss_newton_round(oracle_mod):
    """Per batch: align, adjoint, one Gauss-Newton step, re-align.  Each read's
    step depends on its own path only, so the stream's result equals one round of
    abea_batch_recalibrate over the whole batch, and its AlignedPairs are the
    oracle's for the new scalings."""
    from abea_gb300 import synth
    rng = np.random.default_rng(5)
    batch = synth.make_batch("adjoint", seed=23, perturb=True, lengths=rng.integers(1000, 6001, 48))
    ctx = abea.Context(0, abea.MODE_BATCHED)
    r = ctx.align_stream(batch, batch_bytes=footprint(batch) // 5, recalibrate=True)
    assert r["stats"]["n_batches"] >= 3
    dev = ctx.upload(batch)
    fit = dev.recalibrate(1, first_temperature=1.0)
    assert np.array_equal(r["scalings"].view(np.uint32), fit.view(np.uint32))
    bp, bc = dev.results()
    assert np.array_equal(r["counts"], bc)
    moved = np.abs(r["scalings"]["shift"] - batch.scalings["shift"]) > 0
    assert moved.mean() > 0.5
    op, oc, _ = oracle_mod.align_batch(with_scalings(batch, r["scalings"]))
    assert np.array_equal(r["counts"], oc)
    for x, y in zip(abea.split_pairs(batch, r["pairs"], r["counts"]), abea.split_pairs(batch, op, oc)):
        assert np.array_equal(x, y)


@pytest.mark.gpu
def test_stream_workload_batched_equals_plain():
    """A 6 Mbase slice of the serving workload in ~1.5 Mbase device batches:
    both forms give the same AlignedPairs and the same recalibrated scalings."""
    from abea_gb300 import synth
    batch = synth.make_stream(seed=2, total_bases=6_000_000)
    out = {}
    for mode in (abea.MODE_BATCHED, abea.MODE_PLAIN):
        ctx = abea.Context(0, mode)
        out[mode] = ctx.align_stream(batch, batch_bytes=footprint(batch) // 4, recalibrate=True)
        ctx.close()
    a, b = out[abea.MODE_BATCHED], out[abea.MODE_PLAIN]
    assert a["stats"]["n_batches"] >= 4
    assert np.array_equal(a["counts"], b["counts"])
    assert np.array_equal(a["scalings"].view(np.uint32), b["scalings"].view(np.uint32))
    for x, y in zip(abea.split_pairs(batch, a["pairs"], a["counts"]), abea.split_pairs(batch, b["pairs"], b["counts"])):
        assert np.array_equal(x, y)
