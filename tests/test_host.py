"""Host-side logic that needs no GPU: layouts, dump format, synthetic workloads,
sharding."""
import os

import numpy as np

from conftest import abea


def test_struct_sizes():
    t = abea.types
    assert t.EVENT_DTYPE.itemsize == 24
    assert t.MODEL_DTYPE.itemsize == 12
    assert t.SCALINGS_DTYPE.itemsize == 16
    assert t.PAIR_DTYPE.itemsize == 8


def test_flatten_roundtrip():
    from abea_gb300 import synth
    b = synth.make_batch("small", seed=2)
    sub = b.subset([3, 0, 5])
    assert sub.sequence(0) == b.sequence(3)
    assert np.array_equal(sub.read_events(1), b.read_events(0))
    assert sub.read[sub.read_ptr[1] + sub.read_len[1]] == 0  # NUL separator
    assert int(sub.event_ptr[2]) == int(b.n_events[3] + b.n_events[0])


def test_dump_write_read_roundtrip(tmp_path):
    from abea_gb300 import dump, synth
    b = synth.make_batch("small", seed=4, lengths=[300, 450, 700])
    answers = [np.zeros(5, dtype=abea.PAIR_DTYPE) for _ in range(3)]
    dump.write_dump(str(tmp_path), [b], [answers])
    assert dump.n_batches(str(tmp_path)) == 1
    b2, golden = dump.load_batch(os.path.join(str(tmp_path), "0"))
    assert b2.n_reads == 3
    for i in range(3):
        assert b2.sequence(i) == b.sequence(i)
        assert np.array_equal(b2.read_events(i), b.read_events(i))
        assert len(golden[i]) == 5
    assert np.array_equal(b2.model, b.model)


def test_workload_shapes():
    from abea_gb300 import synth
    rng = np.random.default_rng(0)
    lens = synth.read_lengths(rng, "f5c_batch")
    assert 1_300_000 <= lens.sum() < 1_320_000 and lens.min() >= 500 and lens.max() <= 20000
    lens = synth.read_lengths(rng, "uneven")
    assert 1_300_000 <= lens.sum() < 1_400_000 and lens.max() <= 100000
    assert len(synth.read_lengths(rng, "small")) == 64
    assert len(synth.read_lengths(rng, "adjoint")) == 4096


def test_synthetic_events_follow_the_model():
    from abea_gb300 import synth
    b = synth.make_batch("small", seed=9, lengths=[2000])
    ev = b.read_events(0)
    epk = len(ev) / (2000 - 5)
    assert 1.5 < epk < 1.9  # Geometric(mean 1.8) with 5% skipped k-mers
    assert ev["length"].min() >= 3 and ev["length"].max() <= 34
    assert np.all(np.diff(ev["start"].astype(np.int64)) > 0)
