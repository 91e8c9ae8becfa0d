"""The batched form's wide-shape heuristic (host code, no device): how many of the
longest reads take the 512-thread shape for batch shapes measured on a GB300."""
import ctypes as C
import os

import numpy as np

from conftest import abea


def wide_threshold(bands, blocks=152):
    if not os.path.exists(abea.LIB_PATH):
        abea.build()
    L = abea.lib()
    f = L.abea_internal_wide_threshold
    f.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    f.restype = C.c_int64
    b = np.ascontiguousarray(bands, dtype=np.int64)
    return f(b.ctypes.data, len(b), blocks)


def n_wide(bands, blocks=152):
    thr = wide_threshold(bands, blocks)
    return 0 if thr >= 2**62 else int(np.sum(np.asarray(bands) >= thr))


def test_latency_bound_batch_goes_all_wide():
    """The f5c batch shape: its longest read bounds the batch whatever the split,
    and with every read on the wide shape (the blocks pulling them longest first)
    nothing else is longer (measured 8.46 ms, against 8.49-9.10 ms for the best
    one-wide-read-per-block split and 36.1 ms with none)."""
    from abea_gb300 import synth
    nb = synth.make_batch("f5c_batch", seed=1).n_bands()
    assert n_wide(nb) == len(nb)


def test_few_reads_per_sm_go_all_wide_many_stay_on_the_warp_shape():
    """1,024 reads of 1-10 kb (about 7 per SM): every read wide, 18.5 ms against
    20.8 ms with none.  4,096 such reads (27 per SM): none, 35.5 ms against 68.5
    with every read wide, because 16 warp-shape reads per SM issue more per SM
    than one wide read."""
    rng = np.random.default_rng(11)
    lens = rng.integers(1000, 10001, 1024)
    nb = lens - 5 + (lens * 1.71).astype(np.int64) + 2
    assert n_wide(nb) == 1024
    lens = rng.integers(1000, 10001, 4096)
    nb = lens - 5 + (lens * 1.71).astype(np.int64) + 2
    assert n_wide(nb) == 0
    assert n_wide(np.full(4096, 27000)) == 0


def test_serving_batches_keep_the_split():
    """A serving-stream device batch (about 4,000 reads, lognormal median 8 kb):
    26 reads per SM, not bound by its longest read, so not every read goes wide
    (measured: 1.23 s for the 200 Mbase stream every read wide, 0.99 s split)."""
    rng = np.random.default_rng(5)
    lens = np.clip(rng.lognormal(np.log(8000), 0.6, 3987), 500, 200000).astype(np.int64)
    nb = lens - 5 + (lens * 1.71).astype(np.int64) + 2
    k = n_wide(nb)
    assert 0 <= k < 152, k


def test_fewer_reads_than_blocks_and_edge_inputs():
    assert n_wide([54382]) == 1                        # one read alone: the wide shape
    assert wide_threshold([]) >= 2**62                 # nothing to do
    assert wide_threshold([10, -1]) == -1              # bad input
    assert wide_threshold([10], blocks=0) == -1


def test_checkpointed_reads_keep_the_split():
    """A latency-bound batch with checkpointed reads (trace over the budget): those
    run on the warp shape and would start last behind every wide read, so the
    heuristic keeps at most one wide read per block and never a checkpointed one."""
    if not os.path.exists(abea.LIB_PATH):
        abea.build()
    f = abea.lib().abea_internal_wide_threshold_ck
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]
    f.restype = C.c_int64
    from abea_gb300 import synth
    nb = np.ascontiguousarray(synth.make_batch("f5c_batch", seed=1).n_bands(), dtype=np.int64)
    ck = np.zeros(len(nb), dtype=np.int32)
    assert f(nb.ctypes.data, ck.ctypes.data, len(nb), 152) == 1          # no checkpointed read: every read wide
    ck[np.argsort(-nb)[200:210]] = 1                                     # ten mid-length reads checkpointed
    thr = f(nb.ctypes.data, ck.ctypes.data, len(nb), 152)
    k = int(np.sum((nb >= thr) & (ck == 0)))
    assert thr > 1 and 0 < k < 152, (thr, k)
