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
    return 0 if thr >= 2**62 else int(min(np.sum(np.asarray(bands) >= thr), blocks))


def test_one_long_read_among_short_ones_goes_wide():
    """The f5c batch shape: its longest reads bound the batch on the warp shape."""
    from abea_gb300 import synth
    nb = synth.make_batch("f5c_batch", seed=1).n_bands()
    k = n_wide(nb)
    assert 60 <= k <= 130, k   # measured best: 80-100 wide reads (10.19 ms; 11.57 with 50, 39.2 with none)


def test_flat_length_distribution_stays_on_the_warp_shape():
    """1,024 reads of 1-10 kb: wide reads would take whole SMs for little gain
    (measured 24.4 ms with none, 44.6 ms with one per block)."""
    rng = np.random.default_rng(11)
    lens = rng.integers(1000, 10001, 1024)
    nb = lens - 5 + (lens * 1.71).astype(np.int64) + 2
    assert n_wide(nb) == 0
    assert n_wide(np.full(4096, 27000)) == 0


def test_fewer_reads_than_blocks_and_edge_inputs():
    assert n_wide([54382]) == 1                        # one read alone: the wide shape
    assert wide_threshold([]) >= 2**62                 # nothing to do
    assert wide_threshold([10, -1]) == -1              # bad input
    assert wide_threshold([10], blocks=0) == -1
