"""f5c's calling pattern for the drop-in align(): one read per call from many
host threads at once (GPU/f5c.h:57-59).  Every thread's results must equal the
oracle's, and the reference's golden pairs for the dump subset."""
import concurrent.futures as cf
import os

import numpy as np
import pytest

from conftest import abea

pytestmark = pytest.mark.gpu


def test_align_from_eight_threads_on_the_golden_subset(dump_subset):
    batch, golden = dump_subset
    idx = list(range(batch.n_reads)) * 4  # every read several times, interleaved over the threads

    def one(i):
        return i, abea.align(batch.sequence(i), batch.read_events(i), batch.model, batch.scalings[i])
    with cf.ThreadPoolExecutor(8) as ex:
        for i, got in ex.map(one, idx):
            assert np.array_equal(got, golden[i]), i


def test_align_from_eight_threads_on_synthetic_reads(oracle_mod):
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=31, lengths=np.random.default_rng(5).integers(500, 6000, 48))
    op, oc, _ = oracle_mod.align_batch(batch, threads=os.cpu_count())
    exp = abea.split_pairs(batch, op, oc)

    def one(i):
        return i, abea.align(batch.sequence(i), batch.read_events(i), batch.model, batch.scalings[i])
    with cf.ThreadPoolExecutor(8) as ex:
        results = dict(ex.map(one, range(batch.n_reads)))
    for i in range(batch.n_reads):
        assert np.array_equal(results[i], exp[i]), i
