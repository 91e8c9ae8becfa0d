"""Parity at the benchmark configurations' full sizes, through properties that do
not need the CPU oracle to run the whole workload: the batched and plain forms
agree exactly (AlignedPairs, gradients, recalibrated scalings), and a slice of
each workload matches the oracle."""
import os

import numpy as np
import pytest

from conftest import abea

pytestmark = pytest.mark.gpu


def same_pairs(batch, a_pairs, a_counts, b_pairs, b_counts):
    assert np.array_equal(a_counts, b_counts)
    for x, y in zip(abea.split_pairs(batch, a_pairs, a_counts), abea.split_pairs(batch, b_pairs, b_counts)):
        assert np.array_equal(x, y)


def test_adjoint_workload_forms_agree_with_checkpoints(oracle_mod):
    """4,096 reads of 1-10 kb with perturbed scalings, var-aware emissions and reads
    over 8 kb checkpointed: both forms give the same AlignedPairs and the same FP64
    gradients; 48 reads checked against the oracle in parity mode."""
    from abea_gb300 import synth
    batch = synth.make_batch("adjoint", seed=1, perturb=True)
    budget = (8000 + int(8000 * 1.71) + 2) * 128
    out = {}
    for mode in (abea.MODE_BATCHED, abea.MODE_PLAIN):
        ctx = abea.Context(0, mode)
        ctx.set_option(abea.OPT_VAR_AWARE, 1)
        ctx.set_option(abea.OPT_TRACE_BUDGET, budget)
        dev = ctx.upload(batch)
        dev.run()
        pairs, counts = dev.results()
        out[mode] = (pairs, counts, dev.backward())
    (p1, c1, g1), (p2, c2, g2) = out[abea.MODE_BATCHED], out[abea.MODE_PLAIN]
    same_pairs(batch, p1, c1, p2, c2)
    for key in ("grad_scalings", "path_emission", "status"):
        assert np.array_equal(g1[key], g2[key]), key
    # the model gradient sums the reads' terms with FP64 atomics: equal up to the order of the sum
    gm1, gm2 = g1["grad_model"], g2["grad_model"]
    assert np.allclose(gm1, gm2, rtol=1e-10, atol=1e-10 * np.abs(gm1).max())
    # parity mode on a slice, against the oracle
    sub = batch.subset(range(0, batch.n_reads, batch.n_reads // 48)[:48])
    gp, gc = abea.Context(0, abea.MODE_BATCHED).align_batch(sub)
    op, oc, _ = oracle_mod.align_batch(sub, threads=os.cpu_count())
    same_pairs(sub, gp, gc, op, oc)


def test_serving_stream_full_size_forms_agree():
    """200 Mbases of reads through the serving stream with the recalibration step:
    both forms give the same AlignedPairs and the same recalibrated scalings, in
    device batches sized by the default footprint limit."""
    from abea_gb300 import synth
    batch = synth.make_stream(seed=5, total_bases=200_000_000)
    pb = abea.pin_batch(batch)
    res = {}
    for mode in (abea.MODE_BATCHED, abea.MODE_PLAIN):
        ctx = abea.Context(0, mode)
        pairs = abea.pinned_empty(max(batch.pair_capacity(), 1), abea.types.PAIR_DTYPE)
        counts = abea.pinned_empty(batch.n_reads, np.int32)
        r = ctx.align_stream(pb, recalibrate=True, out_pairs=pairs, out_counts=counts)
        ctx.close()
        assert r["stats"]["n_batches"] >= 2
        assert r["stats"]["band_cells"] == batch.band_cells()
        assert np.all(r["latency_ms"] > 0)
        res[mode] = (pairs, r["counts"].copy(), r["scalings"].copy())
    (p1, c1, s1), (p2, c2, s2) = res[abea.MODE_BATCHED], res[abea.MODE_PLAIN]
    assert np.array_equal(s1.view(np.uint32), s2.view(np.uint32))
    same_pairs(batch, p1, c1, p2, c2)
    # the step moved the scalings towards the generating ones
    true = batch.meta["true_scalings"]
    assert np.median(np.abs(s1["shift"] - true["shift"])) < 0.5


def test_exact_against_the_oracle_over_a_billion_band_cells(oracle_mod):
    """The exact FP32 evaluation of the reference's double arithmetic, checked on
    more than 10^9 band cells: the reads1024 workload (1,024 reads of 1-10 kb,
    1.5x10^9 band cells) in the batched form against the CPU oracle on all host
    cores: AlignedPairs and best-end scores bit-exact."""
    from abea_gb300 import synth
    batch = synth.make_batch("reads1024", seed=2)
    assert batch.band_cells() > 10**9
    ctx = abea.Context(0, abea.MODE_BATCHED)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    best = dev.best_scores()
    op, oc, obest = oracle_mod.align_batch(batch, threads=os.cpu_count())
    same_pairs(batch, gp, gc, op, oc)
    assert np.array_equal(best.view(np.uint32), np.asarray(obest, dtype=np.float32).view(np.uint32))
