"""Band-score checkpoints (ABEA_OPT_TRACE_BUDGET): reads whose trace exceeds the
budget keep checkpoints every 256 bands instead, and their traceback recomputes
the trace segment by segment.  Results must not change at all."""
import numpy as np
import pytest

from conftest import abea

pytestmark = pytest.mark.gpu

BYTES_PER_BAND = 128  # trace bytes per band (one byte per slot)


def align(batch, mode, budget, scores=False):
    ctx = abea.Context(0, mode, store_scores=scores)
    ctx.set_option(abea.OPT_TRACE_BUDGET, budget)
    dev = ctx.upload(batch)
    dev.run()
    pairs, counts = dev.results()
    return ctx, dev, pairs, counts


def same_alignments(batch, p1, c1, p2, c2):
    assert np.array_equal(c1, c2)
    for x, y in zip(abea.split_pairs(batch, p1, c1), abea.split_pairs(batch, p2, c2)):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
def test_checkpointed_reads_match_the_oracle(oracle_mod, mode):
    """A budget that splits the batch: reads over ~5,400 bands checkpointed."""
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=3)
    budget = 5400 * BYTES_PER_BAND
    n_ck = int(np.sum(((batch.n_bands() + 3) // 4) * 4 * BYTES_PER_BAND > budget))
    assert 0 < n_ck < batch.n_reads
    _, dev, gp, gc = align(batch, mode, budget)
    op, oc, obest = oracle_mod.align_batch(batch)
    same_alignments(batch, gp, gc, op, oc)
    assert np.array_equal(dev.best_scores().view(np.uint32), obest.view(np.uint32))


@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
def test_every_read_checkpointed_on_the_edge_cases(ref_synthetic, mode):
    """Budget of one byte: every read recomputes its trace, including tiny reads,
    paths that outgrow their output slot (tiny_20_5, few_events_400: the QC sum
    then needs a second recomputed walk) and reads over several segments."""
    batch, names, counts, pairs, _ = ref_synthetic
    _, dev, gp, gc = align(batch, mode, 1)
    assert np.array_equal(gc, counts)
    got = abea.split_pairs(batch, gp, gc)
    for i, name in enumerate(names):
        assert np.array_equal(got[i], pairs[i]), name
    # the trace is not kept, the band origins and scores are
    with pytest.raises(abea.AbeaError):
        dev.read_bands(len(names) - 1)


def test_checkpoints_leave_scores_origins_and_gradients_unchanged():
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=4)
    _, d0, p0, c0 = align(batch, abea.MODE_BATCHED, 0, scores=True)
    _, d1, p1, c1 = align(batch, abea.MODE_BATCHED, 1, scores=True)
    same_alignments(batch, p0, c0, p1, c1)
    assert np.array_equal(d0.best_scores().view(np.uint32), d1.best_scores().view(np.uint32))
    for i in (0, batch.n_reads // 2, batch.n_reads - 1):
        b0, _, o0 = d0.read_bands(i, scores=True)
        b1 = np.zeros_like(b0)
        o1 = np.zeros_like(o0)
        # scores and band origins only: a checkpointed read has no trace to give
        abea._check(abea.lib().abea_batch_read_bands(d1.ctx.h, d1.h, i, abea._p(b1), None, abea._p(o1)))
        assert np.array_equal(b0.view(np.uint32), b1.view(np.uint32))
        assert np.array_equal(o0, o1)
    g0, g1 = d0.backward(), d1.backward()
    assert np.array_equal(g0["grad_scalings"], g1["grad_scalings"])
    assert np.array_equal(g0["path_emission"], g1["path_emission"])


@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
def test_f5c_batch_with_reads_over_8kb_checkpointed(oracle_mod, mode):
    """The 1.3 Mbase workload with the trace budget of an 8 kb read: the longest
    reads recompute, the rest keep their trace; the batched form's wide shape
    takes only reads that keep their trace."""
    from abea_gb300 import synth
    import os
    batch = synth.make_batch("f5c_batch", seed=1)
    budget = (8000 + int(8000 * 1.71) + 2) * BYTES_PER_BAND
    _, dev, gp, gc = align(batch, mode, budget)
    op, oc, _ = oracle_mod.align_batch(batch, threads=os.cpu_count())
    same_alignments(batch, gp, gc, op, oc)
