"""f5c-facing entries beyond align(): the per-read-array batch call (f5c's db_t,
`abea_align_db`) and the method-of-moments scalings (f5c's
estimate_scalings_using_mom, `abea_batch_estimate_scalings`)."""
import ctypes as C
import os
import subprocess
import time

import numpy as np
import pytest

from conftest import ROOT, abea


def read_of(batch, i):
    seq = bytes(batch.read[batch.read_ptr[i]:batch.read_ptr[i] + batch.read_len[i]])
    ev = batch.events[batch.event_ptr[i]:batch.event_ptr[i] + batch.n_events[i]]
    return seq, ev


def test_header_compiles_as_c_and_links(tmp_path):
    """A C caller of the f5c-style entries builds against include/abea.h and the library."""
    if not os.path.exists(abea.LIB_PATH):
        abea.build()
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "abea.h"\n'
        "int use(abea_ctx_t *ctx, int n, char *const *read, const int *len, const abea_event_table_t *et,\n"
        "        const abea_scalings_t *sc, const abea_model_t *m, abea_aligned_pair_t *const *out, int *cnt) {\n"
        "    return (int)abea_align_db(ctx, n, read, len, et, sc, m, out, cnt);\n"
        "}\n"
        "int main(void) { return use(0, 0, 0, 0, 0, 0, 0, 0, 0) == ABEA_ERR_INVALID_ARG ? 0 : 1; }\n")
    lib_dir = os.path.dirname(abea.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", lib_dir, "-labea", "-o", str(tmp_path / "caller")], check=True)


def test_oracle_mom_is_close_to_the_generating_scalings(oracle_mod):
    from abea_gb300 import synth
    b = synth.make_batch("adjoint", seed=13, lengths=[3000, 5000, 8000])
    true = b.meta["true_scalings"]
    for i in range(b.n_reads):
        seq, ev = read_of(b, i)
        scale, shift = oracle_mod.mom(seq, ev, b.model)
        # event counts per k-mer and skipped k-mers weight the moments a little
        assert abs(scale / true["scale"][i] - 1) < 0.05
        assert abs(shift - true["shift"][i]) < 5.0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
def test_align_db_equals_align_batch(mode, ref_synthetic):
    from abea_gb300 import synth
    # 64 reads of 9-13 kb that pass QC: over 8 MB both ways, so the staging and the
    # copy of the results back run on several host threads
    rng = np.random.default_rng(21)
    model = synth.make_model(rng)
    seqs, evs = [], []
    for L in rng.integers(9000, 13000, 64):
        s, e = synth.make_read(rng, model, int(L), 1.0, 2.0, 1.2, skip_p=0.005)
        seqs.append(s.tobytes())
        evs.append(e)
    sc = np.array([(1.0, 2.0, 1.2, np.log(1.2))] * len(seqs), dtype=abea.types.SCALINGS_DTYPE)
    big = abea.from_reads(seqs, evs, sc, model)
    for batch in (synth.make_batch("small", seed=6), ref_synthetic[0], big):
        ctx = abea.Context(0, mode)
        pairs, counts = ctx.align_batch(batch)
        per_read, c2 = ctx.align_db(batch)
        assert np.array_equal(counts, c2)
        if batch is big:
            assert np.maximum(counts, 0).sum() * 8 > 8 << 20
        for x, y in zip(abea.split_pairs(batch, pairs, counts), per_read):
            assert np.array_equal(x, y)


@pytest.mark.gpu
def test_gpu_mom_matches_the_oracle_and_seeds_recalibration(oracle_mod):
    from abea_gb300 import synth
    rng = np.random.default_rng(8)
    batch = synth.make_batch("adjoint", seed=17, lengths=rng.integers(1000, 10001, 64))
    true = batch.meta["true_scalings"]
    ctx = abea.Context(0, abea.MODE_BATCHED)
    dev = ctx.upload(batch)
    sc = dev.estimate_scalings(apply=True)
    for i in range(batch.n_reads):
        seq, ev = read_of(batch, i)
        scale, shift = oracle_mod.mom(seq, ev, batch.model)
        assert abs(sc["scale"][i] - scale) <= 1e-6 * abs(scale)
        assert abs(sc["shift"][i] - shift) <= 1e-5 * max(abs(shift), 1.0)
    assert np.all(sc["var"] == 1.0) and np.all(sc["log_var"] == 0.0)
    # method of moments, then annealed Gauss-Newton: f5c's scale -> align -> recalibrate loop
    fit = dev.recalibrate(3, first_temperature=5.0)
    ok = (np.abs(fit["shift"] - true["shift"]) < 1.0) & (np.abs(fit["scale"] / true["scale"] - 1) < 0.01)
    assert ok.mean() >= 0.9, ok.mean()


@pytest.mark.gpu
def test_persistent_and_backward_entries(oracle_mod):
    """abea_align_batch_persistent runs the batched form from a plain context;
    abea_backward_batch is abea_batch_backward."""
    import ctypes as C
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=12)
    ctx = abea.Context(0, abea.MODE_PLAIN)
    arrs = abea._batch_arrays(batch)
    pairs = np.zeros(max(batch.pair_capacity(), 1), dtype=abea.types.PAIR_DTYPE)
    counts = np.zeros(batch.n_reads, dtype=np.int32)
    abea._check(abea.lib().abea_align_batch_persistent(ctx.h, batch.n_reads, *[abea._p(a) for a in arrs],
                                                       abea._p(pairs), abea._p(counts)))
    assert ctx.get_option(abea.OPT_MODE) == abea.MODE_PLAIN
    op, oc, _ = oracle_mod.align_batch(batch, threads=os.cpu_count())
    assert np.array_equal(counts, oc)
    for x, y in zip(abea.split_pairs(batch, pairs, counts), abea.split_pairs(batch, op, oc)):
        assert np.array_equal(x, y)
    dev = abea.Context(0, abea.MODE_BATCHED).upload(batch)
    dev.run()
    g = dev.backward(model_grad=False)
    g2 = np.zeros((batch.n_reads, 3))
    abea._check(abea.lib().abea_backward_batch(dev.ctx.h, dev.h, abea._p(g2), None, None, None))
    assert np.array_equal(g["grad_scalings"], g2)


def _stage(batch, threads):
    """abea_align_db's staging of f5c's per-read arrays, on the host alone."""
    n = batch.n_reads
    reads = [np.ascontiguousarray(batch.read[batch.read_ptr[i]:batch.read_ptr[i] + batch.read_len[i]])
             for i in range(n)]
    evs = [np.ascontiguousarray(batch.events[batch.event_ptr[i]:batch.event_ptr[i] + batch.n_events[i]])
           for i in range(n)]
    read_p = (C.c_void_p * max(n, 1))(*[r.ctypes.data if len(r) else None for r in reads])
    et = (abea._EventTable * max(n, 1))()
    for i, e in enumerate(evs):
        et[i].n, et[i].start, et[i].end, et[i].event = len(e), 0, len(e), e.ctypes.data if len(e) else None
    lens = np.ascontiguousarray(batch.read_len, dtype=np.int32)
    seq = np.full(int((batch.read_len + 1).sum()), 0x5A, dtype=np.uint8)
    ev = np.zeros(int(batch.n_events.sum()), dtype=abea.EVENT_DTYPE)
    f = abea.lib().abea_internal_stage_db
    f.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
    f.restype = C.c_int32
    t0 = time.perf_counter()
    assert f(n, read_p, lens.ctypes.data, C.cast(et, C.c_void_p), seq.ctypes.data, ev.ctypes.data, threads) == 0
    return seq, ev, time.perf_counter() - t0


def test_db_staging_on_host_threads():
    """The per-read arrays land in the flattened layout (each read NUL terminated,
    events in order) whatever the number of host threads, with empty reads and
    reads without events among them."""
    if not os.path.exists(abea.LIB_PATH):
        abea.build()
    from abea_gb300 import synth
    b = synth.make_batch("f5c_batch", seed=1)
    seqs = [b.sequence(i) for i in range(b.n_reads)]
    evs = [b.read_events(i) for i in range(b.n_reads)]
    seqs[3], evs[5], seqs[7], evs[7] = b"", evs[5][:0], b"", evs[7][:0]
    b = abea.from_reads(seqs, evs, b.scalings, b.model)
    for threads in (1, 3, 8, 0):
        seq, ev, _ = _stage(b, threads)
        assert np.array_equal(seq, b.read), threads
        assert np.array_equal(ev.view(np.uint8), np.ascontiguousarray(b.events, dtype=abea.EVENT_DTYPE).view(np.uint8))
    # more threads than reads
    small = b.subset([0, 1, 2])
    seq, ev, _ = _stage(small, 8)
    assert np.array_equal(seq, small.read)
