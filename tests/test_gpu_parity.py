"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle and the
reference's golden vectors.  Bit-exact for AlignedPairs, counts, band scores,
backpointers and band placements (integer/index results and the reference's
own float rounding)."""
import numpy as np
import pytest

from conftest import abea

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import os
    if not os.path.exists(abea.LIB_PATH):
        abea.build()
    return abea.lib()


def run(batch, mode=abea.MODE_PLAIN, scores=False):
    ctx = abea.Context(0, mode, store_scores=scores)
    pairs, counts = ctx.align_batch(batch)
    return ctx, pairs, counts


def oracle_batch(oracle_mod, batch):
    return oracle_mod.align_batch(batch, threads=os.cpu_count())


import os  # noqa: E402


def assert_same_alignments(batch, pairs, counts, opairs, ocounts):
    assert np.array_equal(counts, ocounts)
    got = abea.split_pairs(batch, pairs, counts)
    exp = abea.split_pairs(batch, opairs, ocounts)
    for i in range(batch.n_reads):
        assert np.array_equal(got[i], exp[i]), f"read {i}"


@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
def test_dump_subset_matches_f5c(lib, dump_subset, mode):
    batch, golden = dump_subset
    _, pairs, counts = run(batch, mode)
    got = abea.split_pairs(batch, pairs, counts)
    for i, g in enumerate(golden):
        assert counts[i] == len(g)
        assert np.array_equal(got[i], g)


@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
def test_edge_cases_match_reference(lib, oracle_mod, ref_synthetic, mode):
    batch, names, counts, pairs, bands = ref_synthetic
    ctx = abea.Context(0, mode, store_scores=True)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    op, oc, _ = oracle_batch(oracle_mod, batch)
    assert_same_alignments(batch, gp, gc, op, oc)
    assert np.array_equal(gc, counts)
    for i, name in enumerate(names):
        if name not in bands:
            continue
        b, t, bll = dev.read_bands(i, scores=True)
        rb, rt, rbll = bands[name]
        assert np.array_equal(b.view(np.uint32), rb.view(np.uint32)), name
        assert np.array_equal(t, rt), name
        assert np.array_equal(bll.view(np.int32).reshape(-1, 2), rbll), name


@pytest.mark.parametrize("shape", ["warp", "wide", "medium"])
@pytest.mark.parametrize("seed", [1, 2, 4])
def test_small_workload_bit_exact(lib, oracle_mod, seed, shape):
    """Every score, backpointer and band origin of four reads, and every read's
    best score, against the oracle: on the warp shape (plain form), on the wide
    shape (batched form with every read wide) and on the medium shape (batched
    form with every read medium, two per block)."""
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=seed)
    ctx = abea.Context(0, abea.MODE_PLAIN if shape == "warp" else abea.MODE_BATCHED, store_scores=True)
    if shape == "wide":
        ctx.set_option(abea.OPT_LONG_READ_BANDS, 1)
    if shape == "medium":
        ctx.set_option(abea.OPT_LONG_READ_BANDS, 1 << 40)
        ctx.set_option(abea.OPT_MEDIUM_READ_BANDS, 1)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    op, oc, obest = oracle_batch(oracle_mod, batch)
    assert_same_alignments(batch, gp, gc, op, oc)
    assert np.array_equal(dev.best_scores().view(np.uint32), obest.view(np.uint32))
    for i in (0, 7, 47, 63):
        b, t, bll = dev.read_bands(i, scores=True)
        _, _, info = oracle_mod.align(batch.sequence(i), batch.read_events(i), batch.model,
                                      batch.scalings[i], want_bands=True)
        assert np.array_equal(b.view(np.uint32), info["bands"].view(np.uint32))
        assert np.array_equal(t, info["trace"])
        assert np.array_equal(bll, info["bll"])


def test_low_skip_reads_pass_qc_bit_exact(lib, oracle_mod):
    """Reads that pass QC (1% skipped k-mers), so the pair lists are non-empty."""
    from abea_gb300 import synth
    rng = np.random.default_rng(3)
    model = synth.make_model(rng)
    seqs, evs, scs = [], [], []
    for L in rng.integers(500, 4000, 24):
        s, e = synth.make_read(rng, model, L, 1.0, 2.0, 1.2, skip_p=0.01)
        seqs.append(s.tobytes())
        evs.append(e)
        scs.append((1.0, 2.0, 1.2, np.log(1.2)))
    batch = abea.from_reads(seqs, evs, np.array(scs, dtype=abea.types.SCALINGS_DTYPE), model)
    _, gp, gc = run(batch)
    op, oc, _ = oracle_batch(oracle_mod, batch)
    assert (oc > 0).sum() >= 20
    assert_same_alignments(batch, gp, gc, op, oc)


def test_single_read_drop_in(lib, oracle_mod, dump_subset):
    """abea_align(): f5c's align() signature, one read at a time."""
    batch, golden = dump_subset
    for i in range(batch.n_reads):
        p = abea.align(batch.sequence(i), batch.read_events(i), batch.model, batch.scalings[i], 4000.0)
        assert np.array_equal(p, golden[i])


@pytest.mark.parametrize("shape", ["warp", "wide", "medium"])
def test_fp64_fallback_cells_stay_exact(lib, oracle_mod, shape):
    """A pore model with level_stdv near 0.4 makes emissions tiny, which defeats
    the FP32 exactness proof and sends many cells down the FP64 path: on the
    warp shape, and on the wide and medium shapes, which redo a band's unproven
    cells after the band's closing barrier (every score and backpointer of the
    longest read checked)."""
    from abea_gb300 import synth
    rng = np.random.default_rng(17)
    model = synth.make_model(rng)
    model["level_stdv"] = rng.uniform(0.38, 0.42, len(model)).astype(np.float32)
    model["level_log_stdv"] = np.log(model["level_stdv"].astype(np.float64)).astype(np.float32)
    seqs, evs, scs = [], [], []
    for L in (300, 800, 1500):
        s, e = synth.make_read(rng, model, L, 1.0, 0.0, 0.3, skip_p=0.01)
        seqs.append(s.tobytes())
        evs.append(e)
        scs.append((1.0, 0.0, 1.0, 0.0))
    batch = abea.from_reads(seqs, evs, np.array(scs, dtype=abea.types.SCALINGS_DTYPE), model)
    ctx = abea.Context(0, abea.MODE_PLAIN if shape == "warp" else abea.MODE_BATCHED, store_scores=True)
    if shape == "wide":
        ctx.set_option(abea.OPT_LONG_READ_BANDS, 1)
    if shape == "medium":
        ctx.set_option(abea.OPT_LONG_READ_BANDS, 1 << 40)
        ctx.set_option(abea.OPT_MEDIUM_READ_BANDS, 1)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    op, oc, obest = oracle_batch(oracle_mod, batch)
    assert_same_alignments(batch, gp, gc, op, oc)
    assert np.array_equal(dev.best_scores().view(np.uint32), obest.view(np.uint32))
    b, t, bll = dev.read_bands(2, scores=True)
    _, _, info = oracle_mod.align(batch.sequence(2), batch.read_events(2), batch.model,
                                  batch.scalings[2], want_bands=True)
    assert np.array_equal(b.view(np.uint32), info["bands"].view(np.uint32))
    assert np.array_equal(t, info["trace"])
    assert np.array_equal(bll, info["bll"])
    assert dev.slow_cells() > 1000


def test_degenerate_reads(lib, oracle_mod):
    """Reads shorter than a k-mer, reads without events, non-ACGT bases."""
    from abea_gb300 import synth
    rng = np.random.default_rng(23)
    model = synth.make_model(rng)
    ev = np.zeros(10, dtype=abea.types.EVENT_DTYPE)
    ev["mean"] = rng.uniform(60, 130, 10)
    seqs = [b"ACG", b"ACGTACGTAC", b"NNNNNNNNNNNN", b"ACGTAC"]
    evs = [ev, ev[:0], ev, ev[:1]]
    scs = np.array([(1.0, 0.0, 1.0, 0.0)] * 4, dtype=abea.types.SCALINGS_DTYPE)
    batch = abea.from_reads(seqs, evs, scs, model)
    _, gp, gc = run(batch)
    op, oc, _ = oracle_batch(oracle_mod, batch)
    assert_same_alignments(batch, gp, gc, op, oc)


def test_empty_batch(lib):
    from abea_gb300 import synth
    b = synth.make_batch("small", seed=1).subset([])
    _, pairs, counts = run(b)
    assert len(counts) == 0


def test_exact_arithmetic_selftest(lib):
    """The FP32 division and double-rounded sums never claim a wrong result on
    2^28 random and near-midpoint cases; declines stay rare."""
    r = abea.selftest_arith(1 << 28, seed=12345)
    assert r["div_wrong"] == 0
    assert r["sum_wrong"] == 0
    assert r["div_declined"] < r["cases"] * 1e-3
    # two sums per case (exact_sum, exact_skip); half aim at rounding midpoints on
    # purpose and many exact_sum cases draw |c| below the Fast2Sum exponent
    # bound; the rest must be proven on the fast path
    assert 2 * r["cases"] - r["sum_declined"] > r["cases"]


@pytest.mark.parametrize("workload", ["f5c_batch", "uneven"])
@pytest.mark.parametrize("mode", [abea.MODE_PLAIN, abea.MODE_BATCHED])
def test_benchmark_batches_full_size(lib, oracle_mod, mode, workload):
    """The two benchmarked 1.3 Mbase batches exactly as the benchmark builds them
    (seed 1): the f5c batch (~360 reads) and the heavy-tailed uneven batch (reads
    up to 100 kb): AlignedPairs and best-end scores bit-exact with the oracle."""
    from abea_gb300 import synth
    batch = synth.make_batch(workload, seed=1)
    ctx = abea.Context(0, mode)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    op, oc, obest = oracle_batch(oracle_mod, batch)
    assert_same_alignments(batch, gp, gc, op, oc)
    assert np.array_equal(dev.best_scores().view(np.uint32), obest.view(np.uint32))


# Relative error of the FP32 best-end scores against the all-FP64 recurrence,
# measured on these batches (seed 1): small 3.4e-6, f5c 5.5e-6, uneven 2.3e-5 (the
# error grows with read length: 100 kb reads).  The bounds leave a factor ~2.
FP64_REL_BOUND = {"small": 1e-5, "f5c_batch": 1e-5, "uneven": 5e-5}


@pytest.mark.parametrize("workload", ["small", "f5c_batch", "uneven"])
def test_error_against_fp64_is_bounded(lib, oracle_mod, workload):
    """The GPU's best scores are the reference's FP32 results bit for bit; their
    distance to the all-FP64 recurrence (the oracle's FP64 twin) is stated and
    bounded, and only a few reads take other AlignedPairs under FP64."""
    from abea_gb300 import synth
    batch = synth.make_batch(workload, seed=1)
    ctx = abea.Context(0, abea.MODE_BATCHED)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    best = dev.best_scores()
    _, _, obest = oracle_batch(oracle_mod, batch)
    assert np.array_equal(best.view(np.uint32), obest.view(np.uint32))
    e = oracle_mod.fp64_error(batch, best, gp, gc, threads=os.cpu_count())
    print(workload, e)
    assert e["finite_ends"] == batch.n_reads
    assert e["best_score_rel_err_max"] < FP64_REL_BOUND[workload]
    assert e["reads_with_other_pair_count"] == 0
    assert e["reads_with_other_pairs"] <= max(3, batch.n_reads // 20)


@pytest.mark.parametrize("wide_reads, medium_reads", [(0, 300), (8, 200), (30, 600)])
def test_three_shapes_in_one_batch(lib, oracle_mod, wide_reads, medium_reads):
    """The wide shape for the longest reads, the medium shape (two reads per block)
    for the next ones, one warp per read for the rest, in one launch: AlignedPairs
    and best scores bit-exact with the oracle, and the same through the graph
    replay of a second run."""
    from abea_gb300 import synth
    batch = synth.make_batch("reads1024", seed=3)
    nb = np.sort(batch.n_bands())[::-1]
    ctx = abea.Context(0, abea.MODE_BATCHED)
    ctx.set_option(abea.OPT_LONG_READ_BANDS, int(nb[wide_reads - 1]) if wide_reads else 1 << 40)
    ctx.set_option(abea.OPT_MEDIUM_READ_BANDS, int(nb[wide_reads + medium_reads - 1]))
    dev = ctx.upload(batch)
    op, oc, obest = oracle_batch(oracle_mod, batch)
    for _ in range(2):
        dev.run()
        gp, gc = dev.results()
        assert_same_alignments(batch, gp, gc, op, oc)
        assert np.array_equal(dev.best_scores().view(np.uint32), obest.view(np.uint32))


def test_uneven_batch_batched_equals_plain(lib):
    """Heavy-tailed 1.3 Mbase batch: batched (wide + warp shapes, fused post) and
    plain forms give identical AlignedPairs."""
    from abea_gb300 import synth
    batch = synth.make_batch("uneven", seed=2)
    _, p1, c1 = run(batch, abea.MODE_PLAIN)
    _, p2, c2 = run(batch, abea.MODE_BATCHED)
    assert_same_alignments(batch, p2, c2, p1, c1)


def test_autotuned_batched_stays_exact(lib, oracle_mod):
    """The autotuner only changes which reads run on the wide shape; results
    stay bit-exact, through the CUDA-graph replay of the batched form."""
    from abea_gb300 import synth
    batch = synth.make_batch("uneven", seed=5)
    ctx = abea.Context(0, abea.MODE_BATCHED)
    dev = ctx.upload(batch)
    thr, ms = dev.autotune()
    assert thr > 0 and ms > 0
    dev.run()
    gp, gc = dev.results()
    assert dev.timing()["kernel_launches"] == 1  # pre, fill and traceback fused, one graph
    op, oc, _ = oracle_batch(oracle_mod, batch)
    assert_same_alignments(batch, gp, gc, op, oc)


def test_graph_recaptured_for_each_batch_layout(lib, oracle_mod):
    """abea_align_batch reuses one device batch per context: a second batch with
    the same read count but other lengths carves the device slab differently, so
    the batched form's graph must not replay the first batch's pointers."""
    from abea_gb300 import synth
    ctx = abea.Context(0, abea.MODE_BATCHED)
    for lengths in ([1500, 2600, 1200, 900], [2900, 700, 2200, 1800], [1500, 2600, 1200, 900]):
        batch = synth.make_batch("small", seed=len(lengths) + lengths[1], lengths=lengths)
        gp, gc = ctx.align_batch(batch)
        op, oc, _ = oracle_batch(oracle_mod, batch)
        assert_same_alignments(batch, gp, gc, op, oc)


@pytest.mark.parametrize("workload", ["small", "f5c_batch", "uneven"])
def test_cluster_pair_wide_shape_is_exact(lib, oracle_mod, workload):
    """ABEA_OPT_WIDE_CLUSTER: wide reads on a cluster of two blocks (the second
    SM computing the emissions into the first one's shared memory) give the
    plain form's AlignedPairs; on the small workload every read takes that shape."""
    from abea_gb300 import synth
    batch = synth.make_batch(workload, seed=4)
    ctx = abea.Context(0, abea.MODE_BATCHED)
    ctx.set_option(abea.OPT_WIDE_CLUSTER, 1)
    if workload == "small":
        ctx.set_option(abea.OPT_LONG_READ_BANDS, 1)
    gp, gc = ctx.align_batch(batch)
    if workload == "small":
        op, oc, _ = oracle_batch(oracle_mod, batch)
    else:
        op, oc = abea.Context(0, abea.MODE_PLAIN).align_batch(batch)
    assert_same_alignments(batch, gp, gc, op, oc)


@pytest.mark.parametrize("threshold", [1, 512])
def test_wide_shape_block_traceback_on_the_edge_cases(lib, ref_synthetic, threshold):
    """Reads of 512 bands or more on the wide shape have their traceback walked by
    the whole block (speculative segments spliced into the true path).  The
    reference fixture's long edge cases go through it: a path longer than its
    output slot (few_events_400: the serial walk takes over), reads that fail the
    QC, reads over several 256-band segments.  Shorter reads take the serial
    walk on the wide shape when the threshold is one band."""
    batch, names, counts, pairs, _ = ref_synthetic
    ctx = abea.Context(0, abea.MODE_BATCHED)
    ctx.set_option(abea.OPT_LONG_READ_BANDS, threshold)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    assert np.array_equal(gc, counts)
    got = abea.split_pairs(batch, gp, gc)
    for i, name in enumerate(names):
        assert np.array_equal(got[i], pairs[i]), name
    # the adjoint reads the path the traceback left
    g = dev.backward()
    g0 = abea.Context(0, abea.MODE_PLAIN).upload(batch)
    g0.run()
    h = g0.backward()
    assert np.array_equal(g["path_emission"], h["path_emission"])
    assert np.array_equal(g["status"], h["status"])


def test_autotuner_cache_round_trip(lib, tmp_path):
    """abea_autotune_save / abea_autotune_load: the tuned thresholds survive a file;
    a malformed file or one tuned on another SM count is refused."""
    from abea_gb300 import synth
    batch = synth.make_batch("uneven", seed=3)
    ctx = abea.Context(0, abea.MODE_BATCHED)
    dev = ctx.upload(batch)
    thr, _ = dev.autotune()
    path = str(tmp_path / "tuned.txt")
    assert ctx.autotune_save(path) == 1
    other = abea.Context(0, abea.MODE_BATCHED)
    assert other.autotune_load(path) == 1
    p1, c1 = ctx.align_batch(batch)
    p2, c2 = other.align_batch(batch)
    assert_same_alignments(batch, p1, c1, p2, c2)
    lines = open(path).read().split("\n")
    assert lines[0].startswith("abea-autotune 2 sm_count ") and lines[1].split()[1] == str(thr)
    assert int(lines[1].split()[2]) >= 1  # the medium threshold (INT64_MAX: none)
    assert other.get_option(abea.OPT_MEDIUM_READ_BANDS) == 0
    (tmp_path / "bad.txt").write_text("not a cache\n")
    with pytest.raises(abea.AbeaError):
        other.autotune_load(str(tmp_path / "bad.txt"))
    sm = int(lines[0].split()[-1])
    (tmp_path / "other_gpu.txt").write_text(f"abea-autotune 2 sm_count {sm + 1}\n{lines[1]}\n")
    with pytest.raises(abea.AbeaError):
        other.autotune_load(str(tmp_path / "other_gpu.txt"))
    # a version 1 file (wide threshold only) still loads
    sig, wide = lines[1].split()[:2]
    (tmp_path / "v1.txt").write_text(f"abea-autotune 1 sm_count {sm}\n{sig} {wide}\n")
    assert other.autotune_load(str(tmp_path / "v1.txt")) == 1


def _pinned_call(ctx, batch):
    """abea_align_batch on pinned copies of the batch into pinned outputs filled
    with a pattern (so every count and pair of the result must be written)."""
    pb = abea.pin_batch(batch)
    pairs = abea.pinned_empty(max(batch.pair_capacity(), 1), abea.types.PAIR_DTYPE)
    counts = abea.pinned_empty(batch.n_reads, np.int32)
    pairs.view(np.uint8)[:] = 0xA5
    counts[:] = -7
    return ctx.align_batch(pb, out_pairs=pairs, out_counts=counts)


@pytest.mark.parametrize("workload,mode", [("f5c_batch", abea.MODE_BATCHED), ("uneven", abea.MODE_BATCHED),
                                           ("f5c_batch", abea.MODE_PLAIN)])
def test_align_batch_pinned_inputs_and_results_in_place(lib, workload, mode):
    """abea_align_batch with pinned buffers: the pre stage reads every read's
    bases and events from host memory (no input copy) and each read's
    AlignedPairs and count go into the caller's buffers as the read finishes (no
    result copy).  Results equal the device-resident batch's, in both forms, on
    the second call (graph replay) too, and with pageable buffers."""
    from abea_gb300 import synth
    batch = synth.make_batch(workload, seed=1)
    ctx = abea.Context(0, mode)
    dev = ctx.upload(batch)
    dev.run()
    rp, rc = dev.results()
    dev.close()
    for _ in range(2):
        gp, gc = _pinned_call(ctx, batch)
        assert_same_alignments(batch, gp, gc, rp, rc)
    up, uc = ctx.align_batch(batch)
    assert_same_alignments(batch, up, uc, rp, rc)


def test_pinned_results_on_the_edge_cases(lib, oracle_mod, ref_synthetic):
    """Pinned outputs with reads that are skipped (shorter than a k-mer, no
    events), fail QC or overflow: every count is written, the pairs match."""
    batch = ref_synthetic[0]
    op, oc, _ = oracle_batch(oracle_mod, batch)
    for mode in (abea.MODE_PLAIN, abea.MODE_BATCHED):
        gp, gc = _pinned_call(abea.Context(0, mode), batch)
        assert_same_alignments(batch, gp, gc, op, oc)


@pytest.mark.parametrize("workload", ["f5c_batch", "reads1024"])
def test_more_wide_reads_than_blocks(lib, workload):
    """Every read on the wide shape: the blocks pull wide reads one after another
    (each reusing its traceback scratch slot), so most blocks fill several.  The
    AlignedPairs and best scores equal the plain form's."""
    from abea_gb300 import synth
    batch = synth.make_batch(workload, seed=3)
    ctx = abea.Context(0, abea.MODE_BATCHED)
    ctx.set_option(abea.OPT_LONG_READ_BANDS, 1)
    dev = ctx.upload(batch)
    dev.run()
    gp, gc = dev.results()
    gb = dev.best_scores()
    pctx = abea.Context(0, abea.MODE_PLAIN)
    pdev = pctx.upload(batch)
    pdev.run()
    pp, pc = pdev.results()
    assert_same_alignments(batch, gp, gc, pp, pc)
    assert np.array_equal(gb.view(np.uint32), pdev.best_scores().view(np.uint32))
