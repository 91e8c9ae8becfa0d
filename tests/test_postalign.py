"""f5c's postalign (GPU/f5cmisc.h:51-52, a prototype only in the reference):
AlignedPairs -> base-to-event map, events per base and event alignment records
(GPU/f5c.h:184-207).  Parity is unpinned against f5c itself (its body is not in
the reference); the oracle's restatement is checked here against a second,
pure-Python one and against the structure of the reference's golden paths, and
the device kernel against the oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, abea, batch_from_npz, split_fixture_pairs

RANK = {ord("A"): 0, ord("C"): 1, ord("G"): 2, ord("T"): 3}


def py_postalign(seq: bytes, pairs, read_idx=0):
    """The same contract in plain Python loops (the second restatement)."""
    nk = len(seq) - 5
    start, stop = [-1] * nk, [-1] * nk
    lo, hi, prev = None, None, -1
    for k, e in pairs:
        if e != prev:
            if start[k] == -1:
                start[k] = e
            stop[k] = e
        lo = e if lo is None else min(lo, e)
        hi = e if hi is None else max(hi, e)
        prev = e
    epb = 0.0 if lo is None else (hi - lo) / nk
    recs, prev_rank = [], -1
    for k in range(nk):
        if start[k] == -1:
            continue
        rank = 0
        for c in seq[k:k + 6]:
            rank = (rank << 2) | RANK.get(c, 0)
        for e in range(start[k], stop[k] + 1):
            recs.append((seq[k:k + 6], k, read_idx, e, "M" if rank != prev_rank else "E"))
            prev_rank = rank
    return recs, list(zip(start, stop)), epb


def as_tuples(rec):
    return [(bytes(r["ref_kmer"]), int(r["ref_position"]), int(r["read_idx"]), int(r["event_idx"]),
             r["hmm_state"].decode()) for r in rec]


def check_one(oracle_mod, seq, pairs, read_idx=0):
    rec, bmap, epb, n = oracle_mod.postalign(seq, pairs, read_idx)
    recs, m, pepb = py_postalign(seq, [(int(p[0]), int(p[1])) for p in pairs], read_idx)
    assert n == len(recs)
    assert as_tuples(rec) == recs
    assert list(zip(bmap["start"].tolist(), bmap["stop"].tolist())) == m
    assert epb == pepb
    assert np.all(rec["model_kmer"] == rec["ref_kmer"]) and np.all(rec["rc"] == 0)
    return rec, bmap, epb


def test_record_layout_matches_the_c_struct(tmp_path):
    """abea_event_alignment_t / abea_index_pair_t offsets as gcc lays them out,
    against the NumPy mirrors (the reference's member order, GPU/f5c.h:184-207)."""
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "abea.h"\n'
        "int main(void) {\n"
        "  printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(abea_event_alignment_t),\n"
        "    offsetof(abea_event_alignment_t, ref_kmer), offsetof(abea_event_alignment_t, ref_position),\n"
        "    offsetof(abea_event_alignment_t, read_idx), offsetof(abea_event_alignment_t, event_idx),\n"
        "    offsetof(abea_event_alignment_t, rc), offsetof(abea_event_alignment_t, model_kmer),\n"
        "    offsetof(abea_event_alignment_t, hmm_state), sizeof(abea_index_pair_t));\n"
        "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    dt = abea.EVENT_ALIGNMENT_DTYPE
    want = [dt.itemsize] + [dt.fields[f][1] for f in
                            ("ref_kmer", "ref_position", "read_idx", "event_idx", "rc", "model_kmer", "hmm_state")]
    assert got == want + [abea.INDEX_PAIR_DTYPE.itemsize]


def test_oracle_postalign_on_the_reference_golden_paths(oracle_mod):
    """The reference's golden AlignedPairs (dump_small subset): both restatements
    agree, and on these unit-step paths the records are one per event from the
    first event on the path to the last."""
    d = np.load(os.path.join(GOLDEN, "dump_small_subset.npz"))
    batch = batch_from_npz(d)
    golden = split_fixture_pairs(d["golden_pairs"], d["golden_counts"])
    for i in range(batch.n_reads):
        if len(golden[i]) == 0:
            continue
        seq = batch.sequence(i)
        pairs = np.stack([golden[i]["ref_pos"], golden[i]["read_pos"]], axis=1)
        rec, bmap, epb = check_one(oracle_mod, seq, pairs, i)
        e0, e1 = int(pairs[0, 1]), int(pairs[-1, 1])
        assert np.array_equal(rec["event_idx"], np.arange(e0, e1 + 1))
        assert np.all(np.diff(rec["ref_position"]) >= 0)
        assert epb == (e1 - e0) / (len(seq) - 5)
        # every map entry with events covers exactly its records
        has = bmap["start"] >= 0
        counts = np.bincount(rec["ref_position"], minlength=len(bmap))
        assert np.array_equal(counts[has], bmap["stop"][has] - bmap["start"][has] + 1)
        assert np.all(counts[~has] == 0)


def test_oracle_postalign_edge_cases(oracle_mod):
    # no pairs: an empty map and no records
    rec, bmap, epb, n = oracle_mod.postalign(b"ACGTACGTAC", np.zeros((0, 2), np.int32))
    assert n == 0 and epb == 0.0 and np.all(bmap["start"] == -1) and np.all(bmap["stop"] == -1)
    # a homopolymer: every k-mer has rank 0, so only the first record is a match
    seq = b"AAAAAAAAAAAA"
    pairs = np.array([[0, 0], [1, 1], [2, 2], [2, 3], [3, 3], [4, 4]], np.int32)
    rec, _, _ = check_one(oracle_mod, seq, pairs)
    assert rec["hmm_state"].tolist() == [b"M", b"E", b"E", b"E", b"E"]
    # non-ACGT bases rank as A: NNNNNN and AAAAAA are the same k-mer for the state
    seq = b"NNNNNNAAAAAAC"
    pairs = np.array([[0, 0], [1, 1], [2, 2], [3, 3], [4, 4], [5, 5], [6, 6], [7, 7]], np.int32)
    rec, _, _ = check_one(oracle_mod, seq, pairs)
    assert rec["hmm_state"].tolist() == [b"M", b"E", b"E", b"E", b"E", b"E", b"E", b"M"]
    assert rec["ref_kmer"][0] == b"NNNNNN"
    # a skipped k-mer (L move) keeps no events; a stay (U move) extends the range
    seq = b"ACGTTGCAACGT"
    pairs = np.array([[0, 0], [0, 1], [1, 2], [2, 2], [3, 3], [4, 4]], np.int32)
    rec, bmap, epb = check_one(oracle_mod, seq, pairs)
    assert bmap[:5].tolist() == [(0, 1), (2, 2), (-1, -1), (3, 3), (4, 4)]
    assert epb == 4 / 7
    # output capacity and pairs outside the read
    assert oracle_mod.postalign(seq, pairs, out_cap=2)[3] == -2  # ABEA_ERR_CAPACITY
    assert oracle_mod.postalign(seq, np.array([[9, 0]], np.int32))[3] == -1  # ABEA_ERR_INVALID_ARG


def test_oracle_postalign_on_oracle_paths_of_synthetic_reads(oracle_mod):
    """Reads of the synthetic generator aligned by the oracle: both restatements agree."""
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=3, lengths=[300, 800, 1500])
    pairs, counts, _ = oracle_mod.align_batch(batch, threads=2)
    for i, p in enumerate(abea.split_pairs(batch, pairs, counts)):
        check_one(oracle_mod, batch.sequence(i), np.stack([p["ref_pos"], p["read_pos"]], axis=1), i)


def device_vs_oracle(oracle_mod, batch, mode, opts=None):
    ctx = abea.Context(0, mode)
    for k, v in (opts or {}).items():
        ctx.set_option(k, v)
    dev = ctx.upload(batch)
    dev.run()
    pairs, counts = dev.results()
    got = dev.postalign()
    rec, bmap, epb, cnt = oracle_mod.postalign_batch(batch, pairs, counts)
    assert np.array_equal(got["n_alignment"], cnt)
    assert np.array_equal(got["events_per_base"].view(np.uint64), epb.view(np.uint64))
    # records past each read's count stay zero, as the oracle's do
    assert np.array_equal(got["alignment"].view(np.uint8), rec.view(np.uint8))
    assert np.array_equal(got["base_to_event_map"], bmap)
    ctx.close()
    return got, counts


@pytest.mark.gpu
def test_device_postalign_matches_the_oracle_on_edge_cases(oracle_mod):
    """The reference fixture's edge cases (tiny reads, QC failures, non-ACGT
    bases, constant signal) in both forms, and with every read on the wide shape."""
    batch = batch_from_npz(np.load(os.path.join(GOLDEN, "ref_synthetic.npz")))
    for mode, opts in ((abea.MODE_PLAIN, {}), (abea.MODE_BATCHED, {}),
                       (abea.MODE_BATCHED, {abea.OPT_LONG_READ_BANDS: 1})):
        got, counts = device_vs_oracle(oracle_mod, batch, mode, opts)
        assert np.any(counts == 0) and np.any(got["n_alignment"] > 0)


@pytest.mark.gpu
def test_device_postalign_matches_the_oracle_on_the_f5c_batch(oracle_mod):
    """The 1.3 Mbase batch (363 reads), batched form."""
    from abea_gb300 import synth
    batch = synth.make_batch("f5c_batch", seed=1)
    got, counts = device_vs_oracle(oracle_mod, batch, abea.MODE_BATCHED)
    ok = counts > 0
    assert np.all(got["n_alignment"][ok] > 0) and np.all(got["n_alignment"][~ok] == 0)
    for (rec, bmap), n in zip(abea.split_postalign(batch, got), batch.n_events):
        assert len(rec) <= n


@pytest.mark.gpu
def test_postalign_needs_a_run():
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=7, lengths=[600])
    ctx = abea.Context(0, abea.MODE_BATCHED)
    dev = ctx.upload(batch)
    with pytest.raises(abea.AbeaError):
        dev.postalign()
    ctx.close()


def test_batch_layout_of_the_oracle_and_the_split_helper(oracle_mod):
    """postalign_batch writes each read where abea_batch_postalign does (records
    from event_ptr, map entries from read_ptr), and split_postalign cuts them
    back into the per-read results."""
    from abea_gb300 import synth
    batch = synth.make_batch("small", seed=4, lengths=[200, 700, 1300])
    pairs, counts, _ = oracle_mod.align_batch(batch, threads=2)
    rec, bmap, epb, cnt = oracle_mod.postalign_batch(batch, pairs, counts)
    assert len(rec) == int((batch.event_ptr + batch.n_events).max())
    assert len(bmap) == int((batch.read_ptr + batch.read_len).max())
    out = dict(alignment=rec, base_to_event_map=bmap, events_per_base=epb, n_alignment=cnt)
    for i, ((r, m), p) in enumerate(zip(abea.split_postalign(batch, out), abea.split_pairs(batch, pairs, counts))):
        r1, m1, e1, n1 = oracle_mod.postalign(batch.sequence(i), p, i)
        assert n1 == cnt[i] == len(r) and epb[i] == e1
        assert np.array_equal(r.view(np.uint8), r1.view(np.uint8)) and np.array_equal(m, m1)
        assert np.all(r["read_idx"] == i)
