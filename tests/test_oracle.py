"""The CPU oracle against the reference's golden vectors (CPU only)."""
import os

import numpy as np
import pytest

from conftest import ROOT

def _reference_dir():
    """ABEA_REFERENCE_DIR, else the checkout oracle/build_ref.sh compiled from ("" when none)."""
    d = os.environ.get("ABEA_REFERENCE_DIR", "")
    rec = os.path.join(ROOT, "oracle", "_ref", "source_dir")
    if not d and os.path.exists(rec):
        with open(rec) as f:
            d = f.read().strip()
    return d


REF_DUMP = os.path.join(_reference_dir(), "FPGA/code/bins/dump_small/0") if _reference_dir() else ""


def test_oracle_dump_subset_bit_exact(oracle_mod, dump_subset):
    """f5c's own AlignedPairs of six dump reads, bit-exact."""
    batch, golden = dump_subset
    for flags in (0, oracle_mod.LOG_UNCACHED, oracle_mod.QC_FLOAT):
        pairs, counts, _ = oracle_mod.align_batch(batch, flags=flags, threads=4)
        from abea_gb300.types import split_pairs
        got = split_pairs(batch, pairs, counts)
        for i, g in enumerate(golden):
            assert counts[i] == len(g)
            assert np.array_equal(got[i], g), f"read {i} flags {flags}"


@pytest.mark.skipif(not REF_DUMP or not os.path.isdir(REF_DUMP), reason="reference checkout not present")
def test_oracle_full_dump_bit_exact(oracle_mod):
    """All 143 reads / 1,461,052 pairs of the reference's golden dump."""
    from abea_gb300 import dump
    from abea_gb300.types import split_pairs
    batch, golden = dump.load_batch(REF_DUMP)
    pairs, counts, _ = oracle_mod.align_batch(batch, threads=os.cpu_count())
    got = split_pairs(batch, pairs, counts)
    assert batch.n_reads == 143
    assert sum(len(g) for g in golden) == 1461052
    bad = [i for i in range(batch.n_reads) if not np.array_equal(got[i], golden[i])]
    assert bad == []


def test_oracle_matches_reference_code(oracle_mod, ref_synthetic):
    """Edge-case reads run through the reference's own compiled code: counts,
    pairs and (for small reads) full band matrices, bit-exact.  The reference
    build used the single-work-item host post (float QC sum, uncached log)."""
    batch, names, counts, pairs, bands = ref_synthetic
    flags = oracle_mod.QC_FLOAT | oracle_mod.LOG_UNCACHED
    for i, name in enumerate(names):
        p, n, info = oracle_mod.align(batch.sequence(i), batch.read_events(i), batch.model,
                                      batch.scalings[i], flags=flags, want_bands=name in bands)
        assert n == counts[i], name
        assert np.array_equal(p, pairs[i]), name
        if name in bands:
            rb, rt, rbll = bands[name]
            assert np.array_equal(info["bands"].view(np.uint32), rb.view(np.uint32)), name
            assert np.array_equal(info["trace"], rt), name
            assert np.array_equal(info["bll"].view(np.int32).reshape(-1, 2), rbll), name


def test_oracle_default_qc_agrees_on_edge_cases(oracle_mod, ref_synthetic):
    """f5c's double QC sum and the cached log agree with the reference build here."""
    batch, names, counts, pairs, _ = ref_synthetic
    for i, name in enumerate(names):
        p, n, _ = oracle_mod.align(batch.sequence(i), batch.read_events(i), batch.model, batch.scalings[i])
        assert n == counts[i], name


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libref.so")),
                    reason="reference code not compiled here")
def test_oracle_vs_reference_code_random(oracle_mod):
    """Random synthetic reads: oracle == reference code, including band matrices."""
    from abea_gb300 import synth
    b = synth.make_batch("small", seed=11, lengths=np.random.default_rng(5).integers(200, 1500, 12))
    flags = oracle_mod.QC_FLOAT | oracle_mod.LOG_UNCACHED
    for i in range(b.n_reads):
        p1, n1, i1 = oracle_mod.align(b.sequence(i), b.read_events(i), b.model, b.scalings[i],
                                      flags=flags, want_bands=True)
        p2, n2, i2 = oracle_mod.ref_align(b.sequence(i), b.read_events(i), b.model, b.scalings[i],
                                          want_bands=True)
        assert n1 == n2 and np.array_equal(p1, p2)
        assert np.array_equal(i1["bands"].view(np.uint32), i2["bands"].view(np.uint32))
        assert np.array_equal(i1["trace"], i2["trace"])


def test_add3_double_rounding(oracle_mod):
    """The oracle's cell sum is the reference's double-rounded float+double+float."""
    a, b, c = np.float32(-1234.5677), -0.9932717776298523, np.float32(-3.2510002)
    exp = np.float32(np.float64(np.float64(a) + b) + np.float64(c))
    assert oracle_mod.add3(float(a), b, float(c)) == exp
