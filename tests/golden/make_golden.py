"""Generates the committed golden fixtures of tests/golden/.

  dump_small_subset.npz  six reads of the reference's golden dump
                         (FPGA/code/bins/dump_small/0, reads 51, 125, 101, 70, 57, 133)
                         with f5c's AlignedPair answers.  Only the event means are
                         kept: the algorithm reads no other event field.
  ref_synthetic.npz      edge-case reads (tiny reads, few events, non-ACGT bases,
                         constant signals, unrelated signals, high and low
                         events-per-k-mer) run through the reference's own code
                         compiled by oracle/build_ref.sh; full band matrices are kept
                         for the smallest ones.

Run from the repository root with the reference checkout named by
$ABEA_REFERENCE_DIR (required):
    ABEA_REFERENCE_DIR=<checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib.util
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
REF = os.environ.get("ABEA_REFERENCE_DIR", "")
if not REF:
    sys.exit("make_golden.py: set ABEA_REFERENCE_DIR to the reference checkout")
OUT = os.path.dirname(os.path.abspath(__file__))
DUMP_READS = [51, 125, 101, 70, 57, 133]


def load_pkg():
    spec = importlib.util.spec_from_file_location(
        "abea_gb300", os.path.join(ROOT, "abea-opencl_gb300", "__init__.py"),
        submodule_search_locations=[os.path.join(ROOT, "abea-opencl_gb300")])
    m = importlib.util.module_from_spec(spec)
    sys.modules["abea_gb300"] = m
    spec.loader.exec_module(m)
    return m


def pack(batch, prefix, out):
    out[prefix + "read"] = batch.read
    out[prefix + "read_ptr"] = batch.read_ptr
    out[prefix + "read_len"] = batch.read_len
    out[prefix + "event_mean"] = batch.events["mean"].copy()
    out[prefix + "event_ptr"] = batch.event_ptr
    out[prefix + "n_events"] = batch.n_events
    out[prefix + "scalings"] = batch.scalings.view(np.float32).reshape(-1, 4)
    out[prefix + "model"] = batch.model.view(np.float32).reshape(-1, 3)


def make_dump_subset(pkg):
    from abea_gb300 import dump
    batch, golden = dump.load_batch(os.path.join(REF, "FPGA/code/bins/dump_small/0"), reads=DUMP_READS)
    out = {"reads": np.array(DUMP_READS, dtype=np.int32)}
    pack(batch, "", out)
    out["golden_counts"] = np.array([len(g) for g in golden], dtype=np.int32)
    out["golden_pairs"] = np.concatenate(golden).view(np.int32).reshape(-1, 2)
    np.savez_compressed(os.path.join(OUT, "dump_small_subset.npz"), **out)


def edge_reads(pkg, rng):
    """(name, seq bytes, event array, scalings, keep_bands) for the edge cases."""
    from abea_gb300 import synth
    from abea_gb300.types import EVENT_DTYPE, SCALINGS_DTYPE
    model = synth.make_model(rng)
    cases = []

    def sc(scale=1.0, shift=0.0):
        s = np.zeros(1, dtype=SCALINGS_DTYPE)[0]
        s["scale"], s["shift"], s["var"], s["log_var"] = scale, shift, 1.2, np.float32(np.log(1.2))
        return s

    def real(length, skip=0.01, epk=1.8, scale=1.0, shift=0.0):
        seq, ev = synth.make_read(rng, model, length, scale, shift, 1.2, skip_p=skip, mean_events=epk)
        return seq.tobytes(), ev

    def evs(means):
        e = np.zeros(len(means), dtype=EVENT_DTYPE)
        e["mean"] = np.asarray(means, dtype=np.float32)
        return e

    for L, n in ((6, 1), (7, 2), (10, 3), (12, 30), (20, 5), (40, 200), (60, 61)):
        seq = bytes(rng.choice(list(b"ACGT"), L).tolist())
        cases.append((f"tiny_{L}_{n}", seq, evs(rng.uniform(60, 130, n)), sc(), True))
    s, e = real(80, skip=0.0)
    cases.append(("short_real_80", s, e, sc(), True))
    s, e = real(150, skip=0.05)
    cases.append(("short_skip_150", s, e, sc(), True))
    s, e = real(120)
    cases.append(("non_acgt_120", s[:30] + b"NNRY" + s[34:], e, sc(), True))
    cases.append(("constant_signal_90", bytes(rng.choice(list(b"ACGT"), 90).tolist()),
                  evs(np.full(150, 100.0)), sc(), True))
    cases.append(("unrelated_signal_300", bytes(rng.choice(list(b"ACGT"), 300).tolist()),
                  evs(rng.uniform(60, 130, 500)), sc(), False))
    s, e = real(400, skip=0.7)
    cases.append(("few_events_400", s, e, sc(), False))
    s, e = real(600, epk=3.5)
    cases.append(("many_events_600", s, e, sc(), False))
    for i, L in enumerate((1500, 2500, 3000)):
        s, e = real(L, skip=0.01 if i < 2 else 0.05, scale=1.03, shift=4.0)
        cases.append((f"real_{L}", s, e, sc(1.03, 4.0), False))
    return model, cases


def make_ref_synthetic(pkg):
    from oracle import oracle
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libref.so missing: run oracle/build_ref.sh first")
    rng = np.random.default_rng(20261203)
    model, cases = edge_reads(pkg, rng)
    seqs, events, scs, names, counts, pairs = [], [], [], [], [], []
    bands = {}
    for name, seq, ev, s, keep in cases:
        p, n, info = oracle.ref_align(seq, ev, model, s, want_bands=keep)
        seqs.append(seq)
        events.append(ev)
        scs.append(s)
        names.append(name)
        counts.append(n)
        pairs.append(p)
        if keep and info["bands"] is not None:
            bands[name] = info
    batch = pkg.from_reads(seqs, events, np.array(scs), model)
    out = {"names": np.array(names)}
    pack(batch, "", out)
    out["ref_counts"] = np.array(counts, dtype=np.int32)
    out["ref_pairs"] = (np.concatenate(pairs) if pairs else np.zeros(0, pkg.PAIR_DTYPE)).view(np.int32).reshape(-1, 2)
    for name, info in bands.items():
        out[f"bands__{name}"] = info["bands"]
        out[f"trace__{name}"] = info["trace"]
        out[f"bll__{name}"] = info["bll"].view(np.int32).reshape(-1, 2)
    np.savez_compressed(os.path.join(OUT, "ref_synthetic.npz"), **out)


if __name__ == "__main__":
    pkg = load_pkg()
    make_dump_subset(pkg)
    make_ref_synthetic(pkg)
    for f in ("dump_small_subset.npz", "ref_synthetic.npz"):
        print(f, os.path.getsize(os.path.join(OUT, f)), "bytes")
