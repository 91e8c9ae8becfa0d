"""Reader and writer for the reference's raw batch dumps.

Layout (GPU/dump_functions.h:1-177): a dump directory holds
`no_of_batches.dat` (int32) and one directory per batch; a batch directory
holds `n_bam_rec.dat` (int32), `model.dat` (4096 x model_t) and one directory
per read with `read_len[i].dat` (int32), `read[i].dat` (bases, no NUL),
`et[i].dat` (32-byte event_table header: n, start, end, pointer; then n x
event_t), `scalings[i].dat` (scalings_t), `f5[i].sample_rate.dat` (float),
and, when the dump carries f5c's answers, `n_event_align_pairs[i].dat`
(int32) and `event_align_pairs.dat` (n x AlignedPair).
"""
from __future__ import annotations

import os

import numpy as np

from .types import EVENT_DTYPE, MODEL_DTYPE, NUM_KMER, PAIR_DTYPE, SCALINGS_DTYPE, Batch, from_reads


def _read(path, dtype, count=-1):
    with open(path, "rb") as f:
        return np.fromfile(f, dtype=dtype, count=count)


def n_batches(dump_dir: str) -> int:
    return int(_read(os.path.join(dump_dir, "no_of_batches.dat"), "<i4", 1)[0])


def load_batch(batch_dir: str, with_outputs: bool = True, reads=None):
    """Returns (Batch, golden) where golden is a list of AlignedPair arrays or None."""
    n = int(_read(os.path.join(batch_dir, "n_bam_rec.dat"), "<i4", 1)[0])
    model = _read(os.path.join(batch_dir, "model.dat"), MODEL_DTYPE, NUM_KMER)
    if len(model) != NUM_KMER:
        raise ValueError("model.dat is short")
    idx = range(n) if reads is None else reads
    seqs, evs, scs, rates, golden = [], [], [], [], []
    for i in idx:
        d = os.path.join(batch_dir, str(i))
        L = int(_read(os.path.join(d, "read_len[i].dat"), "<i4", 1)[0])
        seq = _read(os.path.join(d, "read[i].dat"), np.uint8, L).tobytes()
        if len(seq) != L:
            raise ValueError(f"read {i}: short sequence")
        with open(os.path.join(d, "et[i].dat"), "rb") as f:
            hdr = np.frombuffer(f.read(32), dtype="<u8")
            ne = int(hdr[0])
            ev = np.frombuffer(f.read(24 * ne), dtype=EVENT_DTYPE).copy()
        if len(ev) != ne:
            raise ValueError(f"read {i}: short event table")
        seqs.append(seq)
        evs.append(ev)
        scs.append(_read(os.path.join(d, "scalings[i].dat"), SCALINGS_DTYPE, 1)[0])
        rates.append(float(_read(os.path.join(d, "f5[i].sample_rate.dat"), "<f4", 1)[0]))
        if with_outputs:
            npairs = int(_read(os.path.join(d, "n_event_align_pairs[i].dat"), "<i4", 1)[0])
            golden.append(_read(os.path.join(d, "event_align_pairs.dat"), PAIR_DTYPE, npairs))
    batch = from_reads(seqs, evs, np.array(scs, dtype=SCALINGS_DTYPE), model,
                       meta={"sample_rate": rates, "source": batch_dir})
    return batch, (golden if with_outputs else None)


def write_batch(batch_dir: str, batch: Batch, pairs_per_read=None, sample_rate: float = 4000.0):
    """Writes a batch (and optionally per-read AlignedPair answers) in the dump layout."""
    os.makedirs(batch_dir, exist_ok=True)
    np.array([batch.n_reads], dtype="<i4").tofile(os.path.join(batch_dir, "n_bam_rec.dat"))
    np.asarray(batch.model, dtype=MODEL_DTYPE).tofile(os.path.join(batch_dir, "model.dat"))
    for i in range(batch.n_reads):
        d = os.path.join(batch_dir, str(i))
        os.makedirs(d, exist_ok=True)
        np.array([batch.read_len[i]], dtype="<i4").tofile(os.path.join(d, "read_len[i].dat"))
        with open(os.path.join(d, "read[i].dat"), "wb") as f:
            f.write(batch.sequence(i))
        ev = batch.read_events(i)
        with open(os.path.join(d, "et[i].dat"), "wb") as f:
            f.write(np.array([len(ev), 0, len(ev), 0], dtype="<u8").tobytes())
            f.write(np.ascontiguousarray(ev).tobytes())
        np.asarray(batch.scalings[i : i + 1], dtype=SCALINGS_DTYPE).tofile(
            os.path.join(d, "scalings[i].dat"))
        np.array([sample_rate], dtype="<f4").tofile(os.path.join(d, "f5[i].sample_rate.dat"))
        if pairs_per_read is not None:
            p = np.asarray(pairs_per_read[i], dtype=PAIR_DTYPE)
            np.array([len(p)], dtype="<i4").tofile(os.path.join(d, "n_event_align_pairs[i].dat"))
            p.tofile(os.path.join(d, "event_align_pairs.dat"))


def write_dump(dump_dir: str, batches, answers=None):
    os.makedirs(dump_dir, exist_ok=True)
    np.array([len(batches)], dtype="<i4").tofile(os.path.join(dump_dir, "no_of_batches.dat"))
    for b, batch in enumerate(batches):
        write_batch(os.path.join(dump_dir, str(b)), batch,
                    None if answers is None else answers[b])
