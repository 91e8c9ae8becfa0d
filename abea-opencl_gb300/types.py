"""NumPy mirrors of the reference's shared C types (GPU/f5c.h:113-207) and the
flattened batch layout of align_ocl() (GPU/align_cuda.c:432-497)."""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

KMER_SIZE = 6
NUM_KMER = 4096
BANDWIDTH = 100

# event_t: u64 start; f32 length, mean, stdv; 4 bytes of tail padding (24 B).
EVENT_DTYPE = np.dtype(
    [("start", "<u8"), ("length", "<f4"), ("mean", "<f4"), ("stdv", "<f4"), ("_pad", "<u4")]
)
# model_t with CACHED_LOG (12 B).
MODEL_DTYPE = np.dtype([("level_mean", "<f4"), ("level_stdv", "<f4"), ("level_log_stdv", "<f4")])
# scalings_t with CACHED_LOG (16 B).
SCALINGS_DTYPE = np.dtype([("scale", "<f4"), ("shift", "<f4"), ("var", "<f4"), ("log_var", "<f4")])
# AlignedPair (8 B).
PAIR_DTYPE = np.dtype([("ref_pos", "<i4"), ("read_pos", "<i4")])
# EventKmerPair (8 B).
EKPAIR_DTYPE = np.dtype([("event_idx", "<i4"), ("kmer_idx", "<i4")])

# index_pair_t (8 B) and event_alignment_t (32 B), the outputs of f5c's postalign
# (GPU/f5c.h:184-207): char ref_kmer[7]; i32 ref_position, read_idx, event_idx;
# bool rc; char model_kmer[7]; char hmm_state.
INDEX_PAIR_DTYPE = np.dtype([("start", "<i4"), ("stop", "<i4")])
EVENT_ALIGNMENT_DTYPE = np.dtype({
    "names": ["ref_kmer", "ref_position", "read_idx", "event_idx", "rc", "model_kmer", "hmm_state"],
    "formats": ["S7", "<i4", "<i4", "<i4", "u1", "S7", "S1"],
    "offsets": [0, 8, 12, 16, 20, 21, 28],
    "itemsize": 32,
})

assert EVENT_DTYPE.itemsize == 24 and MODEL_DTYPE.itemsize == 12
assert SCALINGS_DTYPE.itemsize == 16 and PAIR_DTYPE.itemsize == 8
assert INDEX_PAIR_DTYPE.itemsize == 8 and EVENT_ALIGNMENT_DTYPE.itemsize == 32


def n_kmers_of(read_len):
    return np.asarray(read_len, dtype=np.int64) - KMER_SIZE + 1


def n_bands_of(read_len, n_events):
    """n_events + n_kmers + 2 bands per read (GPU/align_cuda.cl:367-369)."""
    return np.asarray(n_events, dtype=np.int64) + n_kmers_of(read_len) + 2


@dataclass
class Batch:
    """A batch of reads in the reference's flattened layout.

    read      uint8 [sum(read_len+1)]  bases, one NUL after each read
    read_ptr  int64 [n]                offset of read i in `read`
    read_len  int32 [n]
    events    EVENT_DTYPE [sum(n_events)]
    event_ptr int64 [n]
    n_events  int32 [n]
    scalings  SCALINGS_DTYPE [n]
    model     MODEL_DTYPE [4096]
    """

    read: np.ndarray
    read_ptr: np.ndarray
    read_len: np.ndarray
    events: np.ndarray
    event_ptr: np.ndarray
    n_events: np.ndarray
    scalings: np.ndarray
    model: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def n_reads(self) -> int:
        return int(self.read_len.shape[0])

    def n_bands(self) -> np.ndarray:
        return n_bands_of(self.read_len, self.n_events)

    def band_cells(self) -> int:
        """Sum over reads of n_bands * 100."""
        return int(self.n_bands().sum()) * BANDWIDTH

    def sequence(self, i: int) -> bytes:
        p = int(self.read_ptr[i])
        return self.read[p : p + int(self.read_len[i])].tobytes()

    def read_events(self, i: int) -> np.ndarray:
        p = int(self.event_ptr[i])
        return self.events[p : p + int(self.n_events[i])]

    def subset(self, idx) -> "Batch":
        """A new flattened batch holding reads `idx` (in that order)."""
        idx = [int(i) for i in idx]
        seqs = [self.sequence(i) for i in idx]
        evs = [self.read_events(i) for i in idx]
        return from_reads(seqs, evs, self.scalings[idx], self.model, meta=dict(self.meta))

    def pair_capacity(self) -> int:
        return 2 * int(self.n_events.sum())


def from_reads(seqs, event_arrays, scalings, model, meta=None) -> Batch:
    """Flatten per-read sequences and event arrays (GPU/align_cuda.c:432-497)."""
    n = len(seqs)
    read_len = np.array([len(s) for s in seqs], dtype=np.int32)
    read_ptr = np.zeros(n, dtype=np.int64)
    if n:
        read_ptr[1:] = np.cumsum(read_len[:-1].astype(np.int64) + 1)
    total = int(read_len.astype(np.int64).sum()) + n
    read = np.zeros(total, dtype=np.uint8)
    for i, s in enumerate(seqs):
        p = int(read_ptr[i])
        read[p : p + len(s)] = np.frombuffer(bytes(s), dtype=np.uint8)
    n_events = np.array([len(e) for e in event_arrays], dtype=np.int32)
    event_ptr = np.zeros(n, dtype=np.int64)
    if n:
        event_ptr[1:] = np.cumsum(n_events[:-1].astype(np.int64))
    events = (
        np.concatenate([np.asarray(e, dtype=EVENT_DTYPE) for e in event_arrays])
        if n
        else np.zeros(0, dtype=EVENT_DTYPE)
    )
    return Batch(
        read=read,
        read_ptr=read_ptr,
        read_len=read_len,
        events=events,
        event_ptr=event_ptr,
        n_events=n_events,
        scalings=np.ascontiguousarray(np.asarray(scalings, dtype=SCALINGS_DTYPE)),
        model=np.ascontiguousarray(np.asarray(model, dtype=MODEL_DTYPE)),
        meta=dict(meta or {}),
    )


def split_postalign(batch: Batch, out: dict):
    """Per-read (records, base_to_event_map) of a postalign result: read i's
    n_alignment[i] records from event_ptr[i] and its n_kmers map entries from
    read_ptr[i]."""
    res = []
    for i in range(batch.n_reads):
        e, c = int(batch.event_ptr[i]), max(int(out["n_alignment"][i]), 0)
        p, nk = int(batch.read_ptr[i]), max(int(batch.read_len[i]) - KMER_SIZE + 1, 0)
        rec = out["alignment"][e : e + c]
        # a byte copy: ndarray.copy() of a dtype with padding leaves the padding bytes unset
        rec = rec.view(np.uint8).copy().view(rec.dtype)
        res.append((rec, out["base_to_event_map"][p : p + nk].copy()))
    return res


def split_pairs(batch: Batch, pairs: np.ndarray, counts: np.ndarray):
    """Per-read AlignedPair lists out of the flattened output (stride 2*event_ptr)."""
    out = []
    for i in range(batch.n_reads):
        c = int(counts[i])
        p = 2 * int(batch.event_ptr[i])
        out.append(pairs[p : p + max(c, 0)].copy())
    return out
