"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product library never
calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

LOG_UNCACHED = 0x1
QC_FLOAT = 0x2
VAR_AWARE = 0x4

EVENT_DTYPE = np.dtype(
    [("start", "<u8"), ("length", "<f4"), ("mean", "<f4"), ("stdv", "<f4"), ("_pad", "<u4")])
MODEL_DTYPE = np.dtype([("level_mean", "<f4"), ("level_stdv", "<f4"), ("level_log_stdv", "<f4")])
SCALINGS_DTYPE = np.dtype([("scale", "<f4"), ("shift", "<f4"), ("var", "<f4"), ("log_var", "<f4")])
PAIR_DTYPE = np.dtype([("ref_pos", "<i4"), ("read_pos", "<i4")])
EKPAIR_DTYPE = np.dtype([("event_idx", "<i4"), ("kmer_idx", "<i4")])
INDEX_PAIR_DTYPE = np.dtype([("start", "<i4"), ("stop", "<i4")])
EVENT_ALIGNMENT_DTYPE = np.dtype({
    "names": ["ref_kmer", "ref_position", "read_idx", "event_idx", "rc", "model_kmer", "hmm_state"],
    "formats": ["S7", "<i4", "<i4", "<i4", "u1", "S7", "S1"],
    "offsets": [0, 8, 12, 16, 20, 21, 28],
    "itemsize": 32,
})


class _Scalings(C.Structure):
    _fields_ = [("scale", C.c_float), ("shift", C.c_float), ("var", C.c_float), ("log_var", C.c_float)]


class _Debug(C.Structure):
    _fields_ = [
        ("bands", C.c_void_p), ("trace", C.c_void_p), ("band_lower_left", C.c_void_p),
        ("best_score", C.c_float), ("best_event", C.c_int32), ("sum_emission", C.c_double),
        ("path_len", C.c_int32), ("max_gap", C.c_int32), ("last_from", C.c_int32),
    ]


def build(quiet: bool = True) -> str:
    subprocess.run(["make", "-C", HERE], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.oracle_align.restype = C.c_int32
        L.oracle_align.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_int32, C.c_void_p,
                                   C.c_int32, C.c_void_p, _Scalings, C.c_uint32, C.POINTER(_Debug)]
        L.oracle_align_f64.restype = C.c_int32
        L.oracle_align_f64.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_int32, C.c_void_p,
                                       C.c_int32, C.c_void_p, _Scalings, C.c_uint32,
                                       C.POINTER(C.c_double)]
        L.oracle_align_batch.restype = None
        L.oracle_align_batch.argtypes = [C.c_int32] + [C.c_void_p] * 11 + [C.c_uint32, C.c_int]
        L.oracle_align_f64_batch.restype = None
        L.oracle_align_f64_batch.argtypes = [C.c_int32] + [C.c_void_p] * 11 + [C.c_uint32, C.c_int]
        L.oracle_emission.restype = C.c_float
        L.oracle_emission.argtypes = [C.c_float, C.c_void_p, _Scalings, C.c_uint32]
        L.oracle_add3.restype = C.c_float
        L.oracle_add3.argtypes = [C.c_float, C.c_double, C.c_float]
        L.oracle_path_adjoint.restype = C.c_double
        L.oracle_path_adjoint.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_char_p, C.c_void_p,
                                          C.c_void_p, _Scalings, C.c_void_p, C.c_int32, C.c_double,
                                          C.c_double, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_mom.restype = None
        L.oracle_mom.argtypes = [C.c_char_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                 C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.oracle_postalign.restype = C.c_int32
        L.oracle_postalign.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_double), C.c_char_p,
                                       C.c_int32, C.c_void_p, C.c_int32, C.c_int32]
        L.oracle_n_bands.restype = C.c_int64
        L.oracle_n_bands.argtypes = [C.c_int32, C.c_int32]
        _lib = L
    return _lib


def _sc(s) -> _Scalings:
    return _Scalings(float(s["scale"]), float(s["shift"]), float(s["var"]), float(s["log_var"]))


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def align(seq: bytes, events: np.ndarray, model: np.ndarray, scalings, flags: int = 0,
          capacity: int | None = None, want_bands: bool = False):
    """One read.  Returns (pairs, count, info) where info holds best_score,
    sum_emission, path_len, max_gap and (with want_bands) bands/trace/bll in
    the reference layout."""
    L = lib()
    events = np.ascontiguousarray(events, dtype=EVENT_DTYPE)
    model = np.ascontiguousarray(model, dtype=MODEL_DTYPE)
    n_ev = len(events)
    cap = 2 * n_ev if capacity is None else capacity
    out = np.zeros(max(cap, 1), dtype=PAIR_DTYPE)
    dbg = _Debug()
    nb = int(L.oracle_n_bands(len(seq), n_ev))
    bands = trace = bll = None
    if want_bands and nb > 0 and n_ev > 0 and len(seq) >= 6:
        bands = np.zeros(nb * 100, dtype=np.float32)
        trace = np.zeros(nb * 100, dtype=np.uint8)
        bll = np.zeros(nb, dtype=EKPAIR_DTYPE)
        dbg.bands, dbg.trace, dbg.band_lower_left = _ptr(bands), _ptr(trace), _ptr(bll)
    n = L.oracle_align(_ptr(out), cap, bytes(seq), len(seq), _ptr(events), n_ev, _ptr(model),
                       _sc(scalings), flags, C.byref(dbg))
    # the path in walk order (best end first): reversed on success, as walked otherwise
    if n > 0:
        walk = out[:n][::-1].copy()
    else:
        walk = out[: min(dbg.path_len, cap)].copy()
    info = dict(best_score=dbg.best_score, best_event=dbg.best_event,
                sum_emission=dbg.sum_emission, path_len=dbg.path_len, max_gap=dbg.max_gap,
                last_from=dbg.last_from, walk=walk, bands=bands, trace=trace, bll=bll)
    return out[: max(n, 0)], n, info


def align_f64(seq: bytes, events, model, scalings, flags: int = 0):
    L = lib()
    events = np.ascontiguousarray(events, dtype=EVENT_DTYPE)
    model = np.ascontiguousarray(model, dtype=MODEL_DTYPE)
    cap = 2 * len(events)
    out = np.zeros(max(cap, 1), dtype=PAIR_DTYPE)
    best = C.c_double()
    n = L.oracle_align_f64(_ptr(out), cap, bytes(seq), len(seq), _ptr(events), len(events),
                           _ptr(model), _sc(scalings), flags, C.byref(best))
    return out[: max(n, 0)], n, best.value


def align_batch(batch, flags: int = 0, threads: int | None = None):
    """Flattened batch (abea types.Batch); returns (pairs, counts, best_scores)."""
    L = lib()
    n = batch.n_reads
    pairs = np.zeros(max(batch.pair_capacity(), 1), dtype=PAIR_DTYPE)
    counts = np.zeros(n, dtype=np.int32)
    best = np.zeros(n, dtype=np.float32)
    arrs = [np.ascontiguousarray(a) for a in (
        batch.read, batch.read_ptr.astype(np.int64), batch.read_len.astype(np.int32),
        np.asarray(batch.events, dtype=EVENT_DTYPE), batch.event_ptr.astype(np.int64),
        batch.n_events.astype(np.int32), np.asarray(batch.scalings, dtype=SCALINGS_DTYPE),
        np.asarray(batch.model, dtype=MODEL_DTYPE))]
    L.oracle_align_batch(n, *[_ptr(a) for a in arrs], _ptr(pairs), _ptr(counts), _ptr(best),
                         flags, threads or os.cpu_count() or 1)
    return pairs, counts, best


def align_batch_f64(batch, flags: int = 0, threads: int | None = None):
    """The all-FP64 recurrence (oracle_align_f64) over a flattened batch; returns
    (pairs, counts, best_scores as float64)."""
    L = lib()
    n = batch.n_reads
    pairs = np.zeros(max(batch.pair_capacity(), 1), dtype=PAIR_DTYPE)
    counts = np.zeros(n, dtype=np.int32)
    best = np.zeros(n, dtype=np.float64)
    arrs = [np.ascontiguousarray(a) for a in (
        batch.read, batch.read_ptr.astype(np.int64), batch.read_len.astype(np.int32),
        np.asarray(batch.events, dtype=EVENT_DTYPE), batch.event_ptr.astype(np.int64),
        batch.n_events.astype(np.int32), np.asarray(batch.scalings, dtype=SCALINGS_DTYPE),
        np.asarray(batch.model, dtype=MODEL_DTYPE))]
    L.oracle_align_f64_batch(n, *[_ptr(a) for a in arrs], _ptr(pairs), _ptr(counts), _ptr(best),
                             flags, threads or os.cpu_count() or 1)
    return pairs, counts, best


def fp64_error(batch, best32, pairs32, counts32, threads: int | None = None) -> dict:
    """How far the reference's FP32 results lie from the all-FP64 recurrence on
    the same inputs: relative error of the best-end scores (reads with a finite
    end in both), and the reads whose AlignedPairs or pair counts differ."""
    p64, c64, b64 = align_batch_f64(batch, threads=threads)
    b32 = np.asarray(best32, dtype=np.float64)
    fin = np.isfinite(b32) & np.isfinite(b64)
    rel = np.abs(b32[fin] - b64[fin]) / np.maximum(np.abs(b64[fin]), 1e-300)
    diff_counts = int(np.count_nonzero(np.asarray(counts32) != c64))
    diff_pairs = 0
    for i in range(batch.n_reads):
        o, n32, n64 = 2 * int(batch.event_ptr[i]), int(counts32[i]), int(c64[i])
        if n32 != n64 or (n32 > 0 and not np.array_equal(pairs32[o:o + n32], p64[o:o + n64])):
            diff_pairs += 1
    return {"reads": int(batch.n_reads), "finite_ends": int(fin.sum()),
            "best_score_rel_err_max": float(rel.max()) if rel.size else 0.0,
            "best_score_rel_err_median": float(np.median(rel)) if rel.size else 0.0,
            "best_score_rel_err_p99": float(np.percentile(rel, 99)) if rel.size else 0.0,
            "reads_with_other_pair_count": diff_counts,
            "reads_with_other_pairs": diff_pairs,
            "reads_passing_qc_fp32": int(np.count_nonzero(np.asarray(counts32) > 0)),
            "reads_passing_qc_fp64": int(np.count_nonzero(c64 > 0))}


def emission(x: float, model_entry, scalings, flags: int = 0) -> float:
    m = np.ascontiguousarray(np.asarray([model_entry], dtype=MODEL_DTYPE))
    return float(lib().oracle_emission(x, _ptr(m), _sc(scalings), flags))


def path_adjoint(walk, last_from: int, seq: bytes, events, model, scalings, flags: int = 0,
                 theta=None, kmer: int = -1, d_mean: float = 0.0, d_stdv: float = 0.0,
                 want_model: bool = False):
    """FP64 adjoint of one fixed path (walk order, best end first).  Returns
    (emission_sum, grad[shift, scale, var], gn[5], grad_model[4096,2] or None)."""
    walk = np.ascontiguousarray(walk, dtype=PAIR_DTYPE)
    events = np.ascontiguousarray(events, dtype=EVENT_DTYPE)
    model = np.ascontiguousarray(model, dtype=MODEL_DTYPE)
    g = np.zeros(3)
    gn = np.zeros(5)
    gm = np.zeros((4096, 2)) if want_model else None
    th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
    em = lib().oracle_path_adjoint(_ptr(walk), len(walk), int(last_from), bytes(seq), _ptr(events),
                                   _ptr(model), _sc(scalings), _ptr(th), int(kmer), float(d_mean),
                                   float(d_stdv), flags, _ptr(g), _ptr(gn), _ptr(gm))
    return em, g, gn, gm


def mom(seq: bytes, events, model):
    """Method-of-moments (scale, shift) of one read, FP64."""
    events = np.ascontiguousarray(events, dtype=EVENT_DTYPE)
    model = np.ascontiguousarray(model, dtype=MODEL_DTYPE)
    sc, sh = C.c_double(), C.c_double()
    lib().oracle_mom(bytes(seq), len(seq), _ptr(events), len(events), _ptr(model), C.byref(sc), C.byref(sh))
    return sc.value, sh.value


def postalign(seq: bytes, pairs, read_idx: int = 0, out_cap: int | None = None):
    """f5c's postalign of one read's AlignedPairs: (records, base_to_event_map,
    events_per_base, status); status is the record count or a negative code."""
    pairs = np.asarray(pairs)
    if pairs.dtype != PAIR_DTYPE:  # an [n, 2] integer array of (ref_pos, read_pos)
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2).view(PAIR_DTYPE).reshape(-1)
    pairs = np.ascontiguousarray(pairs)
    nk = max(len(seq) - 5, 0)
    cap = len(pairs) if out_cap is None else out_cap
    rec = np.zeros(max(cap, 1), dtype=EVENT_ALIGNMENT_DTYPE)
    bmap = np.zeros(max(nk, 1), dtype=INDEX_PAIR_DTYPE)
    epb = C.c_double()
    n = lib().oracle_postalign(_ptr(rec), cap, _ptr(bmap), C.byref(epb), bytes(seq), nk, _ptr(pairs), len(pairs),
                               int(read_idx))
    return rec[: max(n, 0)], bmap[:nk], epb.value, n


def postalign_batch(batch, pairs, counts):
    """postalign over a batch's flattened AlignedPairs, in the layout of
    abea_batch_postalign: (records [events], map [max(read_ptr + read_len)], events_per_base,
    n_alignment)."""
    n = batch.n_reads
    n_rec = int((batch.event_ptr + batch.n_events).max()) if n else 0
    n_map = int((batch.read_ptr + batch.read_len).max()) if n else 0
    rec = np.zeros(n_rec, dtype=EVENT_ALIGNMENT_DTYPE)
    bmap = np.full(n_map, -1, dtype=INDEX_PAIR_DTYPE)
    epb = np.zeros(n)
    cnt = np.zeros(n, dtype=np.int32)
    for i in range(n):
        e, c, p = int(batch.event_ptr[i]), max(int(counts[i]), 0), int(batch.read_ptr[i])
        seq = batch.read[p : p + int(batch.read_len[i])].tobytes()
        r, m, epb[i], cnt[i] = postalign(seq, pairs[2 * e : 2 * e + c], i, out_cap=int(batch.n_events[i]))
        rec[e : e + len(r)] = r
        bmap[p : p + len(m)] = m
    return rec, bmap, epb, cnt


def add3(a: float, b: float, c: float) -> float:
    return float(lib().oracle_add3(a, b, c))


# ---- the reference's own code, compiled by oracle/build_ref.sh (if present) ----
REF_LIB = os.path.join(HERE, "_ref", "libref.so")
_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_LIB)
        R.ref_align.restype = C.c_int32
        R.ref_align.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_int32, C.c_void_p,
                                C.c_int32, C.c_void_p, _Scalings, C.c_void_p, C.c_void_p,
                                C.c_void_p]
        _ref = R
    return _ref


def ref_align(seq: bytes, events, model, scalings, want_bands: bool = False):
    """One read through the reference's SWI fill + host post (float QC sum)."""
    R = ref_lib()
    events = np.ascontiguousarray(events, dtype=EVENT_DTYPE)
    model = np.ascontiguousarray(model, dtype=MODEL_DTYPE)
    n_ev = len(events)
    cap = 2 * n_ev + len(seq) + 8
    out = np.zeros(max(cap, 1), dtype=PAIR_DTYPE)
    nb = n_ev + len(seq) - 5 + 2
    bands = trace = bll = None
    if want_bands and n_ev > 0 and len(seq) >= 6:
        bands = np.zeros(nb * 100, dtype=np.float32)
        trace = np.zeros(nb * 100, dtype=np.uint8)
        bll = np.zeros(nb, dtype=EKPAIR_DTYPE)
    n = R.ref_align(_ptr(out), cap, bytes(seq), len(seq), _ptr(events), n_ev, _ptr(model),
                    _sc(scalings), _ptr(bands), _ptr(trace), _ptr(bll))
    return out[: max(n, 0)], n, dict(bands=bands, trace=trace, bll=bll)
