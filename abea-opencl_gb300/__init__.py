"""GB300-native Adaptive Banded Event Alignment (ABEA) — Python host binding.

Mirrors the reference's interface for f5c's align() path:
  * align(seq, events, model, scalings, sample_rate)  -> AlignedPair array
      f5c `int32_t align(AlignedPair*, char*, int32_t, event_table, model_t*,
      scalings_t, float)` (GPU/f5cmisc.h:48-50)
  * Context.align_batch(batch) -> (pairs, n_pairs)
      the batch entry align_cuda(core, db) / align_ocl(core, db)
      (GPU/f5cmisc.h:99-102, GPU/align_cuda.c:391-943), flattened layout of
      GPU/align_cuda.c:432-497.
Everything runs in the C-ABI library libabea.so (hand-written sm_103a
kernels).  There is no CPU path: if the library or a GB300 is missing, the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import weakref

import numpy as np

from . import types
from .types import (BANDWIDTH, EKPAIR_DTYPE, EVENT_ALIGNMENT_DTYPE, EVENT_DTYPE, INDEX_PAIR_DTYPE, MODEL_DTYPE,
                    PAIR_DTYPE, SCALINGS_DTYPE, Batch, from_reads, split_pairs, split_postalign)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libabea.so")

MODE_PLAIN = 0
MODE_BATCHED = 1
(OPT_MODE, OPT_STORE_SCORES, OPT_USE_GRAPH, OPT_LONG_READ_BANDS, OPT_SPIN_LIMIT, OPT_VAR_AWARE,
 OPT_TRACE_BUDGET, OPT_WIDE_CLUSTER, OPT_MEDIUM_READ_BANDS) = range(9)

STATUS = {
    0: "ok", -1: "invalid argument", -2: "capacity", -3: "out of memory", -4: "CUDA error",
    -5: "timeout", -6: "no device", -7: "internal", -8: "undefined",
}
EXPORTS = [
    "abea_ctx_create", "abea_ctx_destroy", "abea_ctx_set_option", "abea_ctx_get_option",
    "abea_last_error", "abea_status_string", "abea_version", "abea_align", "abea_align_cap",
    "abea_align_batch", "abea_batch_create", "abea_batch_run", "abea_batch_sync",
    "abea_batch_results", "abea_batch_timing", "abea_batch_destroy", "abea_batch_read_bands",
    "abea_batch_best_scores", "abea_batch_slow_cells", "abea_host_alloc", "abea_host_free",
    "abea_ctx_last_timing", "abea_batch_io_bytes", "abea_ctx_mark", "abea_ctx_elapsed",
    "abea_ctx_flush_l2", "abea_selftest_arith", "abea_align_noalloc", "abea_autotune",
    "abea_batch_backward", "abea_batch_set_scalings", "abea_batch_recalibrate",
    "abea_align_db", "abea_batch_estimate_scalings", "abea_batch_postalign", "abea_align_stream", "abea_autotune_save",
    "abea_autotune_load", "abea_align_batch_persistent", "abea_backward_batch",
]


class AbeaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class _Scalings(C.Structure):
    _fields_ = [("scale", C.c_float), ("shift", C.c_float), ("var", C.c_float), ("log_var", C.c_float)]


class _EventTable(C.Structure):
    _fields_ = [("n", C.c_size_t), ("start", C.c_size_t), ("end", C.c_size_t), ("event", C.c_void_p)]


class Timing(C.Structure):
    _fields_ = [("pre_ms", C.c_float), ("core_ms", C.c_float), ("post_ms", C.c_float),
                ("total_ms", C.c_float), ("h2d_ms", C.c_float), ("d2h_ms", C.c_float),
                ("kernel_launches", C.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class StreamConfig(C.Structure):
    _fields_ = [("batch_bytes", C.c_int64), ("recalibrate", C.c_int32), ("reserved", C.c_int32)]


class StreamStats(C.Structure):
    _fields_ = [("n_batches", C.c_int32), ("max_batch_reads", C.c_int32), ("max_batch_bytes", C.c_int64),
                ("band_cells", C.c_int64), ("wall_ms", C.c_double), ("compute_ms", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def build(quiet: bool = True) -> str:
    """Compiles libabea.so in place (nvcc, sm_103a)."""
    subprocess.run(["make", "-C", HERE, "-j4"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


_lib = None


def lib():
    """Loads libabea.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise AbeaError(-6, f"{LIB_PATH} is not built; run build()")
        L = C.CDLL(LIB_PATH)
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        L.abea_ctx_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int]
        L.abea_ctx_destroy.argtypes = [vp]
        L.abea_ctx_destroy.restype = None
        L.abea_ctx_set_option.argtypes = [vp, C.c_int, i64]
        L.abea_ctx_get_option.argtypes = [vp, C.c_int, C.POINTER(i64)]
        L.abea_last_error.restype = C.c_char_p
        L.abea_version.restype = C.c_char_p
        L.abea_status_string.restype = C.c_char_p
        L.abea_status_string.argtypes = [C.c_int]
        L.abea_align.argtypes = [vp, C.c_char_p, i32, _EventTable, vp, _Scalings, C.c_float]
        L.abea_align.restype = i32
        L.abea_align_cap.argtypes = [vp, i32, C.c_char_p, i32, vp, i32, vp, _Scalings]
        L.abea_align_cap.restype = i32
        L.abea_align_batch.argtypes = [vp, i32] + [vp] * 10
        L.abea_align_batch_persistent.argtypes = [vp, i32] + [vp] * 10
        L.abea_backward_batch.argtypes = [vp, vp, vp, vp, vp, vp]
        L.abea_batch_create.argtypes = [vp, i32] + [vp] * 8 + [C.POINTER(vp)]
        L.abea_batch_run.argtypes = [vp, vp]
        L.abea_batch_sync.argtypes = [vp]
        L.abea_batch_results.argtypes = [vp, vp, vp, vp]
        L.abea_batch_timing.argtypes = [vp, vp, C.POINTER(Timing)]
        L.abea_batch_destroy.argtypes = [vp]
        L.abea_batch_destroy.restype = None
        L.abea_batch_read_bands.argtypes = [vp, vp, i32, vp, vp, vp]
        L.abea_batch_best_scores.argtypes = [vp, vp, vp]
        L.abea_batch_slow_cells.argtypes = [vp, vp, C.POINTER(i64)]
        L.abea_host_alloc.argtypes = [C.c_size_t]
        L.abea_host_alloc.restype = vp
        L.abea_host_free.argtypes = [vp]
        L.abea_host_free.restype = None
        L.abea_ctx_last_timing.argtypes = [vp, C.POINTER(Timing), C.POINTER(i64), C.POINTER(i64)]
        L.abea_batch_io_bytes.argtypes = [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]
        L.abea_ctx_mark.argtypes = [vp, C.c_int]
        L.abea_ctx_elapsed.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_float)]
        L.abea_ctx_flush_l2.argtypes = [vp]
        L.abea_selftest_arith.argtypes = [i64, C.c_uint64, vp]
        L.abea_autotune.argtypes = [vp, vp, C.POINTER(i64), C.POINTER(C.c_float)]
        L.abea_batch_backward.argtypes = [vp, vp, vp, vp, vp, vp]
        L.abea_batch_set_scalings.argtypes = [vp, vp, vp]
        L.abea_batch_recalibrate.argtypes = [vp, vp, i32, C.c_double, vp]
        L.abea_align_db.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, vp]
        L.abea_batch_estimate_scalings.argtypes = [vp, vp, vp, i32]
        L.abea_batch_postalign.argtypes = [vp, vp, vp, vp, vp, vp]
        L.abea_align_stream.argtypes = [vp, C.POINTER(StreamConfig), i32] + [vp] * 13
        L.abea_autotune_save.argtypes = [vp, C.c_char_p, C.POINTER(i32)]
        L.abea_autotune_load.argtypes = [vp, C.c_char_p, C.POINTER(i32)]
        _lib = L
    return _lib


def pinned_empty(n: int, dtype) -> np.ndarray:
    """A 1-D array of `n` elements in pinned host memory (abea_host_alloc), freed
    when the array is collected: copies from and to it overlap device work."""
    dt = np.dtype(dtype)
    nbytes = max(int(n) * dt.itemsize, 1)
    p = lib().abea_host_alloc(nbytes)
    if not p:
        raise AbeaError(-3, f"pinned host allocation of {nbytes} bytes failed")
    buf = (C.c_char * nbytes).from_address(p)
    weakref.finalize(buf, lib().abea_host_free, p)
    return np.frombuffer(buf, dtype=dt, count=int(n))


def pin_batch(b: Batch) -> Batch:
    """The batch with every array copied into pinned host memory."""
    def pin(a, dtype):
        a = np.asarray(a, dtype=dtype)
        out = pinned_empty(a.size, dtype)
        out[:] = a.reshape(-1)
        return out
    return Batch(read=pin(b.read, np.uint8), read_ptr=pin(b.read_ptr, np.int64), read_len=pin(b.read_len, np.int32),
                 events=pin(b.events, EVENT_DTYPE), event_ptr=pin(b.event_ptr, np.int64),
                 n_events=pin(b.n_events, np.int32), scalings=pin(b.scalings, SCALINGS_DTYPE),
                 model=pin(b.model, MODEL_DTYPE), meta=dict(b.meta))


def _check(st: int):
    if st != 0:
        raise AbeaError(st, lib().abea_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _sc(s) -> _Scalings:
    return _Scalings(float(s["scale"]), float(s["shift"]), float(s["var"]), float(s["log_var"]))


def _batch_arrays(b: Batch):
    return [np.ascontiguousarray(a) for a in (
        b.read.astype(np.uint8, copy=False), b.read_ptr.astype(np.int64, copy=False),
        b.read_len.astype(np.int32, copy=False), np.asarray(b.events, dtype=EVENT_DTYPE),
        b.event_ptr.astype(np.int64, copy=False), b.n_events.astype(np.int32, copy=False),
        np.asarray(b.scalings, dtype=SCALINGS_DTYPE), np.asarray(b.model, dtype=MODEL_DTYPE))]


class DeviceBatch:
    """A batch resident in HBM (abea_batch_create)."""

    def __init__(self, ctx: "Context", batch: Batch):
        self.ctx = ctx
        self.batch = batch
        self._arrs = _batch_arrays(batch)
        h = C.c_void_p()
        _check(lib().abea_batch_create(ctx.h, batch.n_reads, *[_p(a) for a in self._arrs], C.byref(h)))
        self.h = h

    def run(self):
        _check(lib().abea_batch_run(self.ctx.h, self.h))

    def sync(self):
        _check(lib().abea_batch_sync(self.ctx.h))

    def results(self):
        pairs = np.zeros(max(self.batch.pair_capacity(), 1), dtype=PAIR_DTYPE)
        counts = np.zeros(self.batch.n_reads, dtype=np.int32)
        _check(lib().abea_batch_results(self.ctx.h, self.h, _p(pairs), _p(counts)))
        return pairs, counts

    def timing(self) -> dict:
        t = Timing()
        _check(lib().abea_batch_timing(self.ctx.h, self.h, C.byref(t)))
        return t.as_dict()

    def best_scores(self):
        out = np.zeros(self.batch.n_reads, dtype=np.float32)
        _check(lib().abea_batch_best_scores(self.ctx.h, self.h, _p(out)))
        return out

    def slow_cells(self) -> int:
        v = C.c_int64()
        _check(lib().abea_batch_slow_cells(self.ctx.h, self.h, C.byref(v)))
        return v.value

    def autotune(self):
        """Picks the wide-shape threshold for this workload (abea_autotune)."""
        thr, ms = C.c_int64(), C.c_float()
        _check(lib().abea_autotune(self.ctx.h, self.h, C.byref(thr), C.byref(ms)))
        return thr.value, ms.value

    def backward(self, model_grad: bool = True):
        """Adjoint of the last run (abea_batch_backward): dict with grad_scalings
        [n,3] (d/d shift, scale, var), grad_model [4096,2] (d/d level_mean,
        level_stdv) or None, path_emission [n] and status [n]."""
        n = self.batch.n_reads
        g = np.zeros((max(n, 1), 3))
        gm = np.zeros((4096, 2)) if model_grad else None
        em = np.zeros(max(n, 1))
        st = np.zeros(max(n, 1), dtype=np.int32)
        _check(lib().abea_batch_backward(self.ctx.h, self.h, _p(g), _p(gm), _p(em), _p(st)))
        return dict(grad_scalings=g[:n], grad_model=gm, path_emission=em[:n], status=st[:n])

    def estimate_scalings(self, apply: bool = False):
        """Method-of-moments scalings of every read (abea_batch_estimate_scalings)."""
        out = np.zeros(max(self.batch.n_reads, 1), dtype=SCALINGS_DTYPE)
        _check(lib().abea_batch_estimate_scalings(self.ctx.h, self.h, _p(out), 1 if apply else 0))
        return out[: self.batch.n_reads]

    def postalign(self, outputs: bool = True):
        """f5c's postalign for every read of the last run (abea_batch_postalign):
        dict with alignment [events] (EVENT_ALIGNMENT_DTYPE, read i's records from
        event_ptr[i]), base_to_event_map [max(read_ptr + read_len)] (INDEX_PAIR_DTYPE, read i's
        n_kmers entries from read_ptr[i]), events_per_base [n] and n_alignment [n];
        `split_postalign` cuts them per read.  outputs=False leaves the records, maps
        and events per base on the device (None here) and returns only the counts."""
        b = self.batch
        n = b.n_reads
        n_rec = int((b.event_ptr + b.n_events).max()) if n else 0
        n_map = int((b.read_ptr + b.read_len).max()) if n else 0
        rec = np.zeros(max(n_rec, 1), dtype=EVENT_ALIGNMENT_DTYPE) if outputs else None
        bmap = np.zeros(max(n_map, 1), dtype=INDEX_PAIR_DTYPE) if outputs else None
        epb = np.zeros(max(n, 1)) if outputs else None
        cnt = np.zeros(max(n, 1), dtype=np.int32)
        _check(lib().abea_batch_postalign(self.ctx.h, self.h, _p(rec), _p(bmap), _p(epb), _p(cnt)))
        if not outputs:
            return dict(alignment=None, base_to_event_map=None, events_per_base=None, n_alignment=cnt[:n])
        return dict(alignment=rec[:n_rec], base_to_event_map=bmap[:n_map], events_per_base=epb[:n],
                    n_alignment=cnt[:n])

    def set_scalings(self, scalings):
        sc = np.ascontiguousarray(scalings, dtype=SCALINGS_DTYPE)
        if len(sc) != self.batch.n_reads:
            raise ValueError("one scalings record per read")
        _check(lib().abea_batch_set_scalings(self.ctx.h, self.h, _p(sc)))

    def recalibrate(self, iterations: int = 3, first_temperature: float = 5.0):
        """Annealed Gauss-Newton recalibration of (shift, scale)
        (abea_batch_recalibrate); returns the final scalings, the batch left
        aligned with them."""
        out = np.zeros(max(self.batch.n_reads, 1), dtype=SCALINGS_DTYPE)
        _check(lib().abea_batch_recalibrate(self.ctx.h, self.h, int(iterations), float(first_temperature),
                                            _p(out)))
        return out[: self.batch.n_reads]

    def io_bytes(self):
        h2d, d2h, cells = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().abea_batch_io_bytes(self.h, C.byref(h2d), C.byref(d2h), C.byref(cells)))
        return h2d.value, d2h.value, cells.value

    def read_bands(self, i: int, scores: bool = False):
        """Band matrices of read i in the reference layout: (bands|None, trace, bll)."""
        b = self.batch
        nk = int(b.read_len[i]) - 5
        ne = int(b.n_events[i])
        if nk <= 0 or ne <= 0:
            return None, None, None
        nb = ne + nk + 2
        bands = np.zeros(nb * BANDWIDTH, dtype=np.float32) if scores else None
        trace = np.zeros(nb * BANDWIDTH, dtype=np.uint8)
        bll = np.zeros(nb, dtype=EKPAIR_DTYPE)
        _check(lib().abea_batch_read_bands(self.ctx.h, self.h, i, _p(bands), _p(trace), _p(bll)))
        return bands, trace, bll

    def close(self):
        if getattr(self, "h", None):
            lib().abea_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One CUDA stream and its buffers (abea_ctx_create)."""

    def __init__(self, device: int = 0, mode: int = MODE_PLAIN, store_scores: bool = False):
        h = C.c_void_p()
        _check(lib().abea_ctx_create(C.byref(h), device, mode))
        self.h = h
        if store_scores:
            self.set_option(OPT_STORE_SCORES, 1)

    def set_option(self, opt: int, value: int):
        _check(lib().abea_ctx_set_option(self.h, opt, int(value)))

    def get_option(self, opt: int) -> int:
        v = C.c_int64()
        _check(lib().abea_ctx_get_option(self.h, opt, C.byref(v)))
        return v.value

    def upload(self, batch: Batch) -> DeviceBatch:
        return DeviceBatch(self, batch)

    def align_batch(self, batch: Batch, out_pairs=None, out_counts=None):
        """Host-to-device, align, device-to-host in one call (abea_align_batch)."""
        arrs = _batch_arrays(batch)
        pairs = out_pairs if out_pairs is not None else np.zeros(max(batch.pair_capacity(), 1), dtype=PAIR_DTYPE)
        counts = out_counts if out_counts is not None else np.zeros(batch.n_reads, dtype=np.int32)
        _check(lib().abea_align_batch(self.h, batch.n_reads, *[_p(a) for a in arrs], _p(pairs), _p(counts)))
        return pairs, counts

    def align_db(self, batch: Batch):
        """f5c's per-read arrays (abea_align_db): one read buffer, event table and
        output buffer per read.  Returns (list of per-read pair arrays, counts)."""
        n = batch.n_reads
        reads = [np.ascontiguousarray(batch.read[batch.read_ptr[i]:batch.read_ptr[i] + batch.read_len[i]])
                 for i in range(n)]
        evs = [np.ascontiguousarray(batch.events[batch.event_ptr[i]:batch.event_ptr[i] + batch.n_events[i]],
                                    dtype=EVENT_DTYPE) for i in range(n)]
        outs = [np.zeros(max(2 * int(batch.n_events[i]), 1), dtype=PAIR_DTYPE) for i in range(n)]
        read_p = (C.c_void_p * max(n, 1))(*[r.ctypes.data for r in reads])
        out_p = (C.c_void_p * max(n, 1))(*[o.ctypes.data for o in outs])
        et = (_EventTable * max(n, 1))()
        for i, e in enumerate(evs):
            et[i].n, et[i].start, et[i].end, et[i].event = len(e), 0, len(e), e.ctypes.data
        lens = np.ascontiguousarray(batch.read_len, dtype=np.int32)
        sc = np.ascontiguousarray(batch.scalings, dtype=SCALINGS_DTYPE)
        model = np.ascontiguousarray(batch.model, dtype=MODEL_DTYPE)
        counts = np.zeros(max(n, 1), dtype=np.int32)
        _check(lib().abea_align_db(self.h, n, read_p, _p(lens), C.cast(et, C.c_void_p), _p(sc), _p(model), out_p,
                                   _p(counts)))
        return [outs[i][:max(int(counts[i]), 0)] for i in range(n)], counts[:n]

    def align_stream(self, batch: Batch, batch_bytes: int = 0, recalibrate: bool = False, out_pairs=None,
                     out_counts=None):
        """The batch as a serving stream (abea_align_stream): admitted in order into
        device batches of at most `batch_bytes` (0 = library default), two in
        flight; with `recalibrate`, each device batch is aligned, differentiated,
        given one Gauss-Newton step of (shift, scale) and re-aligned.  Returns a
        dict: pairs, counts, scalings (final per read), latency_ms (per read, from
        its batch's admission to its results on the host) and stats."""
        arrs = _batch_arrays(batch)
        n = batch.n_reads
        pairs = out_pairs if out_pairs is not None else np.zeros(max(batch.pair_capacity(), 1), dtype=PAIR_DTYPE)
        counts = out_counts if out_counts is not None else np.zeros(max(n, 1), dtype=np.int32)
        sc_out = np.zeros(max(n, 1), dtype=SCALINGS_DTYPE)
        lat = np.zeros(max(n, 1), dtype=np.float64)
        cfg = StreamConfig(int(batch_bytes), 1 if recalibrate else 0, 0)
        stats = StreamStats()
        _check(lib().abea_align_stream(self.h, C.byref(cfg), n, *[_p(a) for a in arrs], _p(pairs), _p(counts),
                                       _p(sc_out), _p(lat), C.byref(stats)))
        return {"pairs": pairs, "counts": counts[:n], "scalings": sc_out[:n], "latency_ms": lat[:n],
                "stats": stats.as_dict()}

    def autotune_save(self, path: str) -> int:
        """Writes the autotuner's results to `path` (abea_autotune_save); returns the entry count."""
        n = C.c_int32()
        _check(lib().abea_autotune_save(self.h, os.fsencode(path), C.byref(n)))
        return n.value

    def autotune_load(self, path: str) -> int:
        """Merges an autotuner cache file into this context (abea_autotune_load)."""
        n = C.c_int32()
        _check(lib().abea_autotune_load(self.h, os.fsencode(path), C.byref(n)))
        return n.value

    def last_timing(self):
        t = Timing()
        h2d, d2h = C.c_int64(), C.c_int64()
        _check(lib().abea_ctx_last_timing(self.h, C.byref(t), C.byref(h2d), C.byref(d2h)))
        return t.as_dict(), h2d.value, d2h.value

    def mark(self, i: int):
        _check(lib().abea_ctx_mark(self.h, i))

    def elapsed(self, i: int, j: int) -> float:
        v = C.c_float()
        _check(lib().abea_ctx_elapsed(self.h, i, j, C.byref(v)))
        return v.value

    def flush_l2(self):
        _check(lib().abea_ctx_flush_l2(self.h))

    def close(self):
        if getattr(self, "h", None):
            lib().abea_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def align(seq: bytes, events: np.ndarray, model: np.ndarray, scalings, sample_rate: float = 4000.0):
    """f5c align(): returns the AlignedPair array (empty when QC fails)."""
    events = np.ascontiguousarray(events, dtype=EVENT_DTYPE)
    model = np.ascontiguousarray(model, dtype=MODEL_DTYPE)
    out = np.zeros(max(2 * len(events), 1), dtype=PAIR_DTYPE)
    et = _EventTable(len(events), 0, len(events), events.ctypes.data)
    n = lib().abea_align(_p(out), bytes(seq), len(seq), et, _p(model), _sc(scalings), float(sample_rate))
    if n < 0:
        raise AbeaError(n, lib().abea_last_error().decode())
    return out[:n]


def selftest_arith(cases: int = 1 << 26, seed: int = 1) -> dict:
    """Device self-test of the exact FP32 arithmetic (see include/abea.h)."""
    out = np.zeros(5, dtype=np.int64)
    _check(lib().abea_selftest_arith(int(cases), int(seed), _p(out)))
    return dict(div_wrong=int(out[0]), div_declined=int(out[1]), sum_wrong=int(out[2]),
                sum_declined=int(out[3]), cases=int(out[4]))


def heuristic_wide_reads(n_bands, blocks: int) -> int:
    """How many of the longest reads the batched form runs on the wide shape when
    left to its own heuristic, for a batch with these band counts on `blocks`
    resident blocks (one per SM).  Host code only (abea_internal_wide_threshold)."""
    L = lib()
    f = L.abea_internal_wide_threshold
    f.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    f.restype = C.c_int64
    b = np.ascontiguousarray(n_bands, dtype=np.int64)
    thr = f(b.ctypes.data, len(b), int(blocks))
    if thr < 0:
        raise AbeaError(-1, "abea_internal_wide_threshold: bad argument")
    return 0 if thr >= 2**62 else int(np.sum(b >= thr))


def version() -> str:
    return lib().abea_version().decode()


__all__ = ["align", "Context", "DeviceBatch", "Batch", "from_reads", "split_pairs", "split_postalign", "build", "lib",
           "AbeaError", "MODE_PLAIN", "MODE_BATCHED", "types", "EXPORTS", "version",
           "selftest_arith", "pinned_empty", "pin_batch", "StreamConfig", "StreamStats", "heuristic_wide_reads"]
