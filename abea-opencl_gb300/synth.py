"""Seeded synthetic nanopore batches with the shapes of the benchmark workloads.

The reference measures on f5c's `ecoli_2kb_region` batches (README.md:37-41),
which are not available here; these generators stand in for them with the
value distributions of the reference's golden dump (FPGA/code/bins/dump_small):

  pore model : 4096 6-mers, level_mean ~ U(60,130) pA, level_stdv ~ U(1,3) pA,
               level_log_stdv = (float)log((double)level_stdv)
  reference  : i.i.d. uniform ACGT
  events     : per k-mer, skipped with p=0.05, else Geometric(mean 1.8, >=1)
               events; mean = level_mean*scale + shift + N(0,(level_stdv*var)^2);
               start/length in samples at 4000 Hz (length >= 3, mean ~5)
  scalings   : scale ~ N(1,0.05), shift ~ N(0,5), var = 1.2, log_var = log(1.2)

Workloads (reads / length law):
  small       64 reads, U(1000,3000)
  f5c_batch   1.3 Mbases, lognormal(median 3 kb, sigma 0.6) clipped to [500, 20000]
  uneven      1.3 Mbases, 80% U(200,5000) + 20% U(20000,100000)
  adjoint     4096 reads, U(1000,10000)
  reads1024   1024 reads, U(1000,10000) (a batch with fewer reads than warps)
  serving     200 Mbases, lognormal(median 8 kb, sigma 0.6) clipped to [500, 200000]
"""
from __future__ import annotations

import numpy as np

from .types import EVENT_DTYPE, KMER_SIZE, MODEL_DTYPE, NUM_KMER, SCALINGS_DTYPE, Batch

_BASES = np.frombuffer(b"ACGT", dtype=np.uint8)
SAMPLE_RATE = 4000.0
LOGNORMAL_SIGMA = 0.6


def make_model(rng: np.random.Generator) -> np.ndarray:
    m = np.zeros(NUM_KMER, dtype=MODEL_DTYPE)
    m["level_mean"] = rng.uniform(60.0, 130.0, NUM_KMER).astype(np.float32)
    m["level_stdv"] = rng.uniform(1.0, 3.0, NUM_KMER).astype(np.float32)
    m["level_log_stdv"] = np.log(m["level_stdv"].astype(np.float64)).astype(np.float32)
    return m


def kmer_ranks(seq: np.ndarray) -> np.ndarray:
    """6-mer ranks of a uint8 ACGT array (first base most significant)."""
    code = np.zeros(256, dtype=np.int64)
    code[ord("C")] = 1
    code[ord("G")] = 2
    code[ord("T")] = 3
    c = code[seq]
    n = len(seq) - KMER_SIZE + 1
    if n <= 0:
        return np.zeros(0, dtype=np.int64)
    r = np.zeros(n, dtype=np.int64)
    for j in range(KMER_SIZE):
        r = (r << 2) | c[j : j + n]
    return r


def read_lengths(rng: np.random.Generator, workload: str, target=None) -> np.ndarray:
    if workload == "small":
        return rng.integers(1000, 3001, 64)
    if workload == "adjoint":
        return rng.integers(1000, 10001, 4096)
    if workload == "reads1024":
        return rng.integers(1000, 10001, 1024)
    if workload in ("f5c_batch", "uneven", "serving"):
        if target is None:
            target = 200_000_000 if workload == "serving" else 1_300_000
        lens = []
        total = 0
        while total < target:
            if workload == "uneven":
                L = rng.integers(200, 5001) if rng.random() < 0.8 else rng.integers(20000, 100001)
            else:
                med = 8000.0 if workload == "serving" else 3000.0
                hi = 200000 if workload == "serving" else 20000
                L = int(np.clip(rng.lognormal(np.log(med), LOGNORMAL_SIGMA), 500, hi))
            lens.append(int(L))
            total += int(L)
        return np.array(lens, dtype=np.int64)
    raise ValueError(f"unknown workload {workload!r}")


def make_read(rng, model, length, scale, shift, var, skip_p=0.05, mean_events=1.8):
    seq = _BASES[rng.integers(0, 4, int(length))]
    ranks = kmer_ranks(seq)
    nk = len(ranks)
    counts = rng.geometric(1.0 / mean_events, nk)
    counts[rng.random(nk) < skip_p] = 0
    kidx = np.repeat(np.arange(nk), counts)
    r = ranks[kidx]
    ev = np.zeros(len(kidx), dtype=EVENT_DTYPE)
    mu = model["level_mean"][r].astype(np.float64) * scale + shift
    sd = model["level_stdv"][r].astype(np.float64) * var
    ev["mean"] = (mu + rng.standard_normal(len(kidx)) * sd).astype(np.float32)
    length_s = 3 + rng.geometric(0.5, len(kidx)) - 1
    length_s = np.minimum(length_s, 34)
    ev["length"] = length_s.astype(np.float32)
    ev["start"] = np.concatenate([[0], np.cumsum(length_s[:-1])]).astype(np.uint64) if len(kidx) else 0
    ev["stdv"] = (model["level_stdv"][r] * rng.uniform(0.8, 1.2, len(kidx))).astype(np.float32)
    return seq, ev


def make_batch(workload: str = "small", seed: int = 1, perturb: bool = False, lengths=None) -> Batch:
    """A flattened synthetic batch.  `perturb` (adjoint workload) returns
    scalings offset from the truth by shift +-8 pA and scale +-10%.  "f5c_longest"
    is the f5c batch's longest read alone (its band chain sets the batch's time)."""
    if workload == "f5c_longest":
        full = make_batch("f5c_batch", seed=seed, perturb=perturb)
        return full.subset(np.array([int(np.argmax(full.n_bands()))]))
    rng = np.random.default_rng(seed)
    model = make_model(rng)
    lens = np.asarray(lengths if lengths is not None else read_lengths(rng, workload), dtype=np.int64)
    n = len(lens)
    true_sc = np.zeros(n, dtype=SCALINGS_DTYPE)
    true_sc["scale"] = rng.normal(1.0, 0.05, n).astype(np.float32)
    true_sc["shift"] = rng.normal(0.0, 5.0, n).astype(np.float32)
    true_sc["var"] = np.float32(1.2)
    true_sc["log_var"] = np.float32(np.log(1.2))
    seq_total = int(lens.sum()) + n
    read = np.zeros(seq_total, dtype=np.uint8)
    read_ptr = np.zeros(n, dtype=np.int64)
    evs = []
    p = 0
    for i in range(n):
        seq, ev = make_read(
            rng, model, lens[i], float(true_sc["scale"][i]), float(true_sc["shift"][i]), 1.2
        )
        read_ptr[i] = p
        read[p : p + len(seq)] = seq
        p += len(seq) + 1
        evs.append(ev)
    n_events = np.array([len(e) for e in evs], dtype=np.int32)
    event_ptr = np.zeros(n, dtype=np.int64)
    if n:
        event_ptr[1:] = np.cumsum(n_events[:-1].astype(np.int64))
    events = np.concatenate(evs) if n else np.zeros(0, dtype=EVENT_DTYPE)
    sc = true_sc.copy()
    if perturb:
        sc["shift"] = (true_sc["shift"] + rng.uniform(-8, 8, n)).astype(np.float32)
        sc["scale"] = (true_sc["scale"] * (1.0 + rng.uniform(-0.1, 0.1, n))).astype(np.float32)
    return Batch(
        read=read,
        read_ptr=read_ptr,
        read_len=lens.astype(np.int32),
        events=events,
        event_ptr=event_ptr,
        n_events=n_events,
        scalings=sc,
        model=model,
        meta={"workload": workload, "seed": seed, "true_scalings": true_sc,
              "sample_rate": SAMPLE_RATE, "lognormal_sigma": LOGNORMAL_SIGMA},
    )



def _stream_chunk(seed_seq, model, lens, sc):
    """Sequences and events of one chunk of reads (make_stream)."""
    rng = np.random.default_rng(seed_seq)
    L = lens.astype(np.int64)
    m = len(L)
    tot = int(L.sum())
    starts = np.zeros(m, dtype=np.int64)
    starts[1:] = np.cumsum(L[:-1])
    codes = rng.integers(0, 4, tot).astype(np.uint8)
    seq = _BASES[codes]
    # k-mer ranks at every position; drop the ones that cross a read's end
    nw = tot - KMER_SIZE + 1
    r = np.zeros(nw, dtype=np.int32)
    for j in range(KMER_SIZE):
        r = (r << 2) | codes[j:j + nw]
    valid = np.ones(nw, dtype=bool)
    tail = ((starts + L)[:, None] - KMER_SIZE + 1 + np.arange(KMER_SIZE - 1)[None, :]).ravel()
    valid[tail[tail < nw]] = False
    ranks = r[valid]
    kread = np.repeat(np.arange(m, dtype=np.int32), L - KMER_SIZE + 1)
    counts = rng.geometric(1.0 / 1.8, len(ranks))
    counts[rng.random(len(ranks)) < 0.05] = 0
    kidx = np.repeat(np.arange(len(ranks), dtype=np.int64), counts)
    rk = ranks[kidx]
    eread = kread[kidx]
    ne = len(kidx)
    ev = np.zeros(ne, dtype=EVENT_DTYPE)
    mu = (model["level_mean"].astype(np.float64)[rk] * sc["scale"].astype(np.float64)[eread]
          + sc["shift"].astype(np.float64)[eread])
    sd = model["level_stdv"].astype(np.float64)[rk] * 1.2
    ev["mean"] = (mu + rng.standard_normal(ne) * sd).astype(np.float32)
    length_s = np.minimum(3 + rng.geometric(0.5, ne) - 1, 34)
    ev["length"] = length_s.astype(np.float32)
    cnt = np.bincount(eread, minlength=m).astype(np.int32)
    first = np.zeros(m, dtype=np.int64)
    first[1:] = np.cumsum(cnt[:-1])
    excl = np.cumsum(length_s) - length_s
    ev["start"] = (excl - excl[first[eread]]).astype(np.uint64)
    ev["stdv"] = (model["level_stdv"][rk] * rng.uniform(0.8, 1.2, ne)).astype(np.float32)
    return seq, starts, ev, cnt


def make_stream(seed: int = 1, total_bases: int = 200_000_000, chunk_reads: int = 512, threads=None) -> Batch:
    """The serving workload (lognormal lengths, median 8 kb, clipped to
    [500, 200000], `total_bases` in all) with the laws of make_read, generated a
    chunk of reads at a time with array operations, chunks on a thread pool, each
    chunk from its own child seed (the result does not depend on `threads`; the
    random stream differs from make_batch's)."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(np.random.SeedSequence(seed, spawn_key=(0,)))
    model = make_model(rng)
    lens = read_lengths(rng, "serving", target=total_bases)
    n = len(lens)
    true_sc = np.zeros(n, dtype=SCALINGS_DTYPE)
    true_sc["scale"] = rng.normal(1.0, 0.05, n).astype(np.float32)
    true_sc["shift"] = rng.normal(0.0, 5.0, n).astype(np.float32)
    true_sc["var"] = np.float32(1.2)
    true_sc["log_var"] = np.float32(np.log(1.2))
    read_ptr = np.zeros(n, dtype=np.int64)
    read_ptr[1:] = np.cumsum(lens[:-1] + 1)
    read = np.zeros(int(lens.sum()) + n, dtype=np.uint8)
    bounds = list(range(0, n, chunk_reads))
    chunk_seeds = np.random.SeedSequence(seed, spawn_key=(1,)).spawn(len(bounds))
    with ThreadPoolExecutor(max_workers=threads or min(16, os.cpu_count() or 1)) as pool:
        parts = list(pool.map(lambda k: _stream_chunk(chunk_seeds[k], model, lens[bounds[k]:bounds[k] + chunk_reads],
                                                      true_sc[bounds[k]:bounds[k] + chunk_reads]),
                              range(len(bounds))))
    n_events = np.zeros(n, dtype=np.int32)
    for k, (seq, starts, _, cnt) in enumerate(parts):
        a = bounds[k]
        n_events[a:a + len(cnt)] = cnt
        for j in range(len(cnt)):  # NUL-separated, as make_batch lays them out
            p = read_ptr[a + j]
            read[p:p + lens[a + j]] = seq[starts[j]:starts[j] + lens[a + j]]
    event_ptr = np.zeros(n, dtype=np.int64)
    if n:
        event_ptr[1:] = np.cumsum(n_events[:-1].astype(np.int64))
    events = np.concatenate([p[2] for p in parts]) if parts else np.zeros(0, dtype=EVENT_DTYPE)
    return Batch(
        read=read, read_ptr=read_ptr, read_len=lens.astype(np.int32), events=events, event_ptr=event_ptr,
        n_events=n_events, scalings=true_sc.copy(), model=model,
        meta={"workload": "serving", "seed": seed, "true_scalings": true_sc, "sample_rate": SAMPLE_RATE,
              "lognormal_sigma": LOGNORMAL_SIGMA, "total_bases": int(lens.sum())},
    )
