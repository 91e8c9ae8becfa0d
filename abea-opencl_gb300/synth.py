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


def read_lengths(rng: np.random.Generator, workload: str) -> np.ndarray:
    if workload == "small":
        return rng.integers(1000, 3001, 64)
    if workload == "adjoint":
        return rng.integers(1000, 10001, 4096)
    if workload in ("f5c_batch", "uneven", "serving"):
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
    scalings offset from the truth by shift +-8 pA and scale +-10%."""
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
