#!/usr/bin/env python3
"""ABEA benchmark: band-cells/s (and reads/s) of the GB300 library on the f5c
batch workload, against the reference's CPU align() on the host cores.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one pass of pre/core/post over the whole synthetic batch (1.3 Mbases,
lognormal read lengths, median 3 kb, clipped 500 b - 20 kb), inputs resident in
HBM, L2 flushed before every timed step.  `e2e` is the same metric through
abea_align_batch with pinned host buffers (host->device and device->host copies
inside the timed region).  The headline uses the library's own choice of wide
reads (its heuristic); the autotuner's choices are reported beside it.

Several GPUs: `--gpus N` starts N ranks (one process per GPU) unless the caller
already did (torchrun sets WORLD_SIZE).  Reads are independent, so the path
shards with no collective on the data path: every rank aligns its own batch of
the same shape (seed + rank; weak scaling); the ranks meet only for the timing
maximum and the totals.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
BYTES_PER_CELL = 5  # 4 B score + 1 B backpointer per band cell (the reference's layout)


def load_package():
    pkg_dir = os.path.join(ROOT, "abea-opencl_gb300")
    spec = importlib.util.spec_from_file_location(
        "abea_gb300", os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir])
    m = importlib.util.module_from_spec(spec)
    sys.modules["abea_gb300"] = m
    spec.loader.exec_module(m)
    return m


WORKLOADS = {
    "f5c_batch": "reads totalling 1.3 Mbases, lognormal lengths (median 3 kb, sigma 0.6) clipped to 500 b-20 kb",
    "uneven": "1.3 Mbases: 80% of reads U(200 b, 5 kb), 20% U(20 kb, 100 kb)",
    "small": "64 reads, U(1 kb, 3 kb)",
    "reads1024": "1,024 reads, U(1 kb, 10 kb) (fewer reads than warps: the throughput regime's latency-bound end)",
    "f5c_longest": "the f5c batch's longest read alone (54,382 bands at seed 1): the wide shape's band chain",
}


# ---------------------------------------------------------------- distributed helpers
class Dist:
    """Rank / world from the launcher's environment; a process group only for
    the timing maximum and the totals (NCCL between GPUs, gloo otherwise)."""

    def __init__(self, use_cuda: bool, init: bool = True):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        self.device = None
        if self.world > 1 and init:
            import torch
            import torch.distributed as dist
            if use_cuda:
                torch.cuda.set_device(self.local_rank)
                self.device = torch.device("cuda", self.local_rank)
            dist.init_process_group("nccl" if use_cuda else "gloo")
            self.pg = dist

    def _reduce(self, v: float, op) -> float:
        import torch
        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        self.pg.all_reduce(t, op=op)
        return float(t.item())

    def barrier(self):
        if self.pg:
            self._reduce(0.0, self.pg.ReduceOp.SUM)

    def max(self, v: float) -> float:
        return self._reduce(v, self.pg.ReduceOp.MAX) if self.pg else v

    def sum(self, v: float) -> float:
        return self._reduce(v, self.pg.ReduceOp.SUM) if self.pg else v

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def visible_gpus() -> int:
    """GPUs this process may use: nvidia-smi's list, cut by CUDA_VISIBLE_DEVICES."""
    try:
        out = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=60).stdout
    except (OSError, subprocess.SubprocessError):
        return 0
    n = sum(1 for line in out.splitlines() if line.startswith("GPU "))
    cvd = os.environ.get("CUDA_VISIBLE_DEVICES")
    if cvd is not None:
        n = min(n, len([x for x in cvd.split(",") if x.strip()]))
    return n


def rank_env(rank: int, world: int, port: int) -> dict:
    env = dict(os.environ)
    env.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                "LOCAL_WORLD_SIZE": str(world), "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    return env


def launch_ranks(args) -> int:
    """`--gpus N` without a launcher: one process per GPU (rank r on GPU r), this
    same command line, rendezvous on 127.0.0.1.  Refuses more GPUs than are
    visible (the reference arm runs on the host and needs none)."""
    n = args.gpus
    if args.impl == "ours":
        have = visible_gpus()
        if n > have:
            print(f"bench.py: --gpus {n} but {have} GPU(s) are visible", file=sys.stderr)
            return 2
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, os.path.abspath(__file__)] + sys.argv[1:]
    procs = [subprocess.Popen(cmd, env=rank_env(r, n, port)) for r in range(n)]
    rcs = [p.wait() for p in procs]
    return next((rc for rc in rcs if rc != 0), 0)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms; the summary keeps
    the samples that arrived while the timed region ran (all of them if none did)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def mark(self):
        """The timed region starts now."""
        self.t_start = time.perf_counter()

    def start(self):
        self.t_start = time.perf_counter()
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        t_end = time.perf_counter()
        time.sleep(0.1)  # the sample taken as the region ended
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        inside = [r for t, r in self.rows if self.t_start <= t <= t_end + 0.06]
        rows = inside if inside else [r for _, r in self.rows]
        self.rows = rows
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in self.rows for j in range(4) if r[5 + j].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def measured_traffic_per_cell(workload: str, mode: str):
    """DRAM bytes per band cell, and the instruction count, of one launch of the
    batched kernel on this workload, from the committed ncu summary (None when
    the summary has no capture of this workload and form)."""
    p = os.path.join(ROOT, "profiles", "core_dram_bytes.json")
    try:
        with open(p) as f:
            d = json.load(f)["workloads"][workload]
        if mode != "batched":
            return None, None
        return float(d["dram_bytes_per_band_cell"]), d
    except (OSError, KeyError, ValueError):
        return None, None


# ---------------------------------------------------------------- CPU side
def cpu_align(batch, threads: int):
    from oracle import oracle
    t0 = time.perf_counter()
    oracle.align_batch(batch, threads=threads)
    return time.perf_counter() - t0


def reference_arm(args, dist):
    """The reference's CPU align() path on the host cores (the oracle port of
    align_swi.cl + align_swi.cpp; the reference's own code when it compiled here)."""
    if dist.rank != 0:
        print(f"bench.py: rank {dist.rank}/{dist.world} exits without work (the reference arm runs on rank 0)",
              file=sys.stderr, flush=True)
        return 0
    pkg = load_package()
    from abea_gb300 import synth
    from oracle import oracle
    oracle.build()
    batch = synth.make_batch(args.workload, seed=args.seed)
    threads = os.cpu_count() or 1
    kind = "port"
    for _ in range(args.warmup if args.warmup < 2 else 1):
        cpu_align(batch, threads)
    times = [cpu_align(batch, threads) for _ in range(args.steps)]
    t = sum(times) / len(times)
    cells = batch.band_cells()
    v = cells / t
    line = {
        "impl": "reference", "metric": "ABEA band-cells/s (f5c align, adaptive band 100)",
        "value": v, "unit": "band-cells/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 scores, f64 transition adds", "data": "synthetic",
        "config": {"workload": args.workload, "description": WORKLOADS.get(args.workload),
                   "reads": batch.n_reads, "band_cells": cells, "seed": args.seed},
        "reads_per_s": batch.n_reads / t, "n_ranks": dist.world,
        "cpu_baseline": {"value": v, "unit": "band-cells/s", "cores": threads, "kind": kind,
                         "sample": f"the whole {args.workload} batch per step"},
        "e2e": {"value": v, "unit": "band-cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU side
def time_device(pkg, ctx, dev, steps: int, warmup: int):
    for _ in range(warmup):
        dev.run()
        dev.sync()
    per_step, core = [], []
    for _ in range(steps):
        ctx.flush_l2()
        ctx.mark(0)
        dev.run()
        ctx.mark(1)
        per_step.append(ctx.elapsed(0, 1))
        core.append(dev.timing()["core_ms"])
    return per_step, core, dev.timing()


def time_e2e(pkg, ctx, batch, steps: int, warmup: int):
    import ctypes as C
    L = pkg.lib()
    # pinned host copies of the inputs and outputs
    arrs = pkg._batch_arrays(batch)
    pinned = []
    for a in arrs:
        p = L.abea_host_alloc(max(a.nbytes, 1))
        if not p:
            raise MemoryError("pinned allocation failed")
        C.memmove(p, a.ctypes.data, a.nbytes)
        pinned.append(p)
    cap = max(batch.pair_capacity(), 1)
    out_p = L.abea_host_alloc(cap * 8)
    out_n = L.abea_host_alloc(max(batch.n_reads, 1) * 4)
    try:
        def call():
            st = L.abea_align_batch(ctx.h, batch.n_reads, *pinned, out_p, out_n)
            if st:
                raise pkg.AbeaError(st, L.abea_last_error().decode())
        for _ in range(warmup):
            call()
        ts = []
        for _ in range(steps):
            ctx.flush_l2()
            ctx.mark(0)
            ctx.elapsed(0, 0)
            t0 = time.perf_counter()
            call()
            ts.append(time.perf_counter() - t0)
        timing, h2d, d2h = ctx.last_timing()
        return ts, timing, h2d, d2h
    finally:
        for p in pinned + [out_p, out_n]:
            L.abea_host_free(p)


def run_mode(pkg, batch, mode, device, steps, warmup, autotune=False):
    ctx = pkg.Context(device, mode)
    dev = ctx.upload(batch)
    if autotune and mode == pkg.MODE_BATCHED:
        dev.autotune()
    per_step, core, timing = time_device(pkg, ctx, dev, steps, warmup)
    res = dict(per_step=per_step, core=core, timing=timing, slow=dev.slow_cells())
    dev.close()
    ctx.close()
    return res


def adjoint_report(pkg, synth, device, seed):
    """The adjoint workload: 4,096 reads U(1 kb, 10 kb) whose scalings are off
    by U(-8, 8) pA and a factor U(0.9, 1.1): forward + backward throughput, and the
    scalings recovered by three annealed Gauss-Newton rounds."""
    b = synth.make_batch("adjoint", seed=seed, perturb=True)
    true = b.meta["true_scalings"]
    ctx = pkg.Context(device, pkg.MODE_BATCHED)
    ctx.set_option(pkg.OPT_VAR_AWARE, 1)
    # reads over 8 kb keep band-score checkpoints every 256 bands, not their trace
    nb8k = 8000 + int(round(8000 * 1.71)) + 2
    budget = ((nb8k + 3) // 4) * 4 * 128
    ctx.set_option(pkg.OPT_TRACE_BUDGET, budget)
    nb = b.n_bands()
    trace_bytes = ((nb + 3) // 4) * 4 * 128
    ck = trace_bytes > budget
    dev = ctx.upload(b)
    dev.run()
    dev.sync()
    fwd, bwd = [], []
    for _ in range(3):
        ctx.flush_l2()
        ctx.mark(0)
        dev.run()
        ctx.mark(1)
        fwd.append(ctx.elapsed(0, 1))
        t0 = time.perf_counter()
        g = dev.backward()
        bwd.append((time.perf_counter() - t0) * 1e3)
    n_grad = int(np.count_nonzero(g["status"] == 0))

    def err(sc):
        ds = np.abs(sc["shift"].astype(np.float64) - true["shift"])
        dk = np.abs(sc["scale"].astype(np.float64) / true["scale"] - 1.0)
        return {"shift_pA_median": float(np.median(ds)), "shift_pA_p90": float(np.percentile(ds, 90)),
                "scale_rel_median": float(np.median(dk)), "scale_rel_p90": float(np.percentile(dk, 90)),
                "within_1pA_1pct": float(np.mean((ds < 1.0) & (dk < 0.01)))}

    before = err(b.scalings)
    t0 = time.perf_counter()
    sc = dev.recalibrate(3, first_temperature=5.0)
    t_gn = time.perf_counter() - t0
    cells = b.band_cells()
    dev.close()
    ctx.close()
    return {
        "workload": "4096 reads U(1 kb, 10 kb); scalings perturbed by shift U(-8, 8) pA, scale x U(0.9, 1.1); "
                    "reads over 8 kb checkpointed",
        "emission": "var-aware (stdv*var, log stdv + log var)",
        "checkpointing": {"trace_budget_bytes": int(budget), "reads_checkpointed": int(ck.sum()),
                          "every_bands": 256,
                          "trace_bytes_kept": int(trace_bytes[~ck].sum()),
                          "trace_bytes_replaced": int(trace_bytes[ck].sum()),
                          "checkpoint_bytes": int(((nb[ck] // 256 + 1) * 264 * 4).sum())},
        "forward_ms": statistics.mean(fwd), "forward_band_cells_per_s": cells / (statistics.mean(fwd) / 1e3),
        "backward_ms_incl_d2h": statistics.mean(bwd), "reads_with_gradient": n_grad, "reads": b.n_reads,
        "gauss_newton": {"iterations": 3, "first_temperature": 5.0, "wall_s": t_gn,
                         "error_before": before, "error_after": err(sc)},
        "checked_in_tests": "FP64 oracle gradient and central differences h=1e-3 (tests/test_adjoint.py)",
    }


def next_rows_report(pkg, synth, device, seed, cpu: bool):
    """The rows after the path, on the f5c batch after one batched run: f5c's
    postalign (abea_batch_postalign) and the method-of-moments scalings
    (abea_batch_estimate_scalings).  Device time by CUDA events on the library's
    stream around the entry (memsets, kernel, the per-read counts or scalings
    back to the host); end to end = wall time with every output copied to
    (pageable) host arrays; the oracle's single-thread loops beside them."""
    b = synth.make_batch("f5c_batch", seed=seed)
    ctx = pkg.Context(device, pkg.MODE_BATCHED)
    dev = ctx.upload(b)
    dev.run()
    pairs, counts = dev.results()
    n_pairs = int(np.maximum(counts, 0).sum())
    dev.postalign(outputs=False)
    dt = []
    for _ in range(5):
        ctx.flush_l2()
        ctx.mark(0)
        got = dev.postalign(outputs=False)
        ctx.mark(1)
        dt.append(ctx.elapsed(0, 1))
    t0 = time.perf_counter()
    dev.postalign()
    e2e = (time.perf_counter() - t0) * 1e3
    n_rec = int(got["n_alignment"].sum())
    n_kmers = int(np.maximum(b.read_len - 5, 0).sum())
    # algorithmic bytes: every pair read once, every record and map entry written once
    algo = 8 * n_pairs + 32 * n_rec + 8 * n_kmers
    ms = min(dt)
    peak, peak_kind = measured_peak_hbm()
    pa = {"reads": b.n_reads, "pairs": n_pairs, "records": n_rec, "device_ms": ms, "device_ms_mean": statistics.mean(dt),
          "e2e_ms_with_host_outputs": e2e, "algorithmic_bytes": algo,
          "achieved_gbs": algo / (ms / 1e3) / 1e9, "peak_gbs": peak, "peak_kind": f"{peak_kind} (hbm_gbs)",
          "note": "device_ms includes the two output memsets and the count copy; a step this small is launch-bound"}
    dev.estimate_scalings()
    mt = []
    for _ in range(5):
        ctx.mark(0)
        dev.estimate_scalings()
        ctx.mark(1)
        mt.append(ctx.elapsed(0, 1))
    mom = {"reads": b.n_reads, "device_ms": min(mt), "device_ms_mean": statistics.mean(mt)}
    if cpu:
        from oracle import oracle
        t0 = time.perf_counter()
        oracle.postalign_batch(b, pairs, counts)
        pa["cpu_oracle_ms"] = (time.perf_counter() - t0) * 1e3
        pa["cpu_oracle_cores"] = 1
        t0 = time.perf_counter()
        for i in range(b.n_reads):
            p, e = int(b.read_ptr[i]), int(b.event_ptr[i])
            oracle.mom(b.read[p:p + int(b.read_len[i])].tobytes(), b.events[e:e + int(b.n_events[i])], b.model)
        mom["cpu_oracle_ms"] = (time.perf_counter() - t0) * 1e3
        mom["cpu_oracle_cores"] = 1
    dev.close()
    ctx.close()
    return {"postalign": pa, "method_of_moments": mom, "workload": "f5c_batch seed %d after one batched run" % seed}


def serving_report(pkg, synth, device, seed, mbases: float):
    """The serving stream: `mbases` Mbases of reads (lognormal, median 8 kb, at
    most 200 kb) admitted in order into device batches by footprint, two in
    flight; per batch align, adjoint, one Gauss-Newton step, re-align.  Batched
    and plain forms side by side, inputs and outputs in pinned host memory; the
    timed call is the second of two identical calls (the first sizes the device
    batches and captures nothing else)."""
    t0 = time.perf_counter()
    b = synth.make_stream(seed=seed, total_bases=int(mbases * 1e6))
    gen_s = time.perf_counter() - t0
    pb = pkg.pin_batch(b)
    cap = max(b.pair_capacity(), 1)
    res, pairs_out = {}, {}
    for name, mode in (("batched", pkg.MODE_BATCHED), ("plain", pkg.MODE_PLAIN)):
        ctx = pkg.Context(device, mode)
        pairs = pkg.pinned_empty(cap, pkg.types.PAIR_DTYPE)
        counts = pkg.pinned_empty(max(b.n_reads, 1), np.int32)
        ctx.align_stream(pb, recalibrate=True, out_pairs=pairs, out_counts=counts)
        r = ctx.align_stream(pb, recalibrate=True, out_pairs=pairs, out_counts=counts)
        ctx.close()
        st = r["stats"]
        lat = r["latency_ms"]
        res[name] = {"wall_s": st["wall_ms"] / 1e3, "reads_per_s": b.n_reads / (st["wall_ms"] / 1e3),
                     "band_cells_per_s": st["band_cells"] / (st["wall_ms"] / 1e3),
                     "device_busy_s": st["compute_ms"] / 1e3, "batches": st["n_batches"],
                     "max_batch_reads": st["max_batch_reads"], "max_batch_bytes": st["max_batch_bytes"],
                     "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
                     "latency_ms_max": float(lat.max())}
        pairs_out[name] = (pairs, r["counts"].copy(), r["scalings"].copy())
    a, p = pairs_out["batched"], pairs_out["plain"]
    same = bool(np.array_equal(a[1], p[1]) and np.array_equal(a[2].view(np.uint32), p[2].view(np.uint32)))
    if same:
        for x, y in zip(pkg.split_pairs(b, a[0], a[1]), pkg.split_pairs(b, p[0], p[1])):
            if not np.array_equal(x, y):
                same = False
                break
    true = b.meta["true_scalings"]
    ds = np.abs(a[2]["shift"].astype(np.float64) - true["shift"])
    dk = np.abs(a[2]["scale"].astype(np.float64) / true["scale"] - 1.0)
    return {
        "workload": f"{b.read_len.sum() / 1e6:.1f} Mbases, {b.n_reads} reads, lognormal median 8 kb (sigma 0.6), "
                    f"clipped to [500, 200000], longest {int(b.read_len.max())}; per device batch: align, adjoint, "
                    "one Gauss-Newton step, re-align",
        "band_cells": b.band_cells(), "events": int(b.n_events.sum()), "generate_s": gen_s,
        "batch_bytes": "default: min(16 GiB, 40% of free device memory)",
        "latency": "per read, from its batch's admission (host queues the copy) to its results in host memory",
        "batched": res["batched"], "plain": res["plain"],
        "batched_over_plain": res["batched"]["band_cells_per_s"] / res["plain"]["band_cells_per_s"],
        "identical_pairs_and_scalings": same,
        "scalings_after_step": {"shift_pA_median_err": float(np.median(ds)), "scale_rel_median_err": float(np.median(dk))},
    }


def longest_read_ms(pkg, batch, device):
    """The batch's longest read alone on the wide shape (batched form, one read):
    the step can be no shorter than this (a read's bands run in sequence)."""
    i = int(np.argmax(batch.n_bands()))
    one = batch.subset(np.array([i]))
    ctx = pkg.Context(device, pkg.MODE_BATCHED)
    ctx.set_option(pkg.OPT_LONG_READ_BANDS, 1)
    dev = ctx.upload(one)
    dev.run()
    dev.sync()
    ts = []
    for _ in range(3):
        ctx.flush_l2()
        ctx.mark(0)
        dev.run()
        ctx.mark(1)
        ts.append(ctx.elapsed(0, 1))
    dev.close()
    ctx.close()
    return min(ts), int(one.n_bands()[0])


def autotune_report(pkg, synth, batch, args, device):
    """The autotuner beside the heuristic headline: a threshold tuned on another
    batch of the same shape (seed + 100) and set on this one's context, and one
    tuned on this very batch."""
    other = synth.make_batch(args.workload, seed=args.seed + 100)
    ctx = pkg.Context(device, pkg.MODE_BATCHED)
    d2 = ctx.upload(other)
    thr_other, _ = d2.autotune()
    d2.close()
    dev = ctx.upload(batch)
    ctx.set_option(pkg.OPT_LONG_READ_BANDS, int(thr_other))
    ms_other = statistics.mean(time_device(pkg, ctx, dev, 5, 1)[0])
    ctx.set_option(pkg.OPT_LONG_READ_BANDS, 0)
    thr_self, _ = dev.autotune()
    ms_self = statistics.mean(time_device(pkg, ctx, dev, 5, 1)[0])
    nb = batch.n_bands()
    dev.close()
    ctx.close()
    return {"tuned_on_other_seed": {"seed": args.seed + 100, "threshold_bands": int(thr_other),
                                    "wide_reads": int((nb >= thr_other).sum()), "ms_per_step": ms_other},
            "tuned_on_this_batch": {"threshold_bands": int(thr_self), "wide_reads": int((nb >= thr_self).sum()),
                                    "ms_per_step": ms_self}}


def align_threads_report(pkg, batch, threads: int = 8, max_reads: int = 256):
    """f5c's calling pattern: align() once per read from `threads` host threads at
    once (each thread its own context and stream inside the library), on the
    batch's reads; reads/s, and the results against one batched run."""
    import concurrent.futures as cf
    n = min(batch.n_reads, max_reads)
    idx = list(range(n))
    seqs = [batch.sequence(i) for i in idx]
    evs = [np.ascontiguousarray(batch.read_events(i)) for i in idx]

    def one(i):
        return pkg.align(seqs[i], evs[i], batch.model, batch.scalings[i])
    with cf.ThreadPoolExecutor(threads) as ex:  # warm-up: each thread's context
        list(ex.map(one, idx[:threads]))
        t0 = time.perf_counter()
        got = list(ex.map(one, idx))
        dt = time.perf_counter() - t0
    ctx = pkg.Context(0, pkg.MODE_BATCHED)
    sub = batch.subset(np.array(idx))
    pairs, counts = ctx.align_batch(sub)
    ctx.close()
    ref = pkg.split_pairs(sub, pairs, counts)
    same = all(np.array_equal(got[i], ref[i]) for i in range(n))
    cells = sub.band_cells()
    return {"host_threads": threads, "reads": n, "wall_s": dt, "reads_per_s": n / dt,
            "band_cells_per_s": cells / dt, "identical_to_batched": bool(same),
            "per_thread_device_footprint": "one context per calling thread (a stream, 24 CUDA events) and a "
                                           "device slab grown to that thread's largest read so far: about 132 B "
                                           "per band + 48 B per event + 17 B per base, plus 136 KB fixed, plus "
                                           "512 KB of traceback scratch for a read of 512 bands or more "
                                           "(a 20 kb read: ~9.5 MB)"}


def ours(args, dist):
    pkg = load_package()
    from abea_gb300 import synth
    device = dist.local_rank
    # weak scaling: every rank aligns its own batch of the workload's shape
    batch = synth.make_batch(args.workload, seed=args.seed + dist.rank)
    cells = batch.band_cells()
    mode = pkg.MODE_BATCHED if args.mode == "batched" else pkg.MODE_PLAIN

    clocks = ClockSampler(device)
    clocks.start()  # nvidia-smi starts sampling during the setup; the summary keeps the timed region
    ctx = pkg.Context(device, mode)
    dev = ctx.upload(batch)
    launches_per_step = None
    for _ in range(args.warmup):
        dev.run()
        dev.sync()
    dist.barrier()
    clocks.mark()
    t_wall0 = time.perf_counter()
    per_step, core = [], []
    for _ in range(args.steps):
        ctx.flush_l2()
        ctx.mark(0)
        dev.run()
        ctx.mark(1)
        per_step.append(ctx.elapsed(0, 1))
        tm = dev.timing()
        core.append(tm["core_ms"])
        launches_per_step = tm["kernel_launches"]
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    slow = dev.slow_cells()
    best = dev.best_scores()
    gpairs, gcounts = dev.results()
    dev.close()
    local_ms = sum(per_step)
    dist.barrier()
    max_ms = dist.max(local_ms)
    total_cells = dist.sum(float(cells))
    total_reads = dist.sum(float(batch.n_reads))
    ms_per_step = max_ms / args.steps
    value = total_cells / (ms_per_step / 1e3)

    # end to end through abea_align_batch (pinned host buffers)
    e2e_ts, e2e_timing, h2d, d2h = time_e2e(pkg, ctx, batch, args.steps, 1)
    e2e_s = dist.max(sum(e2e_ts)) / args.steps
    ctx.close()

    if dist.rank != 0:
        return 0
    nb = batch.n_bands()
    n_wide = None
    if mode == pkg.MODE_BATCHED:
        import torch
        n_wide = pkg.heuristic_wide_reads(nb, torch.cuda.get_device_properties(device).multi_processor_count)
    out = {
        "metric": "ABEA band-cells/s (f5c align, adaptive band 100)",
        "value": value, "unit": "band-cells/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 scores, f64 transition adds (emulated exactly)",
        "data": "synthetic",
        "config": {"workload": args.workload, "description": WORKLOADS.get(args.workload),
                   "reads": int(total_reads), "band_cells": int(total_cells), "seed": args.seed,
                   "l2": "flushed (write of 2x L2) before every timed step"},
        "mode": args.mode,
        "parallelism": f"{dist.world} rank(s), one GPU each; rank r aligns its own batch (seed {args.seed} + r)",
        "wide_reads": n_wide, "wide_threshold": "the library's heuristic (no autotuning)",
        "reads_per_s": total_reads / (ms_per_step / 1e3),
        "gpu_launches": int(launches_per_step or 0) * args.steps,
        "wall_s_timed_region": wall,
        "slow_cells_fp64": slow,
        "clocks": clk,
        "e2e": {"value": total_cells / e2e_s, "unit": "band-cells/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                "stage_ms": {k: round(v, 4) for k, v in e2e_timing.items() if k.endswith("_ms")}},
    }
    # roofline of the dominant kernel (the fused fill + traceback), algorithmic bytes = 5 B per band cell
    peak, peak_kind = measured_peak_hbm()
    core_ms = statistics.mean(core)
    achieved = BYTES_PER_CELL * cells / (core_ms / 1e3) / 1e9
    tpc, tinfo = measured_traffic_per_cell(args.workload, args.mode)
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                       "frac": achieved / peak, "peak_kind": f"{peak_kind} (hbm_gbs)",
                       "traffic": (tpc * cells) if tpc else None,
                       "kernel": "abea_batched_kernel (fill + traceback)", "core_ms": core_ms,
                       "algorithmic_bytes": BYTES_PER_CELL * cells}
    if tinfo:
        out["roofline"]["traffic_source"] = tinfo.get("source")
    if dist.world == 1:
        # the two bounds that do apply: the longest read's band chain, and instruction issue
        lr_ms, lr_bands = longest_read_ms(pkg, batch, device)
        mhz = clk.get("sm_mhz") or 2070.0
        out["roofline"]["latency_bound"] = {
            "longest_read_bands": lr_bands, "longest_read_alone_ms": lr_ms,
            "frac": lr_ms / core_ms, "cycles_per_band": lr_ms * 1e-3 * mhz * 1e6 / lr_bands,
            "note": "the longest read's bands run in sequence: the step can be no shorter than that read alone"}
        if tinfo and tinfo.get("inst_executed_per_launch") and tinfo.get("sm_count"):
            slots = tinfo["sm_count"] * 4 * mhz * 1e6 * core_ms * 1e-3
            out["roofline"]["issue_bound"] = {
                "warp_instructions_per_launch": tinfo["inst_executed_per_launch"],
                "issue_slots": slots, "frac": tinfo["inst_executed_per_launch"] / slots,
                "source": tinfo.get("source"),
                "note": "warp-instructions of one launch (ncu) over the SMs' issue slots in the live step time"}
    if args.compare and dist.world == 1:
        out["autotune"] = autotune_report(pkg, synth, batch, args, device)
        other = "plain" if args.mode == "batched" else "batched"
        om = pkg.MODE_PLAIN if other == "plain" else pkg.MODE_BATCHED
        r = run_mode(pkg, batch, om, device, max(2, args.steps // 2), 1)
        ms = statistics.mean(r["per_step"])
        out[other] = {"value": cells / (ms / 1e3), "ms_per_step": ms, "core_ms": statistics.mean(r["core"])}
        # the uneven (heavy-tail) 1.3 Mbase batch, both forms
        ub = synth.make_batch("uneven", seed=args.seed)
        un = {}
        for name, m in (("batched", pkg.MODE_BATCHED), ("plain", pkg.MODE_PLAIN)):
            r = run_mode(pkg, ub, m, device, 2, 1)
            ms = statistics.mean(r["per_step"])
            un[name] = {"value": ub.band_cells() / (ms / 1e3), "ms_per_step": ms}
        un["batched_over_plain"] = un["batched"]["value"] / un["plain"]["value"]
        un["workload"] = WORKLOADS["uneven"]
        out["uneven"] = un
        # the three batch shapes side by side: batched, plain and the CPU oracle on all host cores
        per = {}
        for wl in ("small", "f5c_batch", "uneven"):
            wb = batch if wl == args.workload else (ub if wl == "uneven" else synth.make_batch(wl, seed=args.seed))
            wc, wr = wb.band_cells(), wb.n_reads
            row = {"reads": wr, "band_cells": wc}
            for name, m in (("batched", pkg.MODE_BATCHED), ("plain", pkg.MODE_PLAIN)):
                if wl == args.workload and name == args.mode:
                    ms = ms_per_step
                elif wl == args.workload:
                    ms = out[name]["ms_per_step"]
                elif wl == "uneven":
                    ms = un[name]["ms_per_step"]
                else:
                    ms = statistics.mean(run_mode(pkg, wb, m, device, 3, 1)["per_step"])
                row[name] = {"band_cells_per_s": wc / (ms / 1e3), "reads_per_s": wr / (ms / 1e3), "ms": ms}
            if args.cpu:
                threads = os.cpu_count() or 1
                t = cpu_align(wb, threads)
                row["cpu"] = {"band_cells_per_s": wc / t, "reads_per_s": wr / t, "ms": t * 1e3, "cores": threads}
            per[wl] = row
        out["per_config"] = per
        out["align_threads"] = align_threads_report(pkg, batch)
    if args.compare and dist.world == 1:
        out["adjoint"] = adjoint_report(pkg, synth, device, args.seed)
        out["next_rows"] = next_rows_report(pkg, synth, device, args.seed, args.cpu)
    if args.compare and dist.world == 1 and args.serving_mbases > 0:
        out["serving"] = serving_report(pkg, synth, device, args.seed, args.serving_mbases)
    if args.cpu and dist.world == 1:
        threads = os.cpu_count() or 1
        t = cpu_align(batch, threads)
        out["cpu_baseline"] = {"value": cells / t, "unit": "band-cells/s", "cores": threads, "kind": "port",
                               "sample": f"the whole {args.workload} batch, once"}
        out["fp64_error"] = fp64_report(pkg, synth, args, batch, best, gpairs, gcounts, device)
    print(json.dumps(out), flush=True)
    return 0


def fp64_report(pkg, synth, args, batch, best, pairs, counts, device):
    """The checker beside the measurement: each result's distance to the all-FP64
    recurrence (the oracle's FP64 twin on the host cores), for the GPU's own
    best scores and AlignedPairs of the timed batch and of the small and uneven
    batches.  The GPU's FP32 results equal the reference's FP32 arithmetic bit
    for bit (tests/test_gpu_parity.py)."""
    from oracle import oracle
    res = {args.workload: oracle.fp64_error(batch, best, pairs, counts)}
    for wl in ("small", "f5c_batch", "uneven"):
        if wl in res:
            continue
        b = synth.make_batch(wl, seed=args.seed)
        ctx = pkg.Context(device, pkg.MODE_BATCHED)
        dev = ctx.upload(b)
        dev.run()
        p, c = dev.results()
        bs = dev.best_scores()
        dev.close()
        ctx.close()
        res[wl] = oracle.fp64_error(b, bs, p, c)
    res["note"] = ("relative error of the FP32 best-end scores against the FP64 recurrence (reads with a finite "
                   "end), and the reads whose AlignedPairs differ under FP64; the error grows with read length")
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="f5c_batch")
    ap.add_argument("--mode", choices=["batched", "plain"], default="batched")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-compare", dest="compare", action="store_false")
    ap.add_argument("--no-cpu", dest="cpu", action="store_false")
    ap.add_argument("--serving-mbases", type=float, default=200.0,
                    help="size of the serving-stream report (0 = skip it)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return launch_ranks(args)
    dist = Dist(use_cuda=args.impl == "ours", init=args.impl == "ours")
    try:
        rc = reference_arm(args, dist) if args.impl == "reference" else ours(args, dist)
    finally:
        dist.close()
    return rc


if __name__ == "__main__":
    sys.exit(main())
