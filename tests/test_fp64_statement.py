"""The error of the reference's FP32 arithmetic against the all-FP64 recurrence,
on the CPU (the oracle and its FP64 twin): the figures the benchmark reports
beside the GPU's results, which equal the FP32 oracle bit for bit."""
import os

import numpy as np
import pytest

from conftest import abea  # noqa: F401  (loads the package as abea_gb300)


@pytest.mark.parametrize("workload, bound", [("small", 1e-5), ("f5c_batch", 1e-5)])
def test_fp32_against_fp64_on_the_cpu(oracle_mod, workload, bound):
    from abea_gb300 import synth
    batch = synth.make_batch(workload, seed=1)
    p, c, best = oracle_mod.align_batch(batch, threads=os.cpu_count())
    e = oracle_mod.fp64_error(batch, best, p, c, threads=os.cpu_count())
    assert e["finite_ends"] == batch.n_reads
    assert 0 < e["best_score_rel_err_median"] <= e["best_score_rel_err_max"] < bound
    assert e["reads_with_other_pair_count"] == 0
    assert e["reads_passing_qc_fp32"] == e["reads_passing_qc_fp64"]
    assert e["reads_with_other_pairs"] <= batch.n_reads // 20


def test_fp64_twin_agrees_with_fp32_on_a_short_read(oracle_mod):
    """One read through both: the same best end and a best score within FP32 rounding."""
    from abea_gb300 import synth
    b = synth.make_batch("small", seed=3, lengths=[1500])
    seq, ev = b.sequence(0), b.read_events(0)
    _, _, info = oracle_mod.align(seq, ev, b.model, b.scalings[0])
    _, _, best64 = oracle_mod.align_f64(seq, ev, b.model, b.scalings[0])
    assert np.isfinite(best64)
    assert abs(info["best_score"] - best64) <= 1e-5 * abs(best64)
