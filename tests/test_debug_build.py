"""The bounds-checked build (libabea_debug.so, ABEA_BOUNDS_CHECK): every global
store of the fill and of the traceback checks its index against its region and
counts a violation instead of writing (the run then fails with
ABEA_ERR_INTERNAL).  Run in a child process so that the two libraries never
share one."""
import os
import subprocess
import sys

import pytest

from conftest import GOLDEN, ROOT, abea

SCRIPT = r'''
import os, sys
import numpy as np
sys.path.insert(0, {tests!r})
from conftest import abea, batch_from_npz, split_fixture_pairs
abea.LIB_PATH = os.path.join(os.path.dirname(abea.LIB_PATH), "libabea_debug.so")
abea._lib = None
from abea_gb300 import synth

d = np.load(os.path.join({golden!r}, "ref_synthetic.npz"))
edge = batch_from_npz(d)
ref_pairs = split_fixture_pairs(d["ref_pairs"], d["ref_counts"])

def run(batch, mode, threshold=0, budget=0):
    ctx = abea.Context(0, mode)
    if threshold:
        ctx.set_option(abea.OPT_LONG_READ_BANDS, threshold)
    if budget:
        ctx.set_option(abea.OPT_TRACE_BUDGET, budget)
    return ctx.align_batch(batch)   # raises on a bounds violation

def same(batch, a, b):
    assert np.array_equal(a[1], b[1])
    for x, y in zip(abea.split_pairs(batch, *a), abea.split_pairs(batch, *b)):
        assert np.array_equal(x, y)

# the reference fixture's edge cases: plain, batched with every read wide, checkpointed
for kw in ({{}}, {{"threshold": 1}}, {{"threshold": 512}}, {{"budget": 1}}):
    for mode in (abea.MODE_PLAIN, abea.MODE_BATCHED):
        p, c = run(edge, mode, **kw)
        assert np.array_equal(c, d["ref_counts"]), (mode, kw)
        for i, got in enumerate(abea.split_pairs(edge, p, c)):
            assert np.array_equal(got, ref_pairs[i]), (mode, kw, i)
# the 1.3 Mbase batch: both forms, and reads over 8 kb checkpointed
f5c = synth.make_batch("f5c_batch", seed=1)
plain = run(f5c, abea.MODE_PLAIN)
same(f5c, run(f5c, abea.MODE_BATCHED), plain)
same(f5c, run(f5c, abea.MODE_BATCHED, budget=(8000 + 13680 + 2) * 128), plain)
print("bounds-checked build: no violation")
'''


@pytest.mark.gpu
def test_bounds_checked_build_runs_clean():
    lib = os.path.join(os.path.dirname(abea.LIB_PATH), "libabea_debug.so")
    if not os.path.exists(lib):
        subprocess.run(["make", "-C", os.path.dirname(abea.LIB_PATH), "debug"], check=True,
                       stdout=subprocess.DEVNULL)
    script = SCRIPT.format(tests=os.path.join(ROOT, "tests"), golden=GOLDEN)
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "no violation" in r.stdout


def test_debug_target_in_the_makefile():
    text = open(os.path.join(os.path.dirname(abea.LIB_PATH), "Makefile")).read()
    assert "-DABEA_BOUNDS_CHECK" in text and "libabea_debug.so" in text
