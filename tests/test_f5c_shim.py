"""The align_cuda(core, db) shim of tests/f5c_shim/align_cuda_shim.c: compiled as
C against include/abea.h and the library, then run on a batch that includes a
200 kb read (f5c would route a read that long to the CPU, GPU/f5c.h:98,105;
here it takes the same call).  Its results must equal abea_align_batch's."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, abea

SHIM = os.path.join(ROOT, "tests", "f5c_shim", "align_cuda_shim.c")


def build_shim(out_dir):
    if not os.path.exists(abea.LIB_PATH):
        abea.build()
    lib_dir = os.path.dirname(abea.LIB_PATH)
    so = os.path.join(str(out_dir), "libshim.so")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-O2", "-fPIC", "-shared", "-I",
                    os.path.join(ROOT, "include"), SHIM, "-L", lib_dir, "-labea", f"-Wl,-rpath,{lib_dir}", "-o", so],
                   check=True)
    return so


def test_shim_compiles_against_the_header(tmp_path):
    assert os.path.exists(build_shim(tmp_path))


@pytest.mark.gpu
def test_shim_with_a_200kb_read_matches_the_batch_entry(tmp_path):
    from abea_gb300 import synth
    from abea_gb300.types import EVENT_DTYPE, MODEL_DTYPE, PAIR_DTYPE, SCALINGS_DTYPE
    abea.lib()  # loads libabea.so first, so the shim binds to the same library
    shim = C.CDLL(build_shim(tmp_path))
    lens = [200000] + list(np.random.default_rng(8).integers(500, 8000, 12))
    batch = synth.make_batch("small", seed=41, lengths=lens)
    n = batch.n_reads
    reads = [np.frombuffer(batch.sequence(i) + b"\0", dtype=np.uint8).copy() for i in range(n)]
    evs = [np.ascontiguousarray(batch.read_events(i), dtype=EVENT_DTYPE) for i in range(n)]
    outs = [np.zeros(max(2 * len(e), 1), dtype=PAIR_DTYPE) for e in evs]
    read_p = (C.c_void_p * n)(*[r.ctypes.data for r in reads])
    out_p = (C.c_void_p * n)(*[o.ctypes.data for o in outs])

    class ET(C.Structure):
        _fields_ = [("n", C.c_size_t), ("start", C.c_size_t), ("end", C.c_size_t), ("event", C.c_void_p)]
    et = (ET * n)()
    for i, e in enumerate(evs):
        et[i].n, et[i].start, et[i].end, et[i].event = len(e), 0, len(e), e.ctypes.data
    lens32 = np.ascontiguousarray(batch.read_len, dtype=np.int32)
    sc = np.ascontiguousarray(batch.scalings, dtype=SCALINGS_DTYPE)
    model = np.ascontiguousarray(batch.model, dtype=MODEL_DTYPE)
    counts = np.full(n, -99, dtype=np.int32)
    shim.shim_align_batch.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 7
    shim.shim_align_batch(0, n, read_p, lens32.ctypes.data, C.cast(et, C.c_void_p), sc.ctypes.data,
                          model.ctypes.data, out_p, counts.ctypes.data)
    ctx = abea.Context(0, abea.MODE_BATCHED)
    pairs, ref_counts = ctx.align_batch(batch)
    ctx.close()
    ref = abea.split_pairs(batch, pairs, ref_counts)
    assert np.array_equal(counts, np.maximum(ref_counts, 0))
    for i in range(n):
        assert np.array_equal(outs[i][:counts[i]], ref[i]), i
    assert int(batch.n_bands()[0]) > 500000  # the 200 kb read: over half a million bands
