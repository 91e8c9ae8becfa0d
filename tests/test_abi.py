"""The C-ABI library: it builds, loads and exports every declared entry point
(no device calls: this file runs without a GPU)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT, abea

HEADER = os.path.join(ROOT, "include", "abea.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(abea_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    if not os.path.exists(abea.LIB_PATH):
        abea.build()
    return abea.LIB_PATH


def test_header_declares_the_f5c_entry():
    names = declared_functions()
    for n in ("abea_align", "abea_align_batch", "abea_batch_create", "abea_batch_run",
              "abea_ctx_create", "abea_ctx_destroy", "abea_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True,
                         check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert missing == []
    # f5c's own symbol, as a weak alias of abea_align
    assert "align" in exported


def test_library_loads_with_ctypes(libpath):
    L = C.CDLL(libpath)
    for n in declared_functions():
        assert hasattr(L, n)
    assert set(abea.EXPORTS) <= set(declared_functions())


def test_no_torch_or_oracle_in_library(libpath):
    out = subprocess.run(["nm", "-D", "--undefined-only", libpath], capture_output=True, text=True,
                         check=True).stdout
    assert "oracle_" not in out and "torch" not in out


def test_status_strings_without_device(libpath):
    L = abea.lib()
    assert L.abea_status_string(-2).decode().startswith("alignment longer")
    assert L.abea_version().decode().startswith("abea-gb300")


def test_argument_checks_without_device(libpath):
    """Entries that are handed null handles fail with ABEA_ERR_INVALID_ARG before
    touching a device (no GPU is needed to reach these checks)."""
    import ctypes as C
    L = abea.lib()
    vp = C.c_void_p
    L.abea_batch_postalign.argtypes = [vp] * 6
    assert L.abea_batch_postalign(None, None, None, None, None, None) == -1
    L.abea_batch_estimate_scalings.argtypes = [vp, vp, vp, C.c_int32]
    assert L.abea_batch_estimate_scalings(None, None, None, 0) == -1
    L.abea_align_db.argtypes = [vp, C.c_int32] + [vp] * 7
    assert L.abea_align_db(None, 1, None, None, None, None, None, None, None) == -1
    f = L.abea_internal_stage_db
    f.argtypes = [C.c_int32] + [vp] * 5 + [C.c_int32]
    f.restype = C.c_int32
    assert f(-1, None, None, None, None, None, 0) == -1
    assert f(0, None, None, None, None, None, 0) == 0


def test_staging_refuses_null_per_read_arrays(libpath):
    """abea_internal_stage_db checks each read as abea_align_db does: a read with
    bases but no sequence pointer, or events but no event pointer, is refused
    (-1) before any copy."""
    import ctypes as C
    import numpy as np
    L = abea.lib()
    vp = C.c_void_p
    f = L.abea_internal_stage_db
    f.argtypes = [C.c_int32] + [vp] * 5 + [C.c_int32]
    f.restype = C.c_int32

    class ET(C.Structure):
        _fields_ = [("n", C.c_size_t), ("start", C.c_size_t), ("end", C.c_size_t), ("event", C.c_void_p)]
    seq = np.zeros(64, dtype=np.uint8)
    ev = np.zeros(64 * 24, dtype=np.uint8)
    good = np.frombuffer(b"ACGTACGTAC\0", dtype=np.uint8).copy()
    evs = np.zeros(3 * 24, dtype=np.uint8)
    lens = np.array([10], dtype=np.int32)
    et = (ET * 1)()
    et[0].n, et[0].start, et[0].end, et[0].event = 3, 0, 3, evs.ctypes.data
    reads = (C.c_void_p * 1)(good.ctypes.data)
    assert f(1, reads, lens.ctypes.data, C.cast(et, vp), seq.ctypes.data, ev.ctypes.data, 1) == 0
    no_read = (C.c_void_p * 1)(None)
    assert f(1, no_read, lens.ctypes.data, C.cast(et, vp), seq.ctypes.data, ev.ctypes.data, 1) == -1
    et[0].event = None
    assert f(1, reads, lens.ctypes.data, C.cast(et, vp), seq.ctypes.data, ev.ctypes.data, 1) == -1
