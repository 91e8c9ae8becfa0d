"""abea_align_noalloc: the entry point for callers that cannot allocate device
memory (a framework whose own allocator owns the whole device, a service with a
device memory budget fixed at start-up).  Its buffers here come from the test
(torch tensors stand in for the caller's allocator); the call itself only uses
the library's fixed device array.  Checked against abea_align on two calls
in a row, bit-exact like every other parity test.  This file sorts last so a
run that stops at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from conftest import abea

pytestmark = pytest.mark.gpu


class _Scalings(C.Structure):
    _fields_ = [("scale", C.c_float), ("shift", C.c_float), ("var", C.c_float), ("log_var", C.c_float)]


def _bind():
    lib = abea.lib()
    lib.abea_align_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                       C.c_int32, C.c_void_p, _Scalings, C.c_void_p]
    lib.abea_align_noalloc.restype = C.c_int32
    return lib


def _noalloc(lib, torch, seq, events, model, scalings, stream):
    dev = torch.device("cuda:0")
    d_seq = torch.from_numpy(np.frombuffer(bytes(seq), dtype=np.uint8).copy()).to(dev)
    d_ev = torch.from_numpy(np.ascontiguousarray(events).view(np.uint8).copy()).to(dev)
    d_model = torch.from_numpy(np.ascontiguousarray(model).view(np.uint8).copy()).to(dev)
    cap = 2 * len(events)
    d_pairs = torch.zeros(max(cap, 1) * 2, dtype=torch.int32, device=dev)
    d_n = torch.full((1,), -99, dtype=torch.int32, device=dev)
    sc = _Scalings(float(scalings["scale"]), float(scalings["shift"]), float(scalings["var"]),
                   float(scalings["log_var"]))
    st = lib.abea_align_noalloc(C.c_void_p(d_pairs.data_ptr()), C.c_void_p(d_n.data_ptr()), cap,
                                C.c_void_p(d_seq.data_ptr()), len(seq), C.c_void_p(d_ev.data_ptr()), len(events),
                                C.c_void_p(d_model.data_ptr()), sc, C.c_void_p(stream))
    assert st == 0, lib.abea_last_error().decode()
    torch.cuda.synchronize()
    n = int(d_n.cpu()[0])
    pairs = d_pairs.cpu().numpy().view(abea.PAIR_DTYPE)[: max(n, 0)]
    return n, pairs


def test_noalloc_matches_align_on_two_calls(dump_subset):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _bind()
    batch, golden = dump_subset
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row on different reads, then the first read again
    for i in (0, 2, 0):
        seq, ev = batch.sequence(i), batch.read_events(i)
        n, pairs = _noalloc(lib, torch, seq, ev, batch.model, batch.scalings[i], stream)
        ref = abea.align(seq, ev, batch.model, batch.scalings[i])
        assert n == len(ref)
        assert np.array_equal(pairs, ref)
        assert np.array_equal(pairs, golden[i])


def test_noalloc_rejects_reads_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _bind()
    # sizes are checked before any pointer is used: 400,000 events cannot fit
    dummy = C.c_void_p(16)
    st = lib.abea_align_noalloc(dummy, dummy, 10, dummy, 200000, dummy, 400000, dummy, _Scalings(1, 0, 1, 0),
                                C.c_void_p(0))
    assert st == -1
    assert "scratch" in lib.abea_last_error().decode()
