"""abea_align_noalloc: the entry point for callers that cannot allocate device
memory (a framework whose own allocator owns the whole device, a service with a
device memory budget fixed at start-up).  Its buffers here come from the test
(torch tensors stand in for the caller's allocator); the call itself only uses
the library's fixed device array.  Checked against abea_align on two calls
in a row, bit-exact like every other parity test.  This file sorts last so a
run that stops at the first failure has already run every other test."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import abea

SCRATCH_BYTES = 32 << 20  # the library's fixed device array


def noalloc_need(seq_len, n_events):
    """Scratch bytes abea_align_noalloc needs for one read, as include/abea.h states it."""
    def a256(x):
        return (x + 255) // 256 * 256

    def r16(x):
        return (max(x, 1) + 15) // 16 * 16
    nk, ne = max(seq_len - 5, 0), max(n_events, 0)
    nb = ne + nk + 2 if (nk > 0 and ne > 0) else 0
    nb4 = (max(nb, 4) + 3) // 4 * 4
    return 256 + 2 * a256(4 * r16(ne)) + 4 * a256(4 * r16(nk)) + a256(128 * nb4) + a256(4 * nb4) + 512


def largest_fitting_events(seq_len):
    lo, hi = 1, 1 << 22
    while lo < hi:  # the largest n_events whose need fits the scratch
        mid = (lo + hi + 1) // 2
        lo, hi = (mid, hi) if noalloc_need(seq_len, mid) <= SCRATCH_BYTES else (lo, mid - 1)
    return lo


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


@pytest.mark.gpu
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


@pytest.mark.gpu
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


def test_noalloc_limit_is_the_stated_formula():
    """One event over the stated limit is refused before any device work; the
    read at the limit passes the size check (without a GPU it then stops at the
    device lookup).  Pointers are never used on either path, so dummies are safe
    only where no device exists; with a device only the refusal runs."""
    torch = pytest.importorskip("torch")
    if not os.path.exists(abea.LIB_PATH):
        abea.build()
    lib = _bind()
    seq_len = 86000
    ne = largest_fitting_events(seq_len)
    nb = ne + seq_len - 5 + 2
    assert 225000 < nb < 240000  # about 143 bytes per band
    dummy = C.c_void_p(16)
    st = lib.abea_align_noalloc(dummy, dummy, 2 * (ne + 1), dummy, seq_len, dummy, ne + 1, dummy,
                                _Scalings(1, 0, 1, 0), C.c_void_p(0))
    assert st == -1  # ABEA_ERR_INVALID_ARG
    assert "scratch" in lib.abea_last_error().decode()
    if not torch.cuda.is_available():
        st = lib.abea_align_noalloc(dummy, dummy, 2 * ne, dummy, seq_len, dummy, ne, dummy,
                                    _Scalings(1, 0, 1, 0), C.c_void_p(0))
        assert st != -1, lib.abea_last_error().decode()


@pytest.mark.gpu
def test_noalloc_read_at_its_limit_matches_align():
    """A read of about 230,000 bands, the largest the scratch holds: the same
    AlignedPairs as abea_align, on two calls in a row."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from abea_gb300 import synth
    lib = _bind()
    seq_len = 87500  # about 149,600 events: more than fit, the read keeps the first ones that do
    b = synth.make_batch("small", seed=21, lengths=[seq_len])
    ne = largest_fitting_events(seq_len)
    assert ne < int(b.n_events[0])
    seq, ev = b.sequence(0), b.read_events(0)[:ne]
    assert noalloc_need(seq_len, ne) <= SCRATCH_BYTES < noalloc_need(seq_len, ne + 1)
    stream = torch.cuda.current_stream().cuda_stream
    ref = abea.align(seq, ev, b.model, b.scalings[0])
    for _ in range(2):
        n, pairs = _noalloc(lib, torch, seq, ev, b.model, b.scalings[0], stream)
        assert n == len(ref)
        assert np.array_equal(pairs, ref)
