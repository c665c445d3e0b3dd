"""gfz_inverse_delta_noalloc: the allocation-free inverse delta.

Its output must equal the inverse-delta step of the allocating path
(gfz_grammar_load with no rules + gfz_decode) on consecutive calls that
share the static scratch.  This file is collected last so that it also runs
after every other test in one process.
"""
import ctypes

import numpy as np
import pytest

from gfaz_gb300 import _ffi


def _segmented_prefix(x: np.ndarray, off: np.ndarray, rounds: int) -> np.ndarray:
    """Per-traversal wrapping int32 prefix sums, `rounds` times."""
    y = x.astype(np.int64)
    for _ in range(rounds):
        for t in range(len(off) - 1):
            a, b = int(off[t]), int(off[t + 1])
            if b > a:
                y[a:b] = np.cumsum(y[a:b]) & 0xFFFFFFFF
        y = y.astype(np.uint32).view(np.int32).astype(np.int64)
    return y.astype(np.int32)


def _case(seed: int, lengths):
    rng = np.random.default_rng(seed)
    off = np.zeros(len(lengths) + 1, dtype=np.uint64)
    off[1:] = np.cumsum(lengths)
    x = rng.integers(-(1 << 31), 1 << 31, size=int(off[-1]), dtype=np.int64).astype(np.int32)
    return x, off


def _decode_with_allocating_path(x: np.ndarray, off: np.ndarray, delta_round: int) -> np.ndarray:
    L = _ffi.lib()
    ntrav = len(off) - 1
    g = ctypes.c_void_p()
    _ffi.check(L.gfz_grammar_load(None, x.ctypes.data, off.ctypes.data, ntrav, None, None, 0, 1, delta_round,
                                  _ffi.WHERE_HOST, ctypes.byref(g)))
    try:
        out = np.empty(max(len(x), 1), dtype=np.int32)
        out_off = np.empty(ntrav + 1, dtype=np.uint64)
        n_out = ctypes.c_uint64()
        _ffi.check(L.gfz_decode(None, g, 0, ntrav, out.ctypes.data, out.size, ctypes.byref(n_out),
                                out_off.ctypes.data, _ffi.WHERE_HOST))
    finally:
        L.gfz_grammar_free(g)
    assert n_out.value == len(x)
    np.testing.assert_array_equal(out_off, off)
    return out[:len(x)]


def test_noalloc_rejects_oversized_stream():
    """The size limit is checked before any CUDA call or buffer access."""
    L = _ffi.lib()
    dummy = np.zeros(4, dtype=np.int32)
    offs = np.zeros(2, dtype=np.uint64)
    n = _ffi.NOALLOC_MAX_STEPS + 1
    st = L.gfz_inverse_delta_noalloc(dummy.ctypes.data, dummy.ctypes.data, n, offs.ctypes.data, 1, 1, None)
    assert _ffi.STATUS[st] == "INVALID"
    assert "limit of 67108864 steps" in L.gfz_last_error().decode()


@pytest.mark.gpu
def test_noalloc_matches_allocating_decode_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _ffi.lib()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)

    # call 1: ragged traversals (empty ones, one spanning many 4096-step
    # tiles), out of place, one round, legacy default stream
    lengths1 = [0, 1, 2, 4095, 4096, 4097, 0, 150_000, 17, 33_333, 0, 1] + [7919] * 40
    x1, off1 = _case(11, lengths1)
    want1 = _decode_with_allocating_path(x1, off1, 1)
    np.testing.assert_array_equal(want1, _segmented_prefix(x1, off1, 1))
    d_in1 = torch.from_numpy(x1).to(dev)
    d_out1 = torch.full_like(d_in1, 0x5A5A5A5A)
    d_off1 = torch.from_numpy(off1.view(np.int64)).to(dev)
    torch.cuda.synchronize()
    _ffi.check(L.gfz_inverse_delta_noalloc(d_in1.data_ptr(), d_out1.data_ptr(), len(x1), d_off1.data_ptr(),
                                           len(off1) - 1, 1, None))
    np.testing.assert_array_equal(d_out1.cpu().numpy(), want1)
    np.testing.assert_array_equal(d_in1.cpu().numpy(), x1)  # input untouched

    # call 2: fewer tiles than call 1 (stale descriptors stay behind in the
    # shared scratch), in place, two rounds, on a side stream
    lengths2 = [3, 0, 12_000, 9000, 1, 4096, 2]
    x2, off2 = _case(12, lengths2)
    want2 = _decode_with_allocating_path(x2, off2, 2)
    np.testing.assert_array_equal(want2, _segmented_prefix(x2, off2, 2))
    side = torch.cuda.Stream(device=dev)
    d_x2 = torch.from_numpy(x2).to(dev)
    d_off2 = torch.from_numpy(off2.view(np.int64)).to(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    _ffi.check(L.gfz_inverse_delta_noalloc(d_x2.data_ptr(), d_x2.data_ptr(), len(x2), d_off2.data_ptr(),
                                           len(off2) - 1, 2, ctypes.c_void_p(side.cuda_stream)))
    np.testing.assert_array_equal(d_x2.cpu().numpy(), want2)

    # a limit violation and bad offsets are errors, not device faults
    n = _ffi.NOALLOC_MAX_STEPS + 1
    st = L.gfz_inverse_delta_noalloc(d_x2.data_ptr(), d_x2.data_ptr(), n, d_off2.data_ptr(), len(off2) - 1, 1, None)
    assert _ffi.STATUS[st] == "INVALID"
    bad = off2.copy()
    bad[-1] += 1
    d_bad = torch.from_numpy(bad.view(np.int64)).to(dev)
    st = L.gfz_inverse_delta_noalloc(d_x2.data_ptr(), d_x2.data_ptr(), len(x2), d_bad.data_ptr(), len(off2) - 1,
                                     1, None)
    assert _ffi.STATUS[st] == "INVALID"
    np.testing.assert_array_equal(d_x2.cpu().numpy(), want2)  # rejected before any write
