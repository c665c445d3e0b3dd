"""C-ABI library checks that need no GPU: every declared symbol is exported,
the .gfaz container round-trips byte for byte, malformed input is rejected
with the reference's error prefixes, and the GPU entry points fail loudly
(never fall back) when no device is present."""
import ctypes
import os
import re

import numpy as np
import pytest

import gfaz_gb300 as gz
from gfaz_gb300 import _ffi
from conftest import GOLDEN, ROOT

CASES = ["tiny", "cfg1_mini", "cfg1_mini_d0", "cfg1_mini_d2_r3", "cfg1_mini_r1", "rich", "named", "cfg1"]


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gfaz_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gfz_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(_ffi.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 40
    for n in names:
        assert hasattr(lib, n), n
    # and the Python binding declares a signature for each
    assert set(names) == set(_ffi.SIGNATURES)


@pytest.mark.parametrize("case", CASES)
def test_container_roundtrip_is_identity(case):
    raw = open(os.path.join(GOLDEN, case + ".gfaz"), "rb").read()
    c = gz.CompressedData.from_bytes(raw)
    assert c.to_bytes() == raw
    z = np.load(os.path.join(GOLDEN, case + ".npz"))
    np.testing.assert_array_equal(c.sequence_lengths, z["sequence_lengths"])
    np.testing.assert_array_equal(c.walk_lengths, z["walk_lengths"])
    lay = c.layer_rule_ranges
    assert [(l.k, l.start_id, l.end_id, l.flattened_offset, l.element_count) for l in lay] == \
        [tuple(r) for r in z["layers"].tolist()]
    assert c.delta_round == int(z["delta_round"][0])
    paths = np.frombuffer(c.block("paths"), np.int32)
    np.testing.assert_array_equal(paths, z["paths"])


def test_serialize_to_file(tmp_path):
    raw = open(os.path.join(GOLDEN, "rich.gfaz"), "rb").read()
    c = gz.deserialize(os.path.join(GOLDEN, "rich.gfaz"))
    p = tmp_path / "copy.gfaz"
    gz.serialize(c, str(p))
    assert p.read_bytes() == raw


def test_malformed_containers_are_rejected(tmp_path):
    raw = open(os.path.join(GOLDEN, "tiny.gfaz"), "rb").read()
    bad_magic = b"XXXX" + raw[4:]
    with pytest.raises(RuntimeError, match="GFAZ serialization error: invalid file format"):
        gz.CompressedData.from_bytes(bad_magic)
    bad_version = raw[:4] + (6).to_bytes(4, "little") + raw[8:]
    with pytest.raises(RuntimeError, match="unsupported file version 6 \\(expected 5\\)"):
        gz.CompressedData.from_bytes(bad_version)
    for cut in (3, 10, 40, len(raw) // 2, len(raw) - 1):
        with pytest.raises(RuntimeError, match="GFAZ serialization error"):
            gz.CompressedData.from_bytes(raw[:cut])
    # a huge length prefix must not be trusted
    huge = bytearray(raw)
    huge[8:16] = (1 << 60).to_bytes(8, "little")
    with pytest.raises(RuntimeError, match="truncated or corrupted"):
        gz.CompressedData.from_bytes(bytes(huge))
    with pytest.raises(RuntimeError, match="failed to open input file"):
        gz.deserialize(str(tmp_path / "missing.gfaz"))


@pytest.mark.skipif(gz.has_gpu_backend(), reason="checks behaviour without a GPU")
def test_gpu_entry_points_fail_loudly_without_gpu(tmp_path):
    c = gz.deserialize(os.path.join(GOLDEN, "tiny.gfaz"))
    with pytest.raises(gz.GfazError) as e:
        gz.gfa_text(c)
    assert e.value.status_name == "CUDA"
    with pytest.raises(gz.GfazError) as e:
        gz.compress_file(os.path.join(GOLDEN, "tiny.gfa"))
    assert e.value.status_name == "CUDA"
    with pytest.raises(gz.GfazError):
        gz.Context(0)


def test_copy_bytes_in_pieces(monkeypatch):
    """Library buffers of 2 GiB and more are copied in pieces (ctypes.string_at
    takes a C int size); the pieces join to the same bytes."""
    import ctypes
    from gfaz_gb300 import _ffi
    data = bytes(range(256)) * 37
    buf = ctypes.create_string_buffer(data, len(data))
    monkeypatch.setattr(_ffi, "COPY_PIECE", 1000)
    assert _ffi.copy_bytes(ctypes.addressof(buf), len(data)) == data
    assert _ffi.copy_bytes(ctypes.c_void_p(ctypes.addressof(buf)), 5) == data[:5]
    assert _ffi.copy_bytes(None, 0) == b""


def test_copy_bytes_parallel():
    """Large library buffers are copied by several threads into a fresh bytes
    object; every piece split gives the same bytes, and the source is not
    touched."""
    import ctypes
    from gfaz_gb300 import _ffi
    rng = np.random.default_rng(5)
    data = rng.integers(0, 256, (5 << 20) + 12345, dtype=np.uint8).tobytes()
    buf = ctypes.create_string_buffer(data, len(data))
    for threads in (1, 2, 3, 4, 7):
        got = _ffi.copy_bytes(ctypes.addressof(buf), len(data), threads=threads)
        assert type(got) is bytes and got == data
    assert buf.raw == data
