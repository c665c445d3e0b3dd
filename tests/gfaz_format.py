"""Independent reader of the .gfaz v5 container, used by the tests and by
tests/golden/make_golden.py to pull pre-entropy arrays out of files.

Follows the field order of the reference writer
(src/codec/serialization.cpp:137-236): little-endian PODs, u64 length
prefixes, blocks as (u64 original_size, u64 n, n payload bytes).  Blocks
are decompressed through the system libzstd.so.1 via ctypes.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import struct

import numpy as np

MAGIC = 0x5A414647
VERSION = 5

_zstd = None


def zstd():
    global _zstd
    if _zstd is None:
        name = ctypes.util.find_library("zstd") or "libzstd.so.1"
        try:
            lib = ctypes.CDLL(name)
        except OSError:
            lib = ctypes.CDLL("libzstd.so.1")
        lib.ZSTD_decompress.restype = ctypes.c_size_t
        lib.ZSTD_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
        lib.ZSTD_isError.restype = ctypes.c_uint
        lib.ZSTD_isError.argtypes = [ctypes.c_size_t]
        lib.ZSTD_versionNumber.restype = ctypes.c_uint
        _zstd = lib
    return _zstd


def unzstd(block) -> bytes:
    orig, payload = block
    if orig == 0:
        return b""
    out = ctypes.create_string_buffer(orig)
    src = ctypes.create_string_buffer(payload, len(payload))
    n = zstd().ZSTD_decompress(out, orig, src, len(payload))
    if zstd().ZSTD_isError(n):
        raise ValueError("zstd decompression failed")
    return out.raw[:n]


class _R:
    def __init__(self, data: bytes):
        self.d, self.p = data, 0

    def take(self, n):
        if self.p + n > len(self.d):
            raise ValueError("truncated .gfaz")
        b = self.d[self.p:self.p + n]
        self.p += n
        return b

    def u32(self):
        return struct.unpack("<I", self.take(4))[0]

    def i32(self):
        return struct.unpack("<i", self.take(4))[0]

    def u64(self):
        return struct.unpack("<Q", self.take(8))[0]

    def s(self):
        return self.take(self.u64())

    def u32vec(self):
        n = self.u64()
        return np.frombuffer(self.take(4 * n), dtype="<u4").copy()

    def block(self):
        orig = self.u64()
        n = self.u64()
        return (orig, self.take(n))

    def optcol(self):
        tag = self.s()
        typ = self.take(1)
        num = self.u64()
        blocks = [self.block() for _ in range(8)]
        return (tag, typ, num, blocks)


def read(path_or_bytes) -> dict:
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    r = _R(bytes(data))
    if r.u32() != MAGIC:
        raise ValueError("magic mismatch")
    if r.u32() != VERSION:
        raise ValueError("version mismatch")
    f = {"header": r.s()}
    f["layers"] = []
    for _ in range(r.u64()):
        k = r.i32()
        start, end = r.u32(), r.u32()
        f["layers"].append((k, start, end, r.u64(), r.u64()))
    f["sequence_lengths"] = r.u32vec()
    f["original_path_lengths"] = r.u32vec()
    f["rules_first"] = r.block()
    f["rules_second"] = r.block()
    f["paths"] = r.block()
    f["delta_round"] = r.i32()
    for k in ("names", "name_lengths", "overlaps", "overlap_lengths",
              "segment_sequences", "segment_seq_lengths"):
        f[k] = r.block()
    f["segment_optional"] = [r.optcol() for _ in range(r.u64())]
    for k in ("link_from_ids", "link_to_ids", "link_from_orients", "link_to_orients",
              "link_overlap_nums", "link_overlap_ops"):
        f[k] = r.block()
    f["num_links"] = r.u64()
    f["link_optional"] = [r.optcol() for _ in range(r.u64())]
    f["num_jumps"] = r.u64()
    for k in ("jump_from_ids", "jump_from_orients", "jump_to_ids", "jump_to_orients",
              "jump_distances", "jump_distance_lengths", "jump_rest_fields", "jump_rest_lengths"):
        f[k] = r.block()
    f["num_containments"] = r.u64()
    for k in ("containment_container_ids", "containment_container_orients",
              "containment_contained_ids", "containment_contained_orients",
              "containment_positions", "containment_overlaps", "containment_overlap_lengths",
              "containment_rest_fields", "containment_rest_lengths"):
        f[k] = r.block()
    f["walk_lengths"] = r.u32vec()
    f["original_walk_lengths"] = r.u32vec()
    for k in ("walks", "walk_sample_ids", "walk_sample_id_lengths", "walk_hap_indices",
              "walk_seq_ids", "walk_seq_id_lengths", "walk_seq_starts", "walk_seq_ends"):
        f[k] = r.block()
    if r.p != len(r.d):
        raise ValueError("trailing bytes")
    return f


def i32(block) -> np.ndarray:
    return np.frombuffer(unzstd(block), dtype="<i4").copy()


def delta_decode(x: np.ndarray) -> np.ndarray:
    return np.cumsum(x.astype(np.int64)).astype(np.int64).astype(np.uint32).view(np.int32) \
        if len(x) else x.astype(np.int32)


def pre_entropy(f: dict) -> dict:
    """Decoded transform arrays: rule columns (delta-decoded), encoded P and
    W streams, lengths, layer ranges, delta_round."""
    return {
        "rules_first": delta_decode(i32(f["rules_first"])),
        "rules_second": delta_decode(i32(f["rules_second"])),
        "paths": i32(f["paths"]),
        "walks": i32(f["walks"]),
        "sequence_lengths": f["sequence_lengths"],
        "original_path_lengths": f["original_path_lengths"],
        "walk_lengths": f["walk_lengths"],
        "original_walk_lengths": f["original_walk_lengths"],
        "layers": np.array(f["layers"], dtype=np.int64).reshape(-1, 5),
        "delta_round": np.array([f["delta_round"]], dtype=np.int64),
    }
