"""ctypes binding of libgfaz_gb300.so (C ABI in include/gfaz_gb300.h).

The library is built in-tree (gfaz_gb300/build.py).  Importing this module
fails loudly when it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgfaz_gb300.so")

P = ctypes.c_void_p
PP = ctypes.POINTER(ctypes.c_void_p)
I = ctypes.c_int
U64 = ctypes.c_uint64
I64 = ctypes.c_int64
U32 = ctypes.c_uint32
SZ = ctypes.c_size_t
CP = ctypes.c_char_p
PSZ = ctypes.POINTER(ctypes.c_size_t)
PU64 = ctypes.POINTER(ctypes.c_uint64)

GFZ_OK = 0
STATUS = {0: "OK", -1: "INVALID", -2: "IO", -3: "FORMAT", -4: "CUDA", -5: "DEVICE", -6: "NOT_FOUND",
          -7: "BUFFER", -8: "INTERNAL"}
WHERE_HOST, WHERE_DEVICE = 0, 1
P_LINES, W_LINES = 0, 1


class WalkKeyC(ctypes.Structure):
    _fields_ = [("sample_id", CP), ("hap_index", U32), ("seq_id", CP), ("seq_start", I64), ("seq_end", I64)]


class ContainerInfo(ctypes.Structure):
    _fields_ = [("num_paths", U64), ("num_walks", U64), ("num_links", U64), ("num_jumps", U64),
                ("num_containments", U64), ("num_layers", U64), ("total_rules", U64),
                ("min_rule_id", U32), ("reserved", U32), ("delta_round", ctypes.c_int32),
                ("reserved2", ctypes.c_int32)]


class GrammarInfo(ctypes.Structure):
    _fields_ = [("ntrav", U64), ("encoded_len", U64), ("num_rules", U64), ("layer_start", U32),
                ("next_id", U32), ("rounds_done", ctypes.c_int32), ("delta_round", ctypes.c_int32)]


class LineMeta(ctypes.Structure):
    _fields_ = [("mode", I), ("names", ctypes.POINTER(CP)), ("overlaps", ctypes.POINTER(CP)),
                ("hap_indices", ctypes.POINTER(U32)), ("seq_ids", ctypes.POINTER(CP)),
                ("seq_starts", ctypes.POINTER(I64)), ("seq_ends", ctypes.POINTER(I64))]


# name -> (restype, argtypes); every symbol declared in include/gfaz_gb300.h
SIGNATURES = {
    "gfz_last_error": (CP, []),
    "gfz_version": (CP, []),
    "gfz_free": (None, [P]),
    "gfz_has_gpu": (I, []),
    "gfz_zstd_version": (ctypes.c_uint, []),
    "gfz_context_create": (I, [I, P, PP]),
    "gfz_context_destroy": (None, [P]),
    "gfz_context_set_timing": (I, [P, I]),
    "gfz_context_kernel_stats": (I, [P, I, PP, PSZ]),
    "gfz_context_set_option": (I, [P, CP, I64]),
    "gfz_compress_file": (I, [P, CP, I, U64, I, I, I, PP]),
    "gfz_serialize": (I, [P, CP]),
    "gfz_serialize_buffer": (I, [P, PP, PSZ]),
    "gfz_deserialize": (I, [CP, PP]),
    "gfz_deserialize_buffer": (I, [P, SZ, PP]),
    "gfz_compressed_free": (None, [P]),
    "gfz_write_gfa": (I, [P, P, CP, I]),
    "gfz_gfa_text": (I, [P, P, I, PP, PSZ]),
    "gfz_extract_path_lines": (I, [P, P, ctypes.POINTER(CP), SZ, I, PP, PSZ]),
    "gfz_extract_walk_lines": (I, [P, P, ctypes.POINTER(WalkKeyC), SZ, I, PP, PSZ]),
    "gfz_extract_walk_lines_by_name": (I, [P, P, ctypes.POINTER(CP), SZ, I, PP, PSZ]),
    "gfz_add_haplotypes": (I, [P, P, CP, I]),
    "gfz_decompress_graph": (I, [P, P, I, PP]),
    "gfz_parse_gfa": (I, [P, CP, I, I, PP]),
    "gfz_pav": (I, [P, P, CP, I, I, PP, PSZ, PP, PSZ, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                    PP, PP]),
    "gfz_growth": (I, [P, P, I, I, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32), PP, PP]),
    "gfz_graph_free": (None, [P]),
    "gfz_compressed_info": (I, [P, ctypes.POINTER(ContainerInfo)]),
    "gfz_compressed_layers": (I, [P, ctypes.POINTER(I64), SZ]),
    "gfz_compressed_u32": (I, [P, CP, PP, PSZ]),
    "gfz_compressed_block": (I, [P, CP, PP, PSZ]),
    "gfz_graph_traversals": (I, [P, I, PP, PP, PU64]),
    "gfz_graph_strings": (I, [P, CP, PP, PSZ]),
    "gfz_graph_walk_numbers": (I, [P, PP, PP, PP, PU64]),
    "gfz_graph_counts": (I, [P, PU64, PU64, PU64, PU64]),
    "gfz_encode": (I, [P, P, P, U64, I, U64, I, I, PP]),
    "gfz_grammar_info_get": (I, [P, ctypes.POINTER(GrammarInfo)]),
    "gfz_grammar_copy": (I, [P, P, P, P, P, I]),
    "gfz_grammar_rule_columns": (I, [P, P, P, P, I]),
    "gfz_grammar_load": (I, [P, P, P, U64, P, P, U64, U32, I, I, PP]),
    "gfz_grammar_free": (None, [P]),
    "gfz_decode": (I, [P, P, U64, U64, P, U64, PU64, P, I]),
    "gfz_decode_text": (I, [P, P, U64, U64, ctypes.POINTER(LineMeta), P, U64, PU64, I]),
    "gfz_grammar_text": (I, [P, PP, PU64]),
    "gfz_server_create": (I, [I, P, U64, I, PP]),
    "gfz_server_submit_path": (I, [P, CP, PU64]),
    "gfz_server_submit_walk": (I, [P, ctypes.POINTER(WalkKeyC), PU64]),
    "gfz_server_submit_append": (I, [P, CP, SZ, PU64]),
    "gfz_server_wait": (I, [P, U64, PP, PSZ, ctypes.POINTER(ctypes.c_double)]),
    "gfz_server_request_times": (I, [P, U64, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_uint32)]),
    "gfz_server_release": (I, [P, U64]),
    "gfz_server_collect": (I, [P, U64, PSZ, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint32)]),
    "gfz_server_stats": (I, [P, PU64, PU64, PU64]),
    "gfz_server_destroy": (None, [P]),
    "gfz_inverse_delta_noalloc": (I, [P, P, U64, P, U64, I, P]),
}
NOALLOC_MAX_STEPS = 1 << 26

_lib = None


class GfazError(RuntimeError):
    """Error raised for a failed library call; `status` is the gfz_status."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status
        self.status_name = STATUS.get(status, str(status))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m gfaz_gb300.build` "
                              "(the GFAz transform has no implementation without it)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int):
    if status != GFZ_OK:
        msg = lib().gfz_last_error().decode(errors="replace")
        raise GfazError(status, msg)


COPY_PIECE = 1 << 30
# Buffers of at least this many bytes are copied by several threads.
PARALLEL_COPY = 64 << 20

_new_bytes = ctypes.pythonapi.PyBytes_FromStringAndSize
_new_bytes.restype = ctypes.py_object
_new_bytes.argtypes = [ctypes.c_void_p, ctypes.c_ssize_t]


def copy_bytes(ptr, n: int, threads: int = 0) -> bytes:
    """n bytes at ptr.  Small buffers go through ctypes.string_at (which
    takes its size as a C int, hence COPY_PIECE).  Larger ones are copied
    into a new, not yet initialised bytes object (PyBytes_FromStringAndSize
    with no source), in pieces by `threads` threads (0: one per core, at
    most 16); ctypes releases the GIL around each memmove, so the pieces
    and the first touch of the new pages run in parallel."""
    if not n:
        return b""
    addr = ptr.value if isinstance(ptr, ctypes.c_void_p) else int(ptr)
    if n <= COPY_PIECE and n < PARALLEL_COPY:
        return ctypes.string_at(addr, n)
    out = _new_bytes(None, n)
    dst = ctypes.cast(ctypes.c_char_p(out), ctypes.c_void_p).value
    nth = threads if threads > 0 else min(16, os.cpu_count() or 1)
    piece = max(1 << 20, -(-n // max(nth, 1)))
    piece = -(-piece // 4096) * 4096
    spans = [(o, min(piece, n - o)) for o in range(0, n, piece)]
    if len(spans) == 1:
        ctypes.memmove(dst, addr, n)
        return out
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=len(spans)) as pool:
        list(pool.map(lambda sp: ctypes.memmove(dst + sp[0], addr + sp[0], sp[1]), spans))
    return out


def take_bytes(ptr: ctypes.c_void_p, n: int) -> bytes:
    """Copies a library-allocated buffer and frees it."""
    try:
        return copy_bytes(ptr, n)
    finally:
        if ptr:
            lib().gfz_free(ptr)
