"""gfaz_gb300 - GB300-native GFAz transform path.

Drop-in counterpart of the reference's `gfa_compression` Python module
(src/python/bindings.cpp) for the compression / decompression / extraction
/ append surface: same function names, argument names and defaults, same
error messages (raised as RuntimeError subclasses).  The traversal transform
(delta coding, 2-mer grammar rounds, expansion, inverse delta, P/W text)
runs on the GPU through libgfaz_gb300.so; containers are byte-compatible
.gfaz v5 files.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from ._ffi import (GfazError, LineMeta, ContainerInfo, GrammarInfo, WalkKeyC, check, copy_bytes, lib, take_bytes,
                   WHERE_HOST, WHERE_DEVICE, P_LINES, W_LINES)

DEFAULT_ROUNDS = 8
DEFAULT_FREQ_THRESHOLD = 2
DEFAULT_DELTA_ROUND = 1
DEFAULT_NUM_THREADS = 0

__all__ = [
    "DEFAULT_ROUNDS", "DEFAULT_FREQ_THRESHOLD", "DEFAULT_DELTA_ROUND", "DEFAULT_NUM_THREADS",
    "GfazError", "Context", "CompressedData", "GfaGraph", "WalkLookupKey", "LayerRuleRange", "Grammar",
    "has_gpu_backend", "compress", "compress_file", "compress_gfa_gpu", "decompress", "decompress_data",
    "decompress_to_host_graph_gpu", "serialize", "serialize_file", "deserialize", "deserialize_file",
    "write_gfa_from_compressed_data", "write_gfa_from_compressed_data_gpu", "gfa_text",
    "extract_path_line", "extract_path_lines", "extract_walk_line", "extract_walk_lines",
    "extract_walk_line_by_name", "extract_walk_lines_by_name", "add_haplotypes", "encode", "load_grammar",
    "Server",
]


def _cstr(s) -> bytes:
    return s if isinstance(s, bytes) else str(s).encode()


def has_gpu_backend() -> bool:
    """True when a CUDA device is usable (bindings.cpp:94-100)."""
    return bool(lib().gfz_has_gpu())


class Context:
    """One GPU and one CUDA stream.  `stream` may be an integer handle
    (e.g. torch.cuda.Stream().cuda_stream) or None for a private stream."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        h = ctypes.c_void_p()
        check(lib().gfz_context_create(device, ctypes.c_void_p(stream or 0), ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().gfz_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_timing(self, enabled: bool = True):
        check(lib().gfz_context_set_timing(self._h, int(enabled)))

    def set_option(self, name: str, value: int):
        check(lib().gfz_context_set_option(self._h, _cstr(name), int(value)))

    def kernel_stats(self, reset: bool = False) -> dict:
        import json
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        check(lib().gfz_context_kernel_stats(self._h, int(reset), ctypes.byref(p), ctypes.byref(n)))
        return json.loads(take_bytes(p, n.value).decode())


def _ctx(ctx: Optional[Context]):
    return ctx.handle if ctx is not None else None


@dataclass
class LayerRuleRange:
    k: int
    start_id: int
    end_id: int
    flattened_offset: int
    element_count: int


@dataclass
class WalkLookupKey:
    sample_id: str = ""
    hap_index: int = 0
    seq_id: str = ""
    seq_start: int = -1
    seq_end: int = -1


class CompressedData:
    """A .gfaz container (include/model/compressed_data.hpp:40-120)."""

    def __init__(self, handle):
        self._h = handle

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().gfz_compressed_free(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _info(self) -> ContainerInfo:
        info = ContainerInfo()
        check(lib().gfz_compressed_info(self._h, ctypes.byref(info)))
        return info

    @property
    def delta_round(self) -> int:
        return self._info().delta_round

    @property
    def num_links(self) -> int:
        return self._info().num_links

    @property
    def num_jumps(self) -> int:
        return self._info().num_jumps

    @property
    def num_containments(self) -> int:
        return self._info().num_containments

    def min_rule_id(self) -> int:
        return self._info().min_rule_id

    def total_rules(self) -> int:
        return self._info().total_rules

    @property
    def layer_rule_ranges(self) -> List[LayerRuleRange]:
        n = self._info().num_layers
        rows = (ctypes.c_int64 * (5 * max(n, 1)))()
        check(lib().gfz_compressed_layers(self._h, rows, n))
        return [LayerRuleRange(*[rows[5 * i + j] for j in range(5)]) for i in range(n)]

    def _u32(self, name) -> np.ndarray:
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        check(lib().gfz_compressed_u32(self._h, _cstr(name), ctypes.byref(p), ctypes.byref(n)))
        if n.value == 0:
            return np.zeros(0, np.uint32)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint32)), (n.value,)).copy()

    @property
    def sequence_lengths(self):
        return self._u32("sequence_lengths")

    @property
    def original_path_lengths(self):
        return self._u32("original_path_lengths")

    @property
    def walk_lengths(self):
        return self._u32("walk_lengths")

    @property
    def original_walk_lengths(self):
        return self._u32("original_walk_lengths")

    def block(self, name: str) -> bytes:
        """zstd-decoded bytes of a column (e.g. 'paths', 'rules_first')."""
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        check(lib().gfz_compressed_block(self._h, _cstr(name), ctypes.byref(p), ctypes.byref(n)))
        return take_bytes(p, n.value)

    def to_bytes(self) -> bytes:
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        check(lib().gfz_serialize_buffer(self._h, ctypes.byref(p), ctypes.byref(n)))
        return take_bytes(p, n.value)

    @staticmethod
    def from_bytes(data: bytes) -> "CompressedData":
        h = ctypes.c_void_p()
        buf = ctypes.create_string_buffer(bytes(data), len(data))
        check(lib().gfz_deserialize_buffer(buf, len(data), ctypes.byref(h)))
        return CompressedData(h)

    def copy(self) -> "CompressedData":
        return CompressedData.from_bytes(self.to_bytes())


@dataclass
class GfaGraph:
    """Decompressed graph (include/model/gfa_graph.hpp:104-126), traversals
    as numpy int32 arrays (sign = orientation)."""

    header_line: str = ""
    path_names: List[str] = field(default_factory=list)
    path_overlaps: List[str] = field(default_factory=list)
    paths: List[np.ndarray] = field(default_factory=list)
    walk_sample_ids: List[str] = field(default_factory=list)
    walk_hap_indices: List[int] = field(default_factory=list)
    walk_seq_ids: List[str] = field(default_factory=list)
    walk_seq_starts: List[int] = field(default_factory=list)
    walk_seq_ends: List[int] = field(default_factory=list)
    walks: List[np.ndarray] = field(default_factory=list)
    num_segments: int = 0
    num_links: int = 0
    num_jumps: int = 0
    num_containments: int = 0
    segment_names: List[str] = field(default_factory=list)      # filled by parse_gfa
    segment_sequences: List[str] = field(default_factory=list)  # filled by parse_gfa


def _split_lines(text: bytes) -> List[str]:
    s = text.decode()
    out, b = [], 0
    for i, ch in enumerate(s):
        if ch == "\n":
            out.append(s[b:i + 1])
            b = i + 1
    return out


# ---------------------------------------------------------------------------
# reference API (bindings.cpp:323-743)
# ---------------------------------------------------------------------------
def compress_file(gfa_file_path, rounds: int = DEFAULT_ROUNDS, threshold: int = DEFAULT_FREQ_THRESHOLD,
                  delta_round: int = DEFAULT_DELTA_ROUND, threads: int = DEFAULT_NUM_THREADS,
                  show_stats: bool = False, ctx: Optional[Context] = None) -> CompressedData:
    h = ctypes.c_void_p()
    check(lib().gfz_compress_file(_ctx(ctx), _cstr(gfa_file_path), int(rounds), int(threshold), int(delta_round),
                                  int(threads), int(bool(show_stats)), ctypes.byref(h)))
    return CompressedData(h)


def compress(gfa_file_path, num_rounds: int = DEFAULT_ROUNDS, freq_threshold: int = DEFAULT_FREQ_THRESHOLD,
             delta_round: int = DEFAULT_DELTA_ROUND, num_threads: int = DEFAULT_NUM_THREADS,
             show_stats: bool = False, ctx: Optional[Context] = None) -> CompressedData:
    return compress_file(gfa_file_path, num_rounds, freq_threshold, delta_round, num_threads, show_stats, ctx)


def compress_gfa_gpu(gfa_file_path, num_rounds: int = DEFAULT_ROUNDS, options=None,
                     ctx: Optional[Context] = None) -> CompressedData:
    """Reference GPU entry point (bindings.cpp:962-975); here the GPU path is
    the CPU-identical one (delta_round 1, threshold 2 as the reference GPU
    forces)."""
    return compress_file(gfa_file_path, num_rounds, 2, 1, 0, False, ctx)


def serialize(data: CompressedData, output_path) -> None:
    check(lib().gfz_serialize(data.handle, _cstr(output_path)))


serialize_file = serialize


def deserialize(input_path) -> CompressedData:
    h = ctypes.c_void_p()
    check(lib().gfz_deserialize(_cstr(input_path), ctypes.byref(h)))
    return CompressedData(h)


deserialize_file = deserialize


def write_gfa_from_compressed_data(data: CompressedData, output_path, num_threads: int = DEFAULT_NUM_THREADS,
                                   ctx: Optional[Context] = None) -> None:
    check(lib().gfz_write_gfa(_ctx(ctx), data.handle, _cstr(output_path), int(num_threads)))


def write_gfa_from_compressed_data_gpu(data: CompressedData, output_path, options=None,
                                       ctx: Optional[Context] = None) -> None:
    write_gfa_from_compressed_data(data, output_path, 0, ctx)


def gfa_text(data: CompressedData, num_threads: int = DEFAULT_NUM_THREADS, ctx: Optional[Context] = None) -> bytes:
    """The whole decompressed GFA (same bytes write_gfa_from_compressed_data writes)."""
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    check(lib().gfz_gfa_text(_ctx(ctx), data.handle, int(num_threads), ctypes.byref(p), ctypes.byref(n)))
    return take_bytes(p, n.value)


def _strarr(items: Sequence[str]):
    enc = [_cstr(x) for x in items]
    arr = (ctypes.c_char_p * max(len(enc), 1))(*enc)
    return arr, enc


def extract_path_lines(data: CompressedData, path_names: Sequence[str], num_threads: int = DEFAULT_NUM_THREADS,
                       ctx: Optional[Context] = None) -> List[str]:
    arr, keep = _strarr(path_names)
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    check(lib().gfz_extract_path_lines(_ctx(ctx), data.handle, arr, len(keep), int(num_threads), ctypes.byref(p),
                                       ctypes.byref(n)))
    return _split_lines(take_bytes(p, n.value))


def extract_path_line(data: CompressedData, path_name: str, num_threads: int = DEFAULT_NUM_THREADS,
                      ctx: Optional[Context] = None) -> str:
    return extract_path_lines(data, [path_name], num_threads, ctx)[0]


def extract_walk_lines(data: CompressedData, walk_keys: Sequence[WalkLookupKey],
                       num_threads: int = DEFAULT_NUM_THREADS, ctx: Optional[Context] = None) -> List[str]:
    keep = [(_cstr(k.sample_id), _cstr(k.seq_id)) for k in walk_keys]
    arr = (WalkKeyC * max(len(keep), 1))()
    for i, (k, (s, q)) in enumerate(zip(walk_keys, keep)):
        arr[i] = WalkKeyC(s, int(k.hap_index), q, int(k.seq_start), int(k.seq_end))
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    check(lib().gfz_extract_walk_lines(_ctx(ctx), data.handle, arr, len(keep), int(num_threads), ctypes.byref(p),
                                       ctypes.byref(n)))
    return _split_lines(take_bytes(p, n.value))


def extract_walk_line(data: CompressedData, sample_id: str, hap_index: int, seq_id: str, seq_start: int,
                      seq_end: int, num_threads: int = DEFAULT_NUM_THREADS, ctx: Optional[Context] = None) -> str:
    return extract_walk_lines(data, [WalkLookupKey(sample_id, hap_index, seq_id, seq_start, seq_end)],
                              num_threads, ctx)[0]


def extract_walk_lines_by_name(data: CompressedData, walk_names: Sequence[str],
                               num_threads: int = DEFAULT_NUM_THREADS, ctx: Optional[Context] = None) -> List[str]:
    arr, keep = _strarr(walk_names)
    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    check(lib().gfz_extract_walk_lines_by_name(_ctx(ctx), data.handle, arr, len(keep), int(num_threads),
                                               ctypes.byref(p), ctypes.byref(n)))
    return _split_lines(take_bytes(p, n.value))


def extract_walk_line_by_name(data: CompressedData, walk_name: str, num_threads: int = DEFAULT_NUM_THREADS,
                              ctx: Optional[Context] = None) -> str:
    return extract_walk_lines_by_name(data, [walk_name], num_threads, ctx)[0]


class Server:
    """Resident extraction server with continuous batching.

    The rules, their prefix buffers and every encoded traversal of `data`
    stay on the GPU.  submit_path / submit_walk / submit_append queue a
    request and return a ticket; wait(ticket) returns (line, latency_ms).
    Extractions that arrive while others run on the GPU join the next batch
    of a free worker (one CUDA stream per worker) while their expanded output
    fits `hbm_budget` bytes; an append is applied once no batch is in flight
    and is visible to every later request.  Lines equal extract_path_line /
    extract_walk_line on the same container (the reference has no server:
    each extraction decodes the whole file, extraction_workflow.cpp:207-357).
    """

    def __init__(self, data: CompressedData, hbm_budget: int = 40 << 30, workers: int = 2, device: int = 0):
        h = ctypes.c_void_p()
        check(lib().gfz_server_create(int(device), data.handle, int(hbm_budget), int(workers), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().gfz_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit_path(self, name: str) -> int:
        t = ctypes.c_uint64()
        check(lib().gfz_server_submit_path(self._h, _cstr(name), ctypes.byref(t)))
        return t.value

    def submit_walk(self, key: WalkLookupKey) -> int:
        s, q = _cstr(key.sample_id), _cstr(key.seq_id)
        k = WalkKeyC(s, int(key.hap_index), q, int(key.seq_start), int(key.seq_end))
        t = ctypes.c_uint64()
        check(lib().gfz_server_submit_walk(self._h, ctypes.byref(k), ctypes.byref(t)))
        return t.value

    def submit_append(self, gfa_text) -> int:
        b = _cstr(gfa_text)
        t = ctypes.c_uint64()
        check(lib().gfz_server_submit_append(self._h, b, len(b), ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, as_bytes: bool = False):
        p, n, ms = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_double()
        check(lib().gfz_server_wait(self._h, int(ticket), ctypes.byref(p), ctypes.byref(n), ctypes.byref(ms)))
        try:
            line = copy_bytes(p, n.value)
        finally:
            check(lib().gfz_server_release(self._h, int(ticket)))
        return (line if as_bytes else line.decode()), ms.value

    def wait_size(self, ticket: int):
        """Like wait, but releases the line without copying it: (bytes, latency_ms)."""
        n, ms, _, _, _ = self.wait_detail(ticket)
        return n, ms

    def wait_detail(self, ticket: int):
        """Waits for the request and releases its line without copying it:
        (bytes, latency_ms, queue_ms, service_ms, batch_size)."""
        n, ms, q, sv, b = ctypes.c_size_t(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_uint32()
        check(lib().gfz_server_collect(self._h, int(ticket), ctypes.byref(n), ctypes.byref(ms), ctypes.byref(q),
                                       ctypes.byref(sv), ctypes.byref(b)))
        return n.value, ms.value, q.value, sv.value, b.value

    def stats(self) -> dict:
        b, r, m = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().gfz_server_stats(self._h, ctypes.byref(b), ctypes.byref(r), ctypes.byref(m)))
        return {"batches": b.value, "requests": r.value, "max_batch": m.value}


def add_haplotypes(data: CompressedData, haplotypes_path, threads: int = DEFAULT_NUM_THREADS,
                   ctx: Optional[Context] = None) -> CompressedData:
    """Returns an updated copy; `data` is left unchanged (bindings.cpp:733-743)."""
    out = data.copy()
    check(lib().gfz_add_haplotypes(_ctx(ctx), out.handle, _cstr(haplotypes_path), int(threads)))
    return out


def _graph_from_handle(L, h) -> GfaGraph:
    """GfaGraph copy of a gfz_graph handle (the caller frees the handle)."""
    g = GfaGraph()

    def strings(name):
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        check(L.gfz_graph_strings(h, _cstr(name), ctypes.byref(p), ctypes.byref(n)))
        s = take_bytes(p, n.value).decode()
        return s.split("\n")[:-1] if s else []

    def trav(kind):
        sp, op, nt = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_uint64()
        check(L.gfz_graph_traversals(h, kind, ctypes.byref(sp), ctypes.byref(op), ctypes.byref(nt)))
        if nt.value == 0:
            return []
        off = np.ctypeslib.as_array(ctypes.cast(op, ctypes.POINTER(ctypes.c_uint64)), (nt.value + 1,)).copy()
        total = int(off[-1])
        steps = (np.ctypeslib.as_array(ctypes.cast(sp, ctypes.POINTER(ctypes.c_int32)), (total,)).copy()
                 if total else np.zeros(0, np.int32))
        return [steps[int(off[i]):int(off[i + 1])] for i in range(nt.value)]

    hp, sp_, ep, nw = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_uint64()
    check(L.gfz_graph_walk_numbers(h, ctypes.byref(hp), ctypes.byref(sp_), ctypes.byref(ep), ctypes.byref(nw)))
    hdr = ctypes.c_void_p()
    hn = ctypes.c_size_t()
    check(L.gfz_graph_strings(h, b"header", ctypes.byref(hdr), ctypes.byref(hn)))
    g.header_line = take_bytes(hdr, hn.value).decode()
    g.path_names = strings("path_names")
    g.path_overlaps = strings("path_overlaps")
    g.walk_sample_ids = strings("walk_sample_ids")
    g.walk_seq_ids = strings("walk_seq_ids")
    g.paths = trav(0)
    g.walks = trav(1)
    n = nw.value
    if n:
        g.walk_hap_indices = np.ctypeslib.as_array(ctypes.cast(hp, ctypes.POINTER(ctypes.c_uint32)), (n,)).tolist()
        g.walk_seq_starts = np.ctypeslib.as_array(ctypes.cast(sp_, ctypes.POINTER(ctypes.c_int64)), (n,)).tolist()
        g.walk_seq_ends = np.ctypeslib.as_array(ctypes.cast(ep, ctypes.POINTER(ctypes.c_int64)), (n,)).tolist()
    c = [ctypes.c_uint64() for _ in range(4)]
    check(L.gfz_graph_counts(h, *[ctypes.byref(x) for x in c]))
    g.num_segments, g.num_links, g.num_jumps, g.num_containments = [x.value for x in c]
    return g


# ---------------------------------------------------------------------------
# reference API (bindings.cpp:323-743)
def parse_gfa(file_path, threads: int = DEFAULT_NUM_THREADS, ctx: Optional[Context] = None,
              device: bool = True) -> GfaGraph:
    """parse / parse_gfa (bindings.cpp:659-660): the GFA file as a graph.
    device=True parses with the GPU front end (line index and P/W steps on
    the device), device=False with the host parser; the graphs are equal.
    The graph also carries segment_names / segment_sequences."""
    L = lib()
    h = ctypes.c_void_p()
    check(L.gfz_parse_gfa(_ctx(ctx) if device else None, _cstr(file_path), int(threads), int(bool(device)),
                          ctypes.byref(h)))
    try:
        g = _graph_from_handle(L, h)
        for name in ("segment_names", "segment_sequences"):
            p, n = ctypes.c_void_p(), ctypes.c_size_t()
            check(L.gfz_graph_strings(h, _cstr(name), ctypes.byref(p), ctypes.byref(n)))
            s = take_bytes(p, n.value).decode()
            setattr(g, name, s.split("\n")[:-1] if s else [])
        return g
    finally:
        L.gfz_graph_free(h)


parse = parse_gfa


@dataclass
class GrowthResult:
    """include/workflows/growth_workflow.hpp:27-32: hist[c] = nodes covered by
    exactly c of the N haplotype groups; growth[k] = expected nodes covered
    by a random k-subset (growth[0] unused)."""

    num_haplotypes: int = 0
    num_nodes: int = 0
    hist: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint64))
    growth: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))


_GROUP_BY = {"path": 0, "per-line": 0, "sample-hap-seq": 1, "panacus": 1, "sample-hap": 2, "haplotype": 2,
             "sample": 3}


def compute_growth(data: CompressedData, num_threads: int = DEFAULT_NUM_THREADS, group_by: str = "path",
                   ctx: Optional[Context] = None) -> GrowthResult:
    """compute_growth (src/workflows/growth_workflow.cpp:261; `gfaz growth`):
    the pangenome growth curve, node coverage computed on the GPU.  group_by
    takes the CLI's --group-by values."""
    if group_by not in _GROUP_BY:
        raise ValueError("unknown group_by %r; expected one of %s" % (group_by, sorted(_GROUP_BY)))
    nh, nn = ctypes.c_uint32(), ctypes.c_uint32()
    hp, gp = ctypes.c_void_p(), ctypes.c_void_p()
    L = lib()
    check(L.gfz_growth(_ctx(ctx), data.handle, int(num_threads), _GROUP_BY[group_by], ctypes.byref(nh),
                       ctypes.byref(nn), ctypes.byref(hp), ctypes.byref(gp)))
    r = GrowthResult(nh.value, nn.value)
    if nh.value:
        r.hist = np.frombuffer(take_bytes(hp, 8 * (nh.value + 1)), np.uint64).copy()
        r.growth = np.frombuffer(take_bytes(gp, 8 * (nh.value + 1)), np.float64).copy()
    return r


def growth_text(result: GrowthResult, group_by: str = "path") -> str:
    """The `gfaz growth` table (src/cli/growth_command.cpp:74-97)."""
    label = {0: "path", 1: "sample-hap-seq", 2: "sample-hap", 3: "sample"}[_GROUP_BY[group_by]]
    out = ["# gfaz growth (count=node, coverage>=1, quorum>=0)\n# group-by=%s\n" % label,
           "# num_haplotypes=%d num_nodes=%d\nk\tgrowth\n" % (result.num_haplotypes, result.num_nodes)]
    out += ["%d\t%.4f\n" % (k, result.growth[k]) for k in range(1, result.num_haplotypes + 1)]
    return "".join(out)


@dataclass
class PavResult:
    """include/workflows/pav_workflow.hpp:30-36: BED ranges (chrom, start,
    end, name), group names, denominators[range] and numerators[range,
    group] in bases."""

    ranges: List[tuple] = field(default_factory=list)
    group_names: List[str] = field(default_factory=list)
    denominators: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint64))
    numerators: np.ndarray = field(default_factory=lambda: np.zeros((0, 0), np.uint64))

    def ratios(self) -> np.ndarray:
        den = self.denominators.astype(np.float64)[:, None]
        with np.errstate(invalid="ignore", divide="ignore"):
            r = self.numerators.astype(np.float64) / den
        return np.where(den == 0, 0.0, r)


_PAV_GROUP = {"path": 0, "haplotype": 2, "sample-hap": 2, "sample": 3}


def compute_pav(data: CompressedData, bed_path, num_threads: int = DEFAULT_NUM_THREADS, group_by: str = "path",
                ctx: Optional[Context] = None) -> PavResult:
    """compute_pav (src/workflows/pav_workflow.cpp:475; `gfaz pav`): PAV
    ratios of the traversal groups over BED ranges on reference traversals;
    traversals are decoded and node membership built on the GPU.  group_by:
    "path" (each traversal name), "haplotype" (-H) or "sample" (-S)."""
    if group_by not in _PAV_GROUP:
        raise ValueError("unknown group_by %r; expected one of %s" % (group_by, sorted(_PAV_GROUP)))
    rs, gs, dp, np_ = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    rl, gl, nr, ng = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().gfz_pav(_ctx(ctx), data.handle, _cstr(bed_path), int(num_threads), _PAV_GROUP[group_by],
                        ctypes.byref(rs), ctypes.byref(rl), ctypes.byref(gs), ctypes.byref(gl), ctypes.byref(nr),
                        ctypes.byref(ng), ctypes.byref(dp), ctypes.byref(np_)))
    ranges = [tuple(l.split("\t")) for l in take_bytes(rs, rl.value).decode().split("\n")[:-1]]
    groups = take_bytes(gs, gl.value).decode().split("\n")[:-1]
    den = np.frombuffer(take_bytes(dp, 8 * nr.value), np.uint64).copy()
    num = np.frombuffer(take_bytes(np_, 8 * nr.value * ng.value), np.uint64).copy().reshape(nr.value, ng.value)
    return PavResult([(c, int(a), int(b), n) for c, a, b, n in ranges], groups, den, num)


def pav_text(result: PavResult, matrix: bool = False, binary_threshold: Optional[float] = None) -> str:
    """The `gfaz pav` table (src/cli/pav_command.cpp:95-137)."""
    r = result.ratios()

    def cell(x):
        return ("1" if x >= binary_threshold else "0") if binary_threshold is not None else "%.5g" % x
    out = ["chrom\tstart\tend\tname"]
    if matrix:
        out.append("".join("\t" + g for g in result.group_names) + "\n")
        for w, (c, a, b, n) in enumerate(result.ranges):
            out.append("%s\t%d\t%d\t%s%s\n" % (c, a, b, n, "".join("\t" + cell(x) for x in r[w])))
    else:
        out.append("\tgroup\tpav\n")
        for w, (c, a, b, n) in enumerate(result.ranges):
            for gi, g in enumerate(result.group_names):
                out.append("%s\t%d\t%d\t%s\t%s\t%s\n" % (c, a, b, n, g, cell(r[w, gi])))
    return "".join(out)


def decompress_data(data: CompressedData, threads: int = DEFAULT_NUM_THREADS,
                    ctx: Optional[Context] = None) -> GfaGraph:
    L = lib()
    h = ctypes.c_void_p()
    check(L.gfz_decompress_graph(_ctx(ctx), data.handle, int(threads), ctypes.byref(h)))
    try:
        return _graph_from_handle(L, h)
    finally:
        L.gfz_graph_free(h)


def decompress(data: CompressedData, num_threads: int = DEFAULT_NUM_THREADS,
               ctx: Optional[Context] = None) -> GfaGraph:
    return decompress_data(data, num_threads, ctx)


def decompress_to_host_graph_gpu(data: CompressedData, options=None, ctx: Optional[Context] = None) -> GfaGraph:
    return decompress_data(data, 0, ctx)


# ---------------------------------------------------------------------------
# transform hot path (device-resident grammar)
# ---------------------------------------------------------------------------
class Grammar:
    """Device-resident grammar produced by `encode` or `load_grammar`."""

    def __init__(self, handle, ctx: Optional[Context]):
        self._h = handle
        self._ctx = ctx

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().gfz_grammar_free(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        i = GrammarInfo()
        check(lib().gfz_grammar_info_get(self._h, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in GrammarInfo._fields_}

    def arrays(self):
        """(encoded int32, offsets uint64, rules int64) on the host."""
        info = self.info()
        enc = np.zeros(max(info["encoded_len"], 1), np.int32)
        off = np.zeros(info["ntrav"] + 1, np.uint64)
        rules = np.zeros(max(info["num_rules"], 1), np.int64)
        check(lib().gfz_grammar_copy(_ctx(self._ctx), self._h, enc.ctypes.data, off.ctypes.data, rules.ctypes.data,
                                     WHERE_HOST))
        return enc[:info["encoded_len"]], off, rules[:info["num_rules"]]

    def rule_columns(self):
        """Delta-coded first/second columns as stored in the container."""
        n = self.info()["num_rules"]
        f = np.zeros(max(n, 1), np.int32)
        s = np.zeros(max(n, 1), np.int32)
        check(lib().gfz_grammar_rule_columns(_ctx(self._ctx), self._h, f.ctypes.data, s.ctypes.data, WHERE_HOST))
        return f[:n], s[:n]

    def decode(self, t0: int = 0, t1: Optional[int] = None):
        """Expanded + inverse-delta steps and offsets of traversals [t0, t1)."""
        if t1 is None:
            t1 = self.info()["ntrav"]
        n = ctypes.c_uint64()
        off = np.zeros(t1 - t0 + 1, np.uint64)
        check(lib().gfz_decode(_ctx(self._ctx), self._h, t0, t1, None, 0, ctypes.byref(n), off.ctypes.data,
                               WHERE_HOST))
        out = np.zeros(max(n.value, 1), np.int32)
        check(lib().gfz_decode(_ctx(self._ctx), self._h, t0, t1, out.ctypes.data, out.size, ctypes.byref(n),
                               off.ctypes.data, WHERE_HOST))
        return out[:n.value], off

    def decode_text(self, t0: int, t1: int, mode: int = P_LINES, names=None, overlaps=None, hap_indices=None,
                    seq_ids=None, seq_starts=None, seq_ends=None, out_ptr: Optional[int] = None,
                    cap: int = 0, where: int = WHERE_HOST) -> int:
        """Emits GFA text for [t0, t1); returns its size.  Without out_ptr the
        text stays on the device (see `text`)."""
        keep = []

        def carr(items):
            if items is None:
                return None
            enc = [_cstr(x) for x in items]
            keep.append(enc)
            a = (ctypes.c_char_p * max(len(enc), 1))(*enc)
            keep.append(a)
            return a

        meta = LineMeta()
        meta.mode = mode
        meta.names = carr(names)
        meta.overlaps = carr(overlaps)
        meta.seq_ids = carr(seq_ids)
        if hap_indices is not None:
            h = np.ascontiguousarray(hap_indices, np.uint32)
            keep.append(h)
            meta.hap_indices = h.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        for fld, arr in (("seq_starts", seq_starts), ("seq_ends", seq_ends)):
            if arr is not None:
                a = np.ascontiguousarray(arr, np.int64)
                keep.append(a)
                setattr(meta, fld, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        size = ctypes.c_uint64()
        check(lib().gfz_decode_text(_ctx(self._ctx), self._h, t0, t1, ctypes.byref(meta),
                                    ctypes.c_void_p(out_ptr or 0), cap, ctypes.byref(size), where))
        return size.value

    def text_device(self):
        p, n = ctypes.c_void_p(), ctypes.c_uint64()
        check(lib().gfz_grammar_text(self._h, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def text(self, t0: int, t1: int, **kw) -> bytes:
        n = self.decode_text(t0, t1, **kw)
        buf = ctypes.create_string_buffer(max(n, 1))
        self.decode_text(t0, t1, out_ptr=ctypes.addressof(buf), cap=n, where=WHERE_HOST, **kw)
        return buf.raw[:n]


def encode(steps, offsets, rounds: int = DEFAULT_ROUNDS, delta_round: int = DEFAULT_DELTA_ROUND,
           threshold: int = DEFAULT_FREQ_THRESHOLD, ctx: Optional[Context] = None,
           device_ptr: Optional[int] = None) -> Grammar:
    """Compresses traversals steps[offsets[t]:offsets[t+1]] on the GPU.
    `steps` is a host int32 array, or pass device_ptr for device data."""
    off = np.ascontiguousarray(offsets, np.uint64)
    h = ctypes.c_void_p()
    if device_ptr is not None:
        check(lib().gfz_encode(_ctx(ctx), ctypes.c_void_p(device_ptr), off.ctypes.data, len(off) - 1, int(rounds),
                               int(threshold), int(delta_round), WHERE_DEVICE, ctypes.byref(h)))
    else:
        s = np.ascontiguousarray(steps, np.int32)
        check(lib().gfz_encode(_ctx(ctx), s.ctypes.data, off.ctypes.data, len(off) - 1, int(rounds), int(threshold),
                               int(delta_round), WHERE_HOST, ctypes.byref(h)))
    return Grammar(h, ctx)


def load_grammar(encoded, enc_offsets, rules_first_delta, rules_second_delta, min_rule_id: int,
                 delta_round: int, ctx: Optional[Context] = None) -> Grammar:
    """Loads a stored rulebook (delta-coded columns) and encoded traversals."""
    e = np.ascontiguousarray(encoded, np.int32)
    o = np.ascontiguousarray(enc_offsets, np.uint64)
    f = np.ascontiguousarray(rules_first_delta, np.int32)
    s = np.ascontiguousarray(rules_second_delta, np.int32)
    h = ctypes.c_void_p()
    check(lib().gfz_grammar_load(_ctx(ctx), e.ctypes.data, o.ctypes.data, len(o) - 1, f.ctypes.data, s.ctypes.data,
                                 len(f), int(min_rule_id), int(delta_round), WHERE_HOST, ctypes.byref(h)))
    return Grammar(h, ctx)
