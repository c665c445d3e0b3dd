"""ctypes front-end of the C oracle (oracle/gfaz_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker / CPU port.  The product package
(gfaz_gb300) never imports this module.

`build()` compiles the restatement with gcc + OpenMP into
oracle/_build/liboracle.so (plain C, builds the same on x86 and Arm).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gfaz_oracle.c")
LIB = os.path.join(HERE, "_build", "liboracle.so")

_lib = None
_P = ctypes.c_void_p
_U64 = ctypes.c_uint64


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c99", SRC, "-o", LIB],
                       check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_delta_encode.restype = ctypes.c_uint32
        L.orc_delta_encode.argtypes = [_P, _P, _U64, ctypes.c_int, ctypes.c_int]
        L.orc_delta_decode.restype = None
        L.orc_delta_decode.argtypes = [_P, _P, _U64, ctypes.c_int, ctypes.c_int]
        L.orc_grammar.restype = ctypes.c_int64
        L.orc_grammar.argtypes = [_P, _P, _U64, ctypes.c_int, _P, _P, _P, _U64, _P, ctypes.c_int]
        L.orc_rule_columns.restype = None
        L.orc_rule_columns.argtypes = [_P, _U64, _P, _P]
        L.orc_expand.restype = ctypes.c_int
        L.orc_expand.argtypes = [_P, _P, _U64, _P, _P, _U64, ctypes.c_uint32, ctypes.c_int, _P, _P,
                                 ctypes.c_int]
        L.orc_format_p_lines.restype = _U64
        L.orc_format_p_lines.argtypes = [_P, _P, _U64, _P, _P, _P, _P, _P]
        L.orc_format_w_lines.restype = _U64
        L.orc_format_w_lines.argtypes = [_P, _P, _U64, _P, _P, _P, _P, _P, _P, _P, _P]
        L.orc_append_encode.restype = ctypes.c_int
        L.orc_append_encode.argtypes = [_P, _P, _U64, _P, _P, _P, _U64, _P, _P, _P, _P, ctypes.c_int]
        L.orc_roundtrip_p.restype = _U64
        L.orc_roundtrip_p.argtypes = [_P, _P, _U64, ctypes.c_int, ctypes.c_int, _P, _U64, ctypes.c_int,
                                      _P, _P, _P, _P, _P, _P]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def compress(raw: np.ndarray, offsets: np.ndarray, rounds: int = 8, delta_round: int = 1,
             threads: int = 0) -> dict:
    """Delta + grammar rounds (compress_gfa's transform).  Returns the
    encoded stream, its offsets, the packed rulebook, layer_start, next_id
    and the decoded rule columns."""
    s = np.ascontiguousarray(raw, dtype=np.int32).copy()
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    ntrav = len(off) - 1
    L = lib()
    seed = L.orc_delta_encode(_p(s), _p(off), ntrav, delta_round, threads)
    if seed == 0:
        raise OverflowError("delta values too large for rule ID assignment")
    next_id = np.array([seed], dtype=np.uint32)
    eoff = np.zeros(ntrav + 1, np.uint64)
    cap = max(1, len(s))
    rules = np.zeros(cap, np.int64)
    rd = np.zeros(1, np.int32)
    nr = L.orc_grammar(_p(s), _p(off), ntrav, rounds, _p(next_id), _p(eoff), _p(rules), cap, _p(rd), threads)
    if nr < 0:
        raise RuntimeError("oracle rule buffer too small")
    rules = rules[:nr].copy()
    first = (rules >> 32).astype(np.int32)
    second = (rules & 0xFFFFFFFF).astype(np.uint32).view(np.int32)
    return {"encoded": s[:int(eoff[-1])].copy(), "enc_offsets": eoff, "rules": rules,
            "layer_start": int(seed), "next_id": int(next_id[0]), "rules_first": first,
            "rules_second": second, "rounds_done": int(rd[0])}


def expand(encoded, enc_offsets, rules_first, rules_second, min_id, delta_round, out_offsets,
           threads: int = 0) -> np.ndarray:
    enc = np.ascontiguousarray(encoded, dtype=np.int32)
    eoff = np.ascontiguousarray(enc_offsets, dtype=np.uint64)
    f = np.ascontiguousarray(rules_first, dtype=np.int32)
    g = np.ascontiguousarray(rules_second, dtype=np.int32)
    ooff = np.ascontiguousarray(out_offsets, dtype=np.uint64)
    out = np.zeros(max(1, int(ooff[-1])), np.int32)
    rc = lib().orc_expand(_p(enc), _p(eoff), len(eoff) - 1, _p(f), _p(g), len(f), int(min_id),
                          delta_round, _p(out), _p(ooff), threads)
    if rc != 0:
        raise ValueError("expanded length does not match the stored original length")
    return out[:int(ooff[-1])]


def _strcol(strings):
    bs = [s.encode() if isinstance(s, str) else bytes(s) for s in strings]
    off = np.zeros(len(bs) + 1, np.uint64)
    np.cumsum([len(b) for b in bs], out=off[1:])
    blob = np.frombuffer(b"".join(bs) + b"\0", dtype=np.uint8)
    return blob, off


def format_p(steps, offsets, names, overlaps) -> bytes:
    st = np.ascontiguousarray(steps, dtype=np.int32)
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    nb, no = _strcol(names)
    ob, oo = _strcol(overlaps)
    L = lib()
    n = L.orc_format_p_lines(_p(st), _p(off), len(off) - 1, _p(nb), _p(no), _p(ob), _p(oo), None)
    out = np.zeros(max(1, n), np.uint8)
    L.orc_format_p_lines(_p(st), _p(off), len(off) - 1, _p(nb), _p(no), _p(ob), _p(oo), _p(out))
    return out[:n].tobytes()


def format_w(steps, offsets, samples, haps, seqids, starts, ends) -> bytes:
    st = np.ascontiguousarray(steps, dtype=np.int32)
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    sb, so = _strcol(samples)
    qb, qo = _strcol(seqids)
    h = np.ascontiguousarray(haps, dtype=np.uint32)
    a = np.ascontiguousarray(starts, dtype=np.int64)
    e = np.ascontiguousarray(ends, dtype=np.int64)
    L = lib()
    args = [_p(st), _p(off), len(off) - 1, _p(sb), _p(so), _p(h), _p(qb), _p(qo), _p(a), _p(e)]
    n = L.orc_format_w_lines(*args, None)
    out = np.zeros(max(1, n), np.uint8)
    L.orc_format_w_lines(*args, _p(out))
    return out[:n].tobytes()


def append_encode(raw, offsets, delta_round, rules_first, rules_second, layers):
    """Append encoding (add-haplotypes): delta + stack encoder per stored
    layer.  layers rows are (k, start, end, flat_offset, element_count)."""
    s = np.ascontiguousarray(raw, dtype=np.int32).copy()
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    ntrav = len(off) - 1
    L = lib()
    L.orc_delta_encode(_p(s), _p(off), ntrav, delta_round, 1)
    lay = np.asarray(layers, dtype=np.int64).reshape(-1, 5)
    k = np.ascontiguousarray(lay[:, 0], dtype=np.int32)
    st = np.ascontiguousarray(lay[:, 1], dtype=np.uint32)
    en = np.ascontiguousarray(lay[:, 2], dtype=np.uint32)
    fo = np.ascontiguousarray(lay[:, 3], dtype=np.uint64)
    f = np.ascontiguousarray(rules_first, dtype=np.int32)
    g = np.ascontiguousarray(rules_second, dtype=np.int32)
    lens = np.zeros(ntrav, np.uint64)
    rc = L.orc_append_encode(_p(s), _p(off), ntrav, _p(lens), _p(f), _p(g), len(f), _p(st), _p(en),
                             _p(fo), _p(k), len(lay))
    if rc != 0:
        raise RuntimeError("rule column is truncated")
    parts = [s[int(off[t]):int(off[t]) + int(lens[t])] for t in range(ntrav)]
    return parts


def roundtrip_p(raw, offsets, rounds=8, delta_round=1, threads=0, phases=False, grammar=False):
    """CPU transform round trip (delta + grammar + expansion + P text);
    returns (text_bytes, encoded_len, nrules), plus (compress_ms,
    decompress_ms) wall-clock phase times when phases is set, plus the
    grammar (encoded stream, its offsets, packed rulebook) when grammar is
    set."""
    s = np.ascontiguousarray(raw, dtype=np.int32)
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    el = np.zeros(1, np.uint64)
    nr = np.zeros(1, np.uint64)
    ph = np.zeros(2, np.float64)
    gram = None
    if grammar:
        gram = (np.empty(max(1, len(s)), np.int32), np.empty(len(off), np.uint64), np.empty(max(1, len(s)), np.int64))
    g_ptrs = [_p(x) for x in gram] if gram else [None, None, None]
    n = lib().orc_roundtrip_p(_p(s), _p(off), len(off) - 1, rounds, delta_round, None, 0, threads,
                              _p(el), _p(nr), _p(ph), *g_ptrs)
    out = (int(n), int(el[0]), int(nr[0]))
    if phases:
        out += ((float(ph[0]), float(ph[1])),)
    if grammar:
        out += ((gram[0][:int(el[0])], gram[1], gram[2][:int(nr[0])]),)
    return out
