"""Pure-Python restatement of the reference GFA parser's traversal rules.

TEST INFRASTRUCTURE ONLY: the checker for the parser tests (host parser and
device front end) on small, hand-written inputs.  The product package never
imports it.

Follows src/io/gfa_parser.cpp:
  * line split on b"\\n" only, typed by the first byte; the last H line is
    the header (:353-404);
  * next_field: skip blanks (space / tab), take non-blanks (:124-131);
  * S lines assign ids 1.. in first-seen name order; names are numeric when
    every first-seen name is all digits and parses to its id (:600-625;
    parse_uint32 :68-90 raises on overflow);
  * resolve_node_id: empty -> 0, numeric -> parse_uint32 (digits up to the
    first non-digit; "no digits" / "overflow" raise), else the name table,
    0 when absent (:1210-1218);
  * P (:676-728): name, steps field, overlap = rest after blanks; steps split
    on ',', empty pieces skipped, last byte = orientation ('-' reverse);
  * W (:730-795): five fields, walk field; steps start at '>' / '<' and run to
    the next marker; other bytes skipped, empty names skipped; start / end
    "*" -> -1, else parse_int64.
Errors are raised as ValueError with the value parser's message.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

BLANK = (0x20, 0x09)


def _next_field(line: bytes, pos: int) -> Tuple[bytes, int]:
    n = len(line)
    while pos < n and line[pos] in BLANK:
        pos += 1
    b = pos
    while pos < n and line[pos] not in BLANK:
        pos += 1
    return line[b:pos], pos


def parse_uint32(s: bytes) -> int:
    if not s:
        raise ValueError("parse_uint32: empty")
    v, any_digit = 0, False
    for c in s:
        if c < 0x30 or c > 0x39:
            break
        any_digit = True
        d = c - 0x30
        if v > 429496729 or (v == 429496729 and d > 5):
            raise ValueError("parse_uint32: overflow")
        v = v * 10 + d
    if not any_digit:
        raise ValueError("parse_uint32: no digits")
    return v


def parse_int64(s: bytes) -> int:
    if not s:
        raise ValueError("parse_int64: empty")
    i, neg = 0, s[0] == 0x2D
    if neg:
        i = 1
    if i >= len(s):
        raise ValueError("parse_int64: no digits")
    v = 0
    for c in s[i:]:
        if c < 0x30 or c > 0x39:
            break
        v = v * 10 + (c - 0x30)
        if (not neg and v > 2**63 - 1) or (neg and v > 2**63):
            raise ValueError("parse_int64: overflow")
    return -v if neg else v


def _i32(v: int) -> int:
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= 1 << 31 else v


def parse(text: bytes) -> Dict[str, object]:
    """Traversal view of a GFA text: header, segment count, paths (name,
    overlap, steps) and walks (sample, hap, seq id, start, end, steps)."""
    lines = [ln for ln in text.split(b"\n") if ln]
    header = b""
    S, P, W = [], [], []
    for ln in lines:
        t = ln[:1]
        if t == b"H":
            header = ln
        elif t == b"S":
            S.append(ln)
        elif t == b"P":
            P.append(ln)
        elif t == b"W":
            W.append(ln)
    ids: Dict[bytes, int] = {}
    numeric = True
    for ln in S:
        name, _ = _next_field(ln, 1)
        if name in ids:
            continue
        nid = len(ids) + 1
        if numeric and not (name and all(0x30 <= c <= 0x39 for c in name)):
            numeric = False
        if numeric and parse_uint32(name) != nid:
            numeric = False
        ids[name] = nid

    def resolve(name: bytes) -> int:
        if not name:
            return 0
        if numeric:
            return parse_uint32(name)
        return ids.get(name, 0)

    paths: List[Tuple[bytes, bytes, List[int]]] = []
    for ln in P:
        name, pos = _next_field(ln, 1)
        steps, pos = _next_field(ln, pos)
        while pos < len(ln) and ln[pos] in BLANK:
            pos += 1
        out = []
        for piece in steps.split(b","):
            if not piece:
                continue
            nid = resolve(piece[:-1])
            if nid:
                out.append(_i32(-nid if piece[-1:] == b"-" else nid))
        paths.append((name, ln[pos:], out))
    walks = []
    for ln in W:
        pos = 1
        f = []
        for _ in range(6):
            x, pos = _next_field(ln, pos)
            f.append(x)
        sample, hap, seqid, st, en, walk = f
        out = []
        p = 0
        while p < len(walk):
            o = walk[p]
            if o not in (0x3E, 0x3C):
                p += 1
                continue
            e = p + 1
            while e < len(walk) and walk[e] not in (0x3E, 0x3C):
                e += 1
            if e > p + 1:
                nid = resolve(walk[p + 1:e])
                if nid:
                    out.append(_i32(-nid if o == 0x3C else nid))
            p = e
        h = 0
        for c in hap:
            h = (h * 10 + (c - 0x30)) & 0xFFFFFFFF
        walks.append((sample, h, seqid, -1 if st == b"*" else parse_int64(st),
                      -1 if en == b"*" else parse_int64(en), out))
    return {"header": header, "segments": len(ids), "paths": paths, "walks": walks}
