"""GFA inputs for the parser tests: edge cases of the reference parser's
traversal rules (src/io/gfa_parser.cpp:353-404, 600-625, 676-795,
1210-1218) and error cases with the message each must raise."""
from __future__ import annotations

import numpy as np

from gfaz_gb300 import synthetic


def _segs(n, named=False):
    return "".join("S\t%s\t%s\n" % (("n%dx" % i) if named else str(i), "ACGT"[: 1 + i % 4]) for i in range(1, n + 1))


# name -> GFA text (bytes)
CASES = {
    "numeric_edges": (
        "H\tVN:Z:1.0\n" + _segs(12)
        + "P\tp1\t1+,2-,3+\t*\n"
        + "P\tp2\t4+,,5-,\t4M,3M\n"            # empty pieces, trailing comma
        + "P\tp3\t6\t*\n"                        # no orientation: name is empty
        + "P\tp4\t007+,0+,12-\t*\tXX:i:1\n"      # leading zeros, id 0, extra field
        + "P  p5  1+,2+  *\n"                     # spaces as separators
        + "P\tp6\t\t*\n"                         # the steps field is '*'
        + "P\tp7\n"                              # name only
        + "W\ts1\t1\tchr1\t0\t100\tjunk>1<2><>3\tXY:Z:a\n"  # junk, empty name
        + "W\ts2\t2\tchr2\t*\t*\t>11<12\n"
        + "P\tp8\t1+,2+\r\n"                     # CR kept in the last piece
        + "W\ts3\t0\tchr3\t5\t6\n"               # no walk field
        + "\n#comment\n"
        + "P\tp9\t" + "0" * 5000 + "3+,4-\t*\n"  # a token longer than a tile
        + "W\tlong\t3\tc\t1\t2\t" + ">1<2" * 3000 + "\n"
        + "P\tp10\t9-,10+"                       # no final newline
    ).encode(),
    "named": (
        "S\tsA\tAC\nS\tsB\tG\nS\tsA\tT\nS\t3\tC\n"     # duplicate name, numeric-looking name
        + "P\tq1\tsA+,sB-,3+,zz+,sA-\t*\n"              # zz is not a segment
        + "W\tx\t1\tc\t0\t1\t>sA<sB>3>nope<sA\n"
    ).encode(),
    "out_of_order": "S\t2\tA\nS\t1\tC\nP\tp\t1+,2-\t*\nW\ts\t0\tc\t*\t*\t<1>2\n".encode(),
    "only_walks": (_segs(5) + "W\ta\t0\tc\t0\t9\t>1>2>3\nW\tb\t1\tc\t*\t*\t<5<4\n").encode(),
    "no_traversals": (_segs(3) + "L\t1\t+\t2\t-\t0M\n").encode(),
    "empty_file": b"",
    "header_only": b"H\tVN:Z:1.0",
}

def _long_lines(seed: int) -> bytes:
    """Long P and W lines (thousands of tokens, so the device lexer's
    whole-window path runs) mixing odd tokens: no orientation, a letter
    inside the name, empty pieces, id 0, leading zeros (also past 16 bytes),
    UINT32_MAX-bounded ids, junk and empty names in walks."""
    rng = np.random.default_rng(seed)
    p_tok = ["%d+", "%d-", "%d", "%da7+", "0%d-", "", "0+", "+", "%d+", "%d-", "00000000000000000000%d+",
             "%d+", "%d-"]
    w_tok = [">%d", "<%d", ">%dx", "<", ">0", "<000000000000000000%d", ">%d", "<%d", "7junk"]
    out = [_segs(50)]
    for t in range(6):
        toks = []
        for _ in range(3000):
            f = p_tok[int(rng.integers(0, len(p_tok)))]
            toks.append(f % int(rng.integers(1, 51)) if "%d" in f else f)
        out.append("P\tlong%d\t%s\t*\n" % (t, ",".join(toks)))
        ws = []
        for _ in range(3000):
            f = w_tok[int(rng.integers(0, len(w_tok)))]
            ws.append(f % int(rng.integers(1, 51)) if "%d" in f else f)
        out.append("W\ts%d\t%d\tc\t0\t9\t%s\n" % (t, t, "".join(ws)))
    out.append("P\tmax\t%s\t*\n" % ",".join(["4294967295+"] * 40 + ["3+"] * 40))
    return "".join(out).encode()


def _long_error(kind: str) -> bytes:
    good = ",".join("%d+" % (1 + i % 50) for i in range(2000))
    if kind == "p_overflow":
        return (_segs(50) + "P\tp\t%s,4294967296+,%s\t*\n" % (good, good)).encode()
    if kind == "p_no_digits":
        return (_segs(50) + "P\tp\t%s,x+,%s\t*\n" % (good, good)).encode()
    walk = "".join(">%d" % (1 + i % 50) for i in range(2000))
    return (_segs(50) + "W\ts\t1\tc\t0\t1\t%s>9999999999%s\n" % (walk, walk)).encode()


CASES["numeric_long_lines"] = _long_lines(3)

# name -> (text, message of the raised error)
ERRORS = {
    "p_no_digits": ((_segs(3) + "P\tp\t1+,x+\t*\n").encode(), "parse_uint32: no digits"),
    "p_overflow": ((_segs(3) + "P\tp\t1+,99999999999+\t*\n").encode(), "parse_uint32: overflow"),
    "w_no_digits": ((_segs(3) + "W\ts\t1\tc\t0\t1\t>1>y\n").encode(), "parse_uint32: no digits"),
    # a P error wins over a W error earlier in the file
    "p_before_w": ((_segs(3) + "W\ts\t1\tc\t0\t1\t>1>y\nP\tp\t99999999999+\t*\n").encode(),
                   "parse_uint32: overflow"),
    # the first W line with an error decides; its start/end after its steps
    "w_header_first": ((_segs(3) + "W\ts\t1\tc\t-\t1\t>1\nW\tt\t1\tc\t0\t1\t>x\n").encode(),
                       "parse_int64: no digits"),
    "w_steps_before_header": ((_segs(3) + "W\ts\t1\tc\t-\t1\t>x\n").encode(), "parse_uint32: no digits"),
    "s_overflow": (("S\t99999999999\tA\nP\tp\t1+\t*\n").encode(), "parse_uint32: overflow"),
    "p_overflow_long_line": (_long_error("p_overflow"), "parse_uint32: overflow"),
    "p_no_digits_long_line": (_long_error("p_no_digits"), "parse_uint32: no digits"),
    "w_overflow_long_line": (_long_error("w_overflow"), "parse_uint32: overflow"),
}


def random_text(seed: int, n_segments: int, n_paths: int, n_walks: int, named: bool = False) -> bytes:
    """A P + W GFA text from the config-2 generator's paths (numeric or
    named segments), P and W lines interleaved."""
    steps, off, _ = synthetic.cfg2_stream(seed=seed, n_segments=n_segments, n_paths=n_paths + n_walks)
    name = (lambda v: "n%dx" % v) if named else str
    parts = ["H\tVN:Z:1.0\n", _segs(n_segments, named)]
    for t in range(n_paths + n_walks):
        s = steps[int(off[t]):int(off[t + 1])]
        a = np.abs(s)
        if t % 2 == 0 and t // 2 < n_walks:
            parts.append("W\tsample%d\t%d\tchr%d\t0\t%d\t%s\n" % (
                t, t % 3, t, len(s), "".join(("<" if v < 0 else ">") + name(int(x)) for v, x in zip(s, a))))
        else:
            parts.append("P\tpath%d\t%s\t*\n" % (
                t, ",".join(name(int(x)) + ("-" if v < 0 else "+") for v, x in zip(s, a))))
    return "".join(parts).encode()


def fuzz_text(seed: int) -> bytes:
    """A random GFA text for front-end parity: numeric (in order, shuffled
    or duplicated) or named segments; P and W lines of random pieces
    (digits, orientations, letters, empty pieces, long zero runs, huge
    numbers), random blank runs between fields, CR, empty and unknown
    lines, optional fields, and sometimes no final newline.  Some texts
    are malformed on purpose (the parsers must then raise the same error)."""
    rng = np.random.default_rng(seed)
    nseg = int(rng.integers(1, 60))
    mode = int(rng.integers(0, 4))  # 0,1 numeric in order; 2 shuffled / duplicates; 3 named
    if mode == 3:
        names = ["s%d" % i for i in range(1, nseg + 1)]
    elif mode == 2:
        names = [str(int(x)) for x in rng.permutation(nseg) + 1] + [str(int(rng.integers(1, nseg + 1)))]
    else:
        names = [str(i) for i in range(1, nseg + 1)]
    pool = names + ["0", "007", "x", "99999999999", "4294967295", "4294967296", "", "1a"]
    weights = np.array([8.0] * len(names) + [0.3] * 8)
    weights /= weights.sum()

    def blank():
        return "".join(rng.choice(["\t", " "]) for _ in range(int(rng.integers(1, 3))))

    def name():
        return pool[int(rng.choice(len(pool), p=weights))]
    lines = []
    for n in names:
        opt = (blank() + "LN:i:%d" % int(rng.integers(0, 99))) if rng.random() < 0.2 else ""
        lines.append("S" + blank() + n + blank() + "ACGT"[: int(rng.integers(1, 5))] + opt)
    for t in range(int(rng.integers(1, 9))):
        if rng.random() < 0.5:
            pieces = []
            for _ in range(int(rng.integers(0, 400))):
                r = rng.random()
                pieces.append("" if r < 0.03 else name() + ("" if r < 0.06 else "+-"[int(rng.integers(0, 2))]))
            tail = blank() + "*" if rng.random() < 0.8 else ""
            lines.append("P" + blank() + "p%d" % t + blank() + ",".join(pieces) + tail)
        else:
            steps = "".join(("><"[int(rng.integers(0, 2))] if rng.random() < 0.97 else "") + name()
                            for _ in range(int(rng.integers(0, 400))))
            st = "*" if rng.random() < 0.3 else str(int(rng.integers(0, 100)))
            lines.append("W" + blank() + "smp%d" % (t % 3) + blank() + str(t % 2) + blank() + "c" + blank() + st +
                         blank() + "*" + blank() + ("junk" if rng.random() < 0.1 else "") + steps)
    for _ in range(int(rng.integers(0, 4))):
        lines.insert(int(rng.integers(0, len(lines) + 1)), rng.choice(["", "#x", "X\ty", "L\t1\t+\t2\t-\t0M"]))
    text = "\n".join(l + ("\r" if rng.random() < 0.05 else "") for l in lines)
    if rng.random() < 0.8:
        text += "\n"
    return text.encode()
