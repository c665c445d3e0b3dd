"""Calibrates the oracle port (oracle/gfaz_oracle.c) against the reference
CLI on the same input, as a CPU baseline.

TEST INFRASTRUCTURE ONLY.  The benchmark's reference arm times the port,
because the reference cannot be built where the GPU runs; this recipe, run
where the reference CLI was built (oracle/build_ref.sh), measures how the
port's speed compares with the reference's own code on one
chromosome-scale-shaped input at reduced size:

    python oracle/calibrate_ref.py [--segments 1000000] [--threads 8] > oracle/calibration.json

It writes a GFA file of the seeded chromosome-scale generator's 90 P-lines
(gfaz_gb300.synthetic.cfg2_stream, seed 2, the given segment count; S lines
of one base, no L lines), then
  * runs `gfaz compress -r 8 -d 1 -j T` and `gfaz decompress -j T` of the
    reference with GFA_COMPRESSION_DEBUG=1 and reads its phase timers: the
    compression transform is delta_transform + run_grammar_compression
    (compression_workflow.cpp), the decompression transform is "expand and
    stream paths" (gfa_writer.cpp's streaming writer);
  * runs the port's round trip with T threads on the same traversals and
    reads its two phases (delta + grammar + rule columns; expansion +
    inverse delta + P text);
and prints one JSON object with both sets of times (the minimum of the
repeats), the P-line text bytes and the ratios port / reference.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this folder comes first on the path; the package
# `oracle` is wanted instead of its module of the same name
sys.path = [ROOT] + [p for p in sys.path if os.path.abspath(p or ".") != HERE]


def write_gfa(path, steps, off, nseg):
    with open(path, "wb") as fh:
        fh.write(b"H\tVN:Z:1.0\n")
        fh.write(b"".join(b"S\t%d\tA\n" % i for i in range(1, nseg + 1)))
        for t in range(len(off) - 1):
            s = steps[int(off[t]):int(off[t + 1])]
            ids = np.abs(s).astype(np.int64)
            marks = np.where(s < 0, "-", "+")
            body = ",".join(f"{a}{m}" for a, m in zip(ids.tolist(), marks.tolist()))
            fh.write(f"P\thap{t}\t{body}\t*\n".encode())


def ms_after(label, text):
    m = re.search(re.escape(label) + r"\s*([0-9.]+) ms", text)
    if not m:
        raise RuntimeError(f"reference debug output lacks '{label}'")
    return float(m.group(1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--segments", type=int, default=1_000_000)
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--gfaz", default=os.path.join(HERE, "_ref", "gfaz"))
    ap.add_argument("--repeats", type=int, default=3)
    a = ap.parse_args()
    from gfaz_gb300 import synthetic
    from oracle import oracle

    steps, off, nseg = synthetic.cfg2_stream(seed=2, n_segments=a.segments, n_paths=90)
    env = dict(os.environ, GFA_COMPRESSION_DEBUG="1")
    ref_c, ref_d = [], []
    with tempfile.TemporaryDirectory() as td:
        gfa = os.path.join(td, "in.gfa")
        write_gfa(gfa, steps, off, nseg)
        gfaz = os.path.join(td, "in.gfaz")
        out = os.path.join(td, "out.gfa")
        for _ in range(a.repeats):
            r = subprocess.run([a.gfaz, "compress", "-r", "8", "-d", "1", "-j", str(a.threads), gfa, gfaz],
                               env=env, capture_output=True, text=True, check=True)
            log = r.stdout + r.stderr
            ref_c.append(ms_after("delta_transform (x1):", log) + ms_after("run_grammar_compression:", log))
            r = subprocess.run([a.gfaz, "decompress", "-j", str(a.threads), gfaz, out], env=env,
                               capture_output=True, text=True, check=True)
            ref_d.append(ms_after("expand and stream paths:", r.stdout + r.stderr))
        with open(out, "rb") as fh:
            ptext = sum(len(ln) for ln in fh if ln.startswith(b"P\t"))
    port_c, port_d = [], []
    n = 0
    for _ in range(a.repeats):
        n, _, _, (c_ms, d_ms) = oracle.roundtrip_p(steps, off, 8, 1, a.threads, phases=True)
        port_c.append(c_ms)
        port_d.append(d_ms)
    rc, rd, pc, pd = (min(x) for x in (ref_c, ref_d, port_c, port_d))
    res = {"input": f"cfg2_stream(seed=2, n_segments={a.segments}, n_paths=90): {len(steps)} steps, "
                    f"{nseg} segments",
           "threads": a.threads, "p_text_bytes": ptext, "port_text_bytes": n,
           "reference_ms": {"compress_transform": rc, "decompress_transform": rd},
           "port_ms": {"compress_transform": pc, "decompress_transform": pd},
           "reference_gbps": ptext / ((rc + rd) / 1e3) / 1e9, "port_gbps": n / ((pc + pd) / 1e3) / 1e9,
           "ratio_port_over_reference_time": {"compress": pc / rc, "decompress": pd / rd,
                                              "total": (pc + pd) / (rc + rd)},
           "when": time.strftime("%Y-%m-%d"), "repeats": a.repeats, "statistic": "minimum"}
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
