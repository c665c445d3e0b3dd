"""Generates the golden fixtures under tests/golden/ from the reference CLI.

Run here (where the reference sources exist) after `oracle/build_ref.sh`:

    python tests/golden/make_golden.py [path/to/oracle/_ref/gfaz]

For every case it writes
  <case>.gfa   - the input (only for the small hand-written / mini cases),
  <case>.gfaz  - the reference compressor's output,
  <case>.npz   - raw traversals (paths then walks), the reference's
                 pre-entropy arrays (rule columns, encoded streams, lengths,
                 layer ranges, delta_round), the reference decompressor's
                 P/W lines, and sha256 digests of the .gfaz and of the whole
                 decompressed GFA,
and a MANIFEST.json with the parameters and the zstd version used.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from gfaz_gb300 import synthetic  # noqa: E402
import gfaz_format  # noqa: E402

TINY = """H\tVN:Z:1.0
S\t1\tACGT\tLN:i:4
S\t2\tGG\tLN:i:2\tRC:i:10
S\t3\tTTA
S\t4\tC\tLN:i:1
L\t1\t+\t2\t+\t0M
L\t2\t+\t3\t+\t2M
L\t1\t+\t3\t-\t*
L\t3\t-\t4\t+\t1M
P\tpathB\t1+,3-,4+\t*
P\tpathA\t1+,2+,3+\t2M,1M
W\tsampleB\t1\tchr2\t*\t*\t>1<3>4
W\tsampleA\t0\tchr1\t0\t7\t>1>2>3
"""

# Optional-field types i/f/A/Z/B on S and L lines, J and C lines, a
# space-separated line, '*' walk coordinates, an empty path and a
# single-step path and walk.
RICH_EXTRA = """J\t1\t+\t3\t-\t100\tSC:i:1
J\t2\t-\t4\t+\t*
C\t1\t+\t2\t-\t3\t2M\tNM:i:0
C\t3\t+\t4\t+\t0\t*
"""


def rich_gfa() -> str:
    g = synthetic.cfg1(seed=11, n_backbone=300, bubble_every=10, n_paths=5)
    lines = ["H\tVN:Z:1.1\tTS:i:7"]
    seq = g.sequences()
    pos = 0
    for i, ln in enumerate(g.seq_lengths.tolist()):
        s = seq[pos:pos + ln].decode()
        pos += ln
        opt = []
        if i % 3 == 0:
            opt.append(f"LN:i:{ln}")
        if i % 5 == 1:
            opt.append(f"DP:f:{(i * 37 % 1000) / 7.0:.4f}")
        if i % 7 == 2:
            opt.append("XA:A:" + "ACGT"[i % 4])
        if i % 4 == 3:
            opt.append(f"ID:Z:seg_{i}")
        if i % 11 == 5:
            opt.append(f"BB:B:i,{i},{-i},{i * 3}")
        sep = " " if i == 17 else "\t"
        lines.append("S\t" + f"{i + 1}\t{s}" + ("" if not opt else sep + "\t".join(opt)))
    for j, (a, b) in enumerate(g.links.tolist()):
        ov = "*" if j % 9 == 0 else f"{j % 5}M"
        opt = f"\tRC:i:{j}" if j % 4 == 0 else ""
        opt += f"\tLF:f:{j / 3.0:.3f}" if j % 6 == 1 else ""
        lines.append(f"L\t{a}\t{'-' if j % 13 == 0 else '+'}\t{b}\t+\t{ov}{opt}")
    for name, p in zip(g.path_names, g.paths):
        steps = ",".join(f"{abs(v)}{'-' if v < 0 else '+'}" for v in p.tolist())
        lines.append(f"P\t{name}\t{steps}\t*")
    lines.append("P\tempty_path\t\t*")
    lines.append("P\tsingle\t5+\t*")
    w = synthetic.cfg3_stream(seed=12, n_backbone=300, n_walks=6, median=120, sigma=0.5,
                              lo=1, hi=600)
    steps, off, _, meta = w
    for k, (sample, hap, seqid, start, end) in enumerate(meta):
        ws = steps[int(off[k]):int(off[k + 1])]
        st = "*" if k == 2 else str(start)
        en = "*" if k == 2 else str(end)
        txt = "".join(f"{'<' if v < 0 else '>'}{abs(v)}" for v in ws.tolist())
        lines.append(f"W\t{sample}\t{hap}\t{seqid}\t{st}\t{en}\t{txt}")
    lines.append("W\tsolo\t0\tchrU\t*\t*\t>3")
    return "\n".join(lines) + "\n" + RICH_EXTRA


def named_gfa() -> str:
    """Non-numeric segment names: IDs come from S-line order."""
    g = synthetic.cfg1(seed=21, n_backbone=200, bubble_every=10, n_paths=4)
    lines = ["H\tVN:Z:1.0"]
    seq = g.sequences()
    pos = 0
    order = list(range(g.num_segments))
    for i in order:
        ln = int(g.seq_lengths[i])
        lines.append(f"S\tseg{i + 1}x\t{seq[pos:pos + ln].decode()}")
        pos += ln
    for a, b in g.links.tolist():
        lines.append(f"L\tseg{a}x\t+\tseg{b}x\t+\t0M")
    for name, p in zip(g.path_names, g.paths):
        steps = ",".join(f"seg{abs(v)}x{'-' if v < 0 else '+'}" for v in p.tolist())
        lines.append(f"P\t{name}\t{steps}\t*")
    return "\n".join(lines) + "\n"


def parse_pw(gfa_text: str):
    """Traversals of a decompressed (numeric) GFA: paths then walks."""
    paths, walks, plines, wlines = [], [], [], []
    for ln in gfa_text.splitlines(keepends=True):
        if ln.startswith("P\t"):
            f = ln.rstrip("\n").split("\t")
            steps = [] if f[2] == "" else [int(s[:-1]) * (-1 if s[-1] == "-" else 1) for s in f[2].split(",")]
            paths.append(np.array(steps, np.int32))
            plines.append(ln)
        elif ln.startswith("W\t"):
            f = ln.rstrip("\n").split("\t")
            ws, cur = [], None
            for ch in f[6]:
                if ch in "<>":
                    if cur is not None:
                        ws.append(cur)
                    cur = [ch, ""]
                else:
                    cur[1] += ch
            if cur is not None:
                ws.append(cur)
            walks.append(np.array([int(n) * (-1 if o == "<" else 1) for o, n in ws], np.int32))
            wlines.append(ln)
    return paths, walks, "".join(plines), "".join(wlines)


def run_case(gfaz_bin, name, gfa_text, rounds=8, delta=1, keep_input=True, extra=None, store_raw=True):
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "in.gfa")
        with open(src, "w") as fh:
            fh.write(gfa_text)
        out = os.path.join(td, "out.gfaz")
        subprocess.run([gfaz_bin, "compress", "-r", str(rounds), "-d", str(delta), "-j", "4", src, out],
                       check=True, capture_output=True)
        dec = os.path.join(td, "dec.gfa")
        subprocess.run([gfaz_bin, "decompress", "-j", "4", out, dec], check=True, capture_output=True)
        gfaz_bytes = open(out, "rb").read()
        dec_text = open(dec).read()
    f = gfaz_format.read(gfaz_bytes)
    pe = gfaz_format.pre_entropy(f)
    # raw traversals come from the original text through the same
    # resolution the decoder reproduces (numeric IDs in S-line order)
    paths, walks, ptxt, wtxt = parse_pw(dec_text)
    seqs = paths + walks
    off = np.zeros(len(seqs) + 1, np.uint64)
    np.cumsum([len(s) for s in seqs], out=off[1:])
    raw = np.concatenate(seqs).astype(np.int32) if seqs else np.zeros(0, np.int32)
    arrays = dict(pe)
    arrays.update(raw_offsets=off, n_paths=np.array([len(paths)]), rounds=np.array([rounds]))
    if store_raw:
        arrays.update(raw_steps=raw, p_text=np.frombuffer(ptxt.encode(), np.uint8),
                      w_text=np.frombuffer(wtxt.encode(), np.uint8))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    with open(os.path.join(HERE, name + ".gfaz"), "wb") as fh:
        fh.write(gfaz_bytes)
    if keep_input:
        with open(os.path.join(HERE, name + ".gfa"), "w") as fh:
            fh.write(gfa_text)
    meta = {"rounds": rounds, "delta_round": delta,
            "gfaz_sha256": hashlib.sha256(gfaz_bytes).hexdigest(),
            "gfa_out_sha256": hashlib.sha256(dec_text.encode()).hexdigest(),
            "gfa_in_sha256": hashlib.sha256(gfa_text.encode()).hexdigest(),
            "input_in_repo": keep_input,
            "raw_steps_sha256": hashlib.sha256(raw.tobytes()).hexdigest(),
            "p_text_sha256": hashlib.sha256(ptxt.encode()).hexdigest(),
            "w_text_sha256": hashlib.sha256(wtxt.encode()).hexdigest()}
    if extra:
        meta.update(extra)
    return meta


def main():
    gfaz_bin = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "oracle", "_ref", "gfaz")
    manifest = {"zstd_version": int(gfaz_format.zstd().ZSTD_versionNumber()), "cases": {}}
    cases = manifest["cases"]
    cases["tiny"] = run_case(gfaz_bin, "tiny", TINY)
    mini = synthetic.cfg1(seed=5, n_backbone=2000, n_paths=8).to_gfa().decode()
    cases["cfg1_mini"] = run_case(gfaz_bin, "cfg1_mini", mini)
    cases["cfg1_mini_d0"] = run_case(gfaz_bin, "cfg1_mini_d0", mini, delta=0, keep_input=False,
                                     extra={"input_from": "cfg1_mini"})
    cases["cfg1_mini_d2_r3"] = run_case(gfaz_bin, "cfg1_mini_d2_r3", mini, rounds=3, delta=2,
                                        keep_input=False, extra={"input_from": "cfg1_mini"})
    cases["cfg1_mini_r1"] = run_case(gfaz_bin, "cfg1_mini_r1", mini, rounds=1, keep_input=False,
                                     extra={"input_from": "cfg1_mini"})
    cases["rich"] = run_case(gfaz_bin, "rich", rich_gfa())
    cases["named"] = run_case(gfaz_bin, "named", named_gfa())
    # full-size config 1 (352k steps): input regenerated from the seed at
    # test time; only digests and pre-entropy arrays are kept
    full = synthetic.cfg1(seed=1).to_gfa().decode()
    cases["cfg1"] = run_case(gfaz_bin, "cfg1", full, keep_input=False, store_raw=False,
                             extra={"generator": "synthetic.cfg1(seed=1)"})
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)
    print(json.dumps(manifest, indent=1))


if __name__ == "__main__":
    main()
