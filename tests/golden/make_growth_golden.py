"""Golden outputs of the reference `gfaz growth` (src/cli/growth_command.cpp)
for every golden container and grouping mode, plus a PanSN-named case.

Run here (where the reference sources exist) after `oracle/build_ref.sh`:

    python tests/golden/make_growth_golden.py [path/to/oracle/_ref/gfaz]

Writes pansn.gfa (PanSN path names with and without coordinates, walks of
several samples), pansn.gfaz (the reference compressor's output) and
growth.json: {case: {group_by: the reference's stdout}}.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
MODES = ["path", "sample-hap-seq", "sample-hap", "sample"]
CASES = ["tiny", "named", "rich", "cfg1_mini", "cfg1_mini_d0", "cfg1_mini_d2_r3", "cfg1_mini_r1", "cfg1", "pansn"]


def pansn_gfa() -> str:
    """Segments 1..400; paths named sample#hap#contig(:start-end), some
    names without hap or contig, and walks; each traversal covers a random
    subset of the segments in order (seeded)."""
    rng = np.random.default_rng(17)
    lines = ["H\tVN:Z:1.0\n"]
    lines += ["S\t%d\t%s\n" % (i, "ACGT"[i % 4] * (1 + i % 5)) for i in range(1, 401)]
    names = ["HG002#1#chr1", "HG002#1#chr1:0-1000", "HG002#2#chr1", "HG003#1#chr1:5-99", "HG003#1#chr2",
             "HG003", "HG004#2", "HG004#2:10-20", "CHM13#0#chr1", "weird##x", "HG005#1#", "HG005#1##y:1-2"]
    for name in names:
        keep = np.sort(rng.choice(np.arange(1, 401), int(rng.integers(40, 300)), replace=False))
        steps = ",".join("%d%s" % (v, "-" if rng.random() < 0.05 else "+") for v in keep)
        lines.append("P\t%s\t%s\t*\n" % (name, steps))
    for sample, hap, seq in [("HG002", 1, "chr1"), ("HG002", 2, "chr1"), ("HG006", 0, "chrX"), ("HG002", 1, "chr3")]:
        keep = np.sort(rng.choice(np.arange(1, 401), int(rng.integers(40, 300)), replace=False))
        lines.append("W\t%s\t%d\t%s\t0\t%d\t%s\n" % (sample, hap, seq, len(keep),
                                                     "".join(">%d" % v for v in keep)))
    return "".join(lines)


def main() -> None:
    gfaz = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "oracle", "_ref", "gfaz")
    with open(os.path.join(HERE, "pansn.gfa"), "w") as fh:
        fh.write(pansn_gfa())
    subprocess.run([gfaz, "compress", "-j", "1", os.path.join(HERE, "pansn.gfa"), os.path.join(HERE, "pansn.gfaz")],
                   check=True, stdout=subprocess.DEVNULL)
    out = {}
    for case in CASES:
        src = os.path.join(HERE, case + ".gfaz")
        out[case] = {m: subprocess.run([gfaz, "growth", "-j", "1", "-G", m, src], check=True, capture_output=True,
                                       text=True).stdout for m in MODES}
    with open(os.path.join(HERE, "growth.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
