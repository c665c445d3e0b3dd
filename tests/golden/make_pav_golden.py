"""Golden outputs of the reference `gfaz pav` (src/cli/pav_command.cpp).

Run here (where the reference sources exist) after `oracle/build_ref.sh`
and make_growth_golden.py (which writes pansn.gfaz):

    python tests/golden/make_pav_golden.py [path/to/oracle/_ref/gfaz]

Writes the BED files pav_<case>.bed and pav_err_<kind>.bed and pav.json:
{"runs": [[case, bed, [options], stdout]], "errors": [[case, bed, stderr]]}.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

BEDS = {
    "rich": "# ranges on paths, on walks by their reference names, past the end, empty\n"
            "hap0\t0\t100\n"
            "hap0\t50\t5000\tmid\n"
            "hap0\t4000\t4000\tempty_range\n"
            "hap0\t100000\t200000\tpast_end\n"
            "hap3\t200\t900\n"
            "sample0#1#chr1:4800-11100\t0\t300\n"
            "sample1#1#chr3\t10\t400\tw3\n"
            "single\t0\t5\n"
            "empty_path\t0\t10\n"
            "hap0 20 60 spaced\n",
    "cfg1_mini": "".join("hap0\t%d\t%d\n" % (a, a + 1000) for a in range(0, 60000, 1000)) + "hap1\t0\t70000\tall\n",
    "pansn": "HG002#1#chr1\t0\t200\n"
             "HG002#1#chr1\t150\t900\tb\n"
             "HG003#1#chr1:5-99\t10\t500\n"
             "HG003\t0\t50\n"
             "weird##x\t0\t1000\n",
}
ERRS = {
    "unknown": "hap0\t0\t10\nno_such_path\t0\t10\n",
    "malformed": "hap0\tx\t10\n",
    "backwards": "hap0\t50\t10\n",
    "no_ranges": "# only a comment\n\n",
}
OPTS = [[], ["-S"], ["-H"], ["-M"], ["-B", "0.5"], ["-M", "-H", "-B", "0.25"]]


def main() -> None:
    gfaz = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "oracle", "_ref", "gfaz")
    out = {"runs": [], "errors": []}
    for case, text in BEDS.items():
        bed = "pav_%s.bed" % case
        with open(os.path.join(HERE, bed), "w") as fh:
            fh.write(text)
        for o in OPTS:
            r = subprocess.run([gfaz, "pav", "-t", "1", "-i", os.path.join(HERE, case + ".gfaz"), "-b",
                                os.path.join(HERE, bed)] + o, capture_output=True, text=True, check=True)
            out["runs"].append([case, bed, o, r.stdout])
    for kind, text in ERRS.items():
        bed = "pav_err_%s.bed" % kind
        with open(os.path.join(HERE, bed), "w") as fh:
            fh.write(text)
        r = subprocess.run([gfaz, "pav", "-i", os.path.join(HERE, "rich.gfaz"), "-b", os.path.join(HERE, bed)],
                           capture_output=True, text=True)
        assert r.returncode == 1
        out["errors"].append(["rich", bed, r.stderr.strip()])
    with open(os.path.join(HERE, "pav.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
