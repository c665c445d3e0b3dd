"""Generates the add-haplotypes golden fixtures from the reference CLI.

Run here (where the reference sources exist) after `oracle/build_ref.sh` and
tests/golden/make_golden.py:

    python tests/golden/make_append_golden.py [path/to/oracle/_ref/gfaz]

For every case it appends a deterministic set of P-lines or W-lines
(tests/append_cases.py) to a golden container with the reference's
`gfaz add-haplotypes`, decompresses the result with the reference's
`gfaz decompress`, and records in append.npz, under the case's prefix,
  <case>:<array>  - the updated container's pre-entropy arrays (rule
                    columns, encoded P and W streams, lengths, layer ranges,
                    delta_round),
and in append.json the append set's parameters, the sha256 of the appended
GFA text, of the updated .gfaz and of its decompressed GFA.  The updated
containers themselves are not stored: they are the golden container plus
these arrays, and the digests pin their bytes.
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
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

import append_cases  # noqa: E402
import gfaz_format  # noqa: E402


def main():
    gfaz_bin = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "oracle", "_ref", "gfaz")
    with open(os.path.join(HERE, "MANIFEST.json")) as fh:
        manifest = json.load(fh)
    out_meta = {"zstd_version": manifest["zstd_version"], "cases": {}}
    arrays = {}
    for case, kind in append_cases.GOLDEN_CASES:
        text, _, _ = append_cases.golden_append(case, kind, manifest)
        with tempfile.TemporaryDirectory() as td:
            app = os.path.join(td, "append.gfa")
            with open(app, "w") as fh:
                fh.write(text)
            upd = os.path.join(td, "updated.gfaz")
            subprocess.run([gfaz_bin, "add-haplotypes", "-j", "4", os.path.join(HERE, case + ".gfaz"), app, upd],
                           check=True, capture_output=True)
            dec = os.path.join(td, "dec.gfa")
            subprocess.run([gfaz_bin, "decompress", "-j", "4", upd, dec], check=True, capture_output=True)
            gfaz_bytes = open(upd, "rb").read()
            dec_bytes = open(dec, "rb").read()
        pe = gfaz_format.pre_entropy(gfaz_format.read(gfaz_bytes))
        for k, v in pe.items():
            arrays[case + ":" + k] = np.asarray(v)
        out_meta["cases"][case] = {
            "kind": kind, "lines": text.count("\n"),
            "append_sha256": hashlib.sha256(text.encode()).hexdigest(),
            "updated_gfaz_sha256": hashlib.sha256(gfaz_bytes).hexdigest(),
            "updated_gfa_out_sha256": hashlib.sha256(dec_bytes).hexdigest()}
    np.savez_compressed(os.path.join(HERE, "append.npz"), **arrays)
    with open(os.path.join(HERE, "append.json"), "w") as fh:
        json.dump(out_meta, fh, indent=1, sort_keys=True)
    print(json.dumps(out_meta, indent=1))


if __name__ == "__main__":
    main()
