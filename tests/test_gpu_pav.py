"""PAV ratios over BED ranges with traversals decoded and node membership
built on the GPU: the `gfaz pav` output equals the reference CLI's
(tests/golden/pav.json, made by tests/golden/make_pav_golden.py) for every
golden BED file and option set (-S, -H, -M, -B), ranges on paths and on
walks by their reference names, past the traversal's end and empty; the
Python API formats the same table; BED errors give the same messages."""
import json
import os
import subprocess

import pytest

import gfaz_gb300 as gz
from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "pav.json")) as fh:
    WANT = json.load(fh)
CLI = os.path.join(ROOT, "gfaz_gb300", "gfaz")


@pytest.mark.parametrize("i", range(len(WANT["runs"])))
def test_pav_cli_matches_reference(i):
    case, bed, opts, want = WANT["runs"][i]
    got = subprocess.run([CLI, "pav", "-t", "1", "-i", os.path.join(GOLDEN, case + ".gfaz"), "-b",
                          os.path.join(GOLDEN, bed)] + opts, capture_output=True, text=True, check=True).stdout
    assert got == want


@pytest.mark.parametrize("case", ["rich", "pansn"])
def test_pav_python_api(case, gpu_ctx):
    c = gz.deserialize(os.path.join(GOLDEN, case + ".gfaz"))
    bed = os.path.join(GOLDEN, "pav_%s.bed" % case)
    for opts, group_by, kw in ((["-H"], "haplotype", {}), (["-M"], "path", {"matrix": True}),
                               (["-B", "0.5"], "path", {"binary_threshold": 0.5})):
        want = [r[3] for r in WANT["runs"] if r[0] == case and r[2] == opts][0]
        assert gz.pav_text(gz.compute_pav(c, bed, group_by=group_by, ctx=gpu_ctx), **kw) == want


@pytest.mark.parametrize("i", range(len(WANT["errors"])))
def test_pav_errors(i):
    case, bed, msg = WANT["errors"][i]
    r = subprocess.run([CLI, "pav", "-i", os.path.join(GOLDEN, case + ".gfaz"), "-b", os.path.join(GOLDEN, bed)],
                       capture_output=True, text=True)
    assert r.returncode == 1 and r.stderr.strip() == msg
