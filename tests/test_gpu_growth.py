"""Pangenome growth with node coverage on the GPU: the `gfaz growth` table
equals the reference CLI's (tests/golden/growth.json) for every golden
container and grouping mode, through the Python API and the CLI; the
coverage histogram and curve equal the restatement (oracle/growth.py) on a
graph of 96 uneven walks, also when the group bitmap is built in passes
under a small HBM budget."""
import json
import os
import subprocess

import numpy as np
import pytest

import gfaz_gb300 as gz
from conftest import GOLDEN, ROOT
from gfaz_gb300 import synthetic
from oracle import growth

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "growth.json")) as fh:
    WANT = json.load(fh)
MODES = ["path", "sample-hap-seq", "sample-hap", "sample"]


@pytest.mark.parametrize("case", sorted(WANT))
def test_growth_matches_reference(case, gpu_ctx):
    c = gz.deserialize(os.path.join(GOLDEN, case + ".gfaz"))
    for mode in MODES:
        r = gz.compute_growth(c, group_by=mode, ctx=gpu_ctx)
        assert gz.growth_text(r, mode) == WANT[case][mode], (case, mode)


@pytest.mark.parametrize("case", ["rich", "pansn"])
def test_growth_cli(case):
    cli = os.path.join(ROOT, "gfaz_gb300", "gfaz")
    for mode in ("path", "sample-hap"):
        out = subprocess.run([cli, "growth", "-G", mode, os.path.join(GOLDEN, case + ".gfaz")], capture_output=True,
                             text=True, check=True).stdout
        assert out == WANT[case][mode]


def test_growth_compressed_here(gpu_ctx):
    c = gz.compress_file(os.path.join(GOLDEN, "pansn.gfa"), ctx=gpu_ctx)
    assert gz.growth_text(gz.compute_growth(c, group_by="sample-hap-seq", ctx=gpu_ctx),
                          "sample-hap-seq") == WANT["pansn"]["sample-hap-seq"]


@pytest.mark.parametrize("budget", [0, 400_000])
def test_growth_uneven_walks(budget, tmp_path, gpu_ctx):
    steps, off, _, meta = synthetic.cfg3_stream(seed=5, n_backbone=20_000, n_walks=96, median=3e3, sigma=1.5,
                                                hi=200_000, max_total=2_000_000)
    samples, haps, seqids, starts, ends = (list(x) for x in zip(*meta))
    nseg = int(np.abs(steps).max())
    lines = ["S\t%d\tA\n" % i for i in range(1, nseg + 1)]
    for t in range(len(off) - 1):
        walk = "".join(("<" if v < 0 else ">") + str(abs(int(v))) for v in steps[int(off[t]):int(off[t + 1])])
        lines.append("W\t%s\t%d\t%s\t%d\t%d\t%s\n" % (samples[t], haps[t], seqids[t], starts[t], ends[t], walk))
    path = tmp_path / "uneven.gfa"
    path.write_text("".join(lines))
    c = gz.compress_file(str(path), ctx=gpu_ctx)
    ctx = gz.Context(0)
    if budget:  # group bitmap rows in passes of one word
        ctx.set_option("hbm_budget", budget)
    trav = [steps[int(off[t]):int(off[t + 1])] for t in range(len(off) - 1)]
    for mode in ("path", "sample-hap"):
        r = gz.compute_growth(c, group_by=mode, ctx=ctx)
        gid = growth.groups([], list(zip(samples, haps, seqids)), mode)
        hist = growth.coverage_hist(trav, gid, r.num_nodes)
        np.testing.assert_array_equal(r.hist, hist)
        np.testing.assert_array_equal(r.growth, np.array(growth.growth_curve(hist, len(hist) - 1)))
