"""Pangenome growth: the restatement in oracle/growth.py reproduces the
reference `gfaz growth` output (tests/golden/growth.json, made by
tests/golden/make_growth_golden.py with the reference CLI) on every golden
container and grouping mode, from the containers' decoded traversals."""
import json
import os

import numpy as np
import pytest

import gfaz_format as fmt
from conftest import GOLDEN
from oracle import growth, oracle

with open(os.path.join(GOLDEN, "growth.json")) as fh:
    WANT = json.load(fh)
MODES = ["path", "sample-hap-seq", "sample-hap", "sample"]


def container_view(case):
    """Decoded traversals (paths, then walks), path names, walk columns and
    the node count of a golden container (oracle decode)."""
    f = fmt.read(os.path.join(GOLDEN, case + ".gfaz"))
    z = fmt.pre_entropy(f)
    lens = np.concatenate([z["sequence_lengths"], z["walk_lengths"]]).astype(np.uint64)
    olens = np.concatenate([z["original_path_lengths"], z["original_walk_lengths"]]).astype(np.uint64)
    enc = np.concatenate([z["paths"][:int(np.sum(z["sequence_lengths"]))], z["walks"][:int(np.sum(z["walk_lengths"]))]])
    eoff = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    ooff = np.concatenate([[0], np.cumsum(olens)]).astype(np.uint64)
    min_id = int(z["layers"][0, 1]) if len(z["layers"]) else 1 << 31
    x = oracle.expand(enc, eoff, z["rules_first"], z["rules_second"], min_id, int(z["delta_round"][0]), ooff)
    trav = [x[int(ooff[t]):int(ooff[t + 1])] for t in range(len(lens))]

    def strings(cat, lens_block):
        s, ls = fmt.unzstd(f[cat]), np.frombuffer(fmt.unzstd(f[lens_block]), "<u4")
        out, o = [], 0
        for n in ls:
            out.append(s[o:o + int(n)].decode() if o + int(n) <= len(s) else "")
            o += int(n)
        return out
    names = strings("names", "name_lengths") if len(z["sequence_lengths"]) else []
    walks = []
    if len(z["walk_lengths"]):
        haps = np.frombuffer(fmt.unzstd(f["walk_hap_indices"]), "<u4")
        walks = list(zip(strings("walk_sample_ids", "walk_sample_id_lengths"), [int(h) for h in haps],
                         strings("walk_seq_ids", "walk_seq_id_lengths")))
    num_nodes = len(fmt.unzstd(f["segment_seq_lengths"])) // 4
    return trav, names, walks, num_nodes


@pytest.mark.parametrize("case", sorted(WANT))
def test_growth_restatement_matches_reference(case):
    trav, names, walks, num_nodes = container_view(case)
    for mode in MODES:
        gid = growth.groups(names, walks, mode)
        hist = growth.coverage_hist(trav, gid, num_nodes)
        g = growth.growth_curve(hist, len(hist) - 1)
        assert growth.growth_text(num_nodes, hist, g, mode) == WANT[case][mode], (case, mode)
