"""The C oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference CLI).  CPU only."""
import hashlib

import numpy as np
import pytest

from conftest import golden_raw
from oracle import oracle

CASES = ["tiny", "cfg1_mini", "cfg1_mini_d0", "cfg1_mini_d2_r3", "cfg1_mini_r1", "rich", "named", "cfg1"]


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_streams(case, manifest):
    meta = manifest["cases"][case]
    raw, off, z = golden_raw(case, meta)
    assert hashlib.sha256(raw.astype(np.int32).tobytes()).hexdigest() == meta["raw_steps_sha256"]
    npaths = int(z["n_paths"][0])
    r = oracle.compress(raw, off, rounds=meta["rounds"], delta_round=meta["delta_round"])
    lay = z["layers"]
    assert lay.shape[0] == 1
    assert (r["layer_start"], r["next_id"]) == (lay[0, 1], lay[0, 2])
    assert lay[0, 4] == 2 * (lay[0, 2] - lay[0, 1])
    np.testing.assert_array_equal(r["rules_first"], z["rules_first"])
    np.testing.assert_array_equal(r["rules_second"], z["rules_second"])
    enc, eoff = r["encoded"], r["enc_offsets"]
    np.testing.assert_array_equal(enc[:int(eoff[npaths])], z["paths"])
    np.testing.assert_array_equal(enc[int(eoff[npaths]):], z["walks"])
    lens = np.diff(eoff.astype(np.int64))
    np.testing.assert_array_equal(lens[:npaths], z["sequence_lengths"])
    np.testing.assert_array_equal(lens[npaths:], z["walk_lengths"])
    # the stored rule columns are the delta-coded form of the rulebook
    f = np.zeros(len(r["rules"]), np.int32)
    s = np.zeros(len(r["rules"]), np.int32)
    oracle.lib().orc_rule_columns(r["rules"].ctypes.data, len(r["rules"]), f.ctypes.data, s.ctypes.data)
    assert np.array_equal(np.cumsum(f.astype(np.int64)).astype(np.int32), z["rules_first"]) or len(f) == 0


@pytest.mark.parametrize("case", CASES)
def test_oracle_expansion_and_text(case, manifest):
    meta = manifest["cases"][case]
    raw, off, z = golden_raw(case, meta)
    npaths = int(z["n_paths"][0])
    enc = np.concatenate([z["paths"], z["walks"]]).astype(np.int32)
    lens = np.concatenate([z["sequence_lengths"], z["walk_lengths"]]).astype(np.uint64)
    eoff = np.zeros(len(lens) + 1, np.uint64)
    np.cumsum(lens, out=eoff[1:])
    x = oracle.expand(enc, eoff, z["rules_first"], z["rules_second"], int(z["layers"][0, 1]),
                      int(z["delta_round"][0]), off)
    np.testing.assert_array_equal(x, raw)
    if "p_text" not in z:
        return
    ptxt = z["p_text"].tobytes()
    # names/overlaps from the reference output lines
    lines = ptxt.decode().splitlines(keepends=True)
    names = [ln.split("\t")[1] for ln in lines]
    ovs = [ln.rstrip("\n").split("\t")[3] for ln in lines]
    assert oracle.format_p(x[:int(off[npaths])], off[:npaths + 1], names, ovs) == ptxt
    wtxt = z["w_text"].tobytes()
    if wtxt:
        wl = [ln.rstrip("\n").split("\t") for ln in wtxt.decode().splitlines()]
        woff = off[npaths:] - off[npaths]
        starts = [-1 if f[4] == "*" else int(f[4]) for f in wl]
        ends = [-1 if f[5] == "*" else int(f[5]) for f in wl]
        got = oracle.format_w(x[int(off[npaths]):], woff, [f[1] for f in wl], [int(f[2]) for f in wl],
                              [f[3] for f in wl], starts, ends)
        assert got == wtxt


def test_oracle_append_encoding_cascades():
    """A multi-round rulebook lets a rule symbol pair with the next push: the
    stack encoder replaces (R1, x) by R2 when (R1, x) is a later rule."""
    # canonical keys as a compressor stores them: 10 = (-1, -1), the
    # canonical form of (1, 1); 11 = (-10, 1) (child id < parent id)
    first = np.array([-1, -10], np.int32)
    second = np.array([-1, 1], np.int32)
    layers = [(2, 10, 12, 0, 4)]
    # raw 1,2,3 -> delta 1,1,1 -> push 1,1 -> reverse match -> -10;
    # push 1 -> (-10, 1) is rule 11 -> [11]
    parts = oracle.append_encode(np.array([1, 2, 3], np.int32), np.array([0, 3], np.uint64), 1, first, second,
                                 layers)
    assert parts[0].tolist() == [11]


@pytest.fixture(scope="module")
def append_golden():
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "append.json")) as fh:
        meta = json.load(fh)
    return meta, np.load(os.path.join(GOLDEN, "append.npz"))


@pytest.mark.parametrize("case,kind", __import__("append_cases").GOLDEN_CASES)
def test_oracle_append_matches_reference(case, kind, manifest, append_golden):
    """The oracle's append encoder against the reference CLI's
    add-haplotypes output (tests/golden/make_append_golden.py): the
    appended encoded traversals and their lengths, and everything the
    append leaves alone."""
    import append_cases
    meta, z = append_golden
    text, steps, before = append_cases.golden_append(case, kind, manifest)
    m = meta["cases"][case]
    assert hashlib.sha256(text.encode()).hexdigest() == m["append_sha256"]
    after = {k.split(":", 1)[1]: z[k] for k in z.files if k.startswith(case + ":")}
    for k in ("rules_first", "rules_second", "layers", "delta_round"):
        np.testing.assert_array_equal(after[k], before[k], err_msg=k)
    off = np.zeros(len(steps) + 1, np.uint64)
    np.cumsum([len(s) for s in steps], out=off[1:])
    parts = oracle.append_encode(np.concatenate(steps), off, int(before["delta_round"][0]), before["rules_first"],
                                 before["rules_second"], before["layers"])
    col, lens, orig = ("paths", "sequence_lengths", "original_path_lengths") if kind == "P" else \
        ("walks", "walk_lengths", "original_walk_lengths")
    old = len(before[lens])
    base = int(np.sum(before[lens]))
    np.testing.assert_array_equal(after[col][:base], before[col])
    np.testing.assert_array_equal(after[col][base:], np.concatenate(parts))
    np.testing.assert_array_equal(after[lens][:old], before[lens])
    assert [int(x) for x in after[lens][old:]] == [len(p) for p in parts]
    assert [int(x) for x in after[orig][old:]] == [len(s) for s in steps]
    other = ("walks", "walk_lengths") if kind == "P" else ("paths", "sequence_lengths")
    for k in other:
        np.testing.assert_array_equal(after[k], before[k], err_msg=k)
