"""Append encoding (add-haplotypes).

Against the reference CLI's own add-haplotypes output
(tests/golden/append.*, made by tests/golden/make_append_golden.py;
add_haplotypes_workflow.cpp:336-379, 447-465, 579-592): the updated .gfaz
bytes, through the Python API, the `gfaz add-haplotypes` binary and the
server's concurrent append, and the decompressed GFA of the updated file.

Against the oracle's stack encoder (path_encoder.cpp:31-79 applied per
stored layer; the oracle is pinned to the same reference output): the
encoded streams of the appended traversals are identical for copies of
stored paths, mutated and reversed copies, random steps, long paths
spanning many chunks of the chunked pass, single-step paths, and
repetitive paths whose pairings cascade over long stretches, with every
chunk size of the chunked pass."""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

import gfaz_format as fmt
import gfaz_gb300 as gz
import append_cases
from conftest import GOLDEN, golden_raw
from oracle import oracle
from test_gpu_golden import _same_zstd

pytestmark = pytest.mark.gpu

CASES = ["cfg1", "cfg1_mini_d2_r3", "cfg1_mini_d0", "cfg1_mini_r1"]


@pytest.mark.parametrize("case,chunk", [(c, 0) for c in CASES] + [("cfg1", 8), ("cfg1_mini_r1", 8), ("cfg1", 1)])
def test_append_encoding_matches_oracle(case, chunk, manifest, tmp_path, gpu_ctx):
    """chunk 0: the automatic chunk ladder; 8: many fix-ups settling across
    short chunks; 1: every fix-up fails, so the one-thread-per-traversal
    pass runs."""
    ctx = gpu_ctx
    if chunk:
        ctx = gz.Context(0)
        ctx.set_option("append_chunk", chunk)
    meta = manifest["cases"][case]
    raw, off, _ = golden_raw(case, meta)
    src = os.path.join(GOLDEN, case + ".gfaz")
    before = fmt.pre_entropy(fmt.read(src))
    dr = int(before["delta_round"][0])
    npaths = len(before["sequence_lengths"])
    new = [p for p in append_cases.path_set(raw, off, npaths, seed=21)
           if append_cases.fits(p, dr, int(before["layers"][0][1]))]
    assert len(new) >= 6
    ap = tmp_path / "append.gfa"
    ap.write_text("".join(append_cases.p_line("app%d" % i, p) for i, p in enumerate(new)))
    c2 = gz.add_haplotypes(gz.deserialize(src), str(ap), ctx=ctx)
    out = tmp_path / "out.gfaz"
    gz.serialize(c2, str(out))
    after = fmt.pre_entropy(fmt.read(str(out)))

    noff = np.zeros(len(new) + 1, np.uint64)
    noff[1:] = np.cumsum([len(p) for p in new])
    want = oracle.append_encode(np.concatenate(new), noff, int(before["delta_round"][0]), before["rules_first"],
                                before["rules_second"], before["layers"])
    np_old = len(before["sequence_lengths"])
    got_lens = [int(x) for x in after["sequence_lengths"][np_old:]]
    assert got_lens == [len(w) for w in want]
    base = int(np.sum(before["sequence_lengths"]))
    assert np.array_equal(after["paths"][:base], before["paths"])
    assert np.array_equal(after["paths"][base:], np.concatenate(want))
    # and the appended paths read back as written
    lines = gz.extract_path_lines(c2, ["app%d" % i for i in range(len(new))], ctx=gpu_ctx)
    assert "".join(lines) == "".join(append_cases.p_line("app%d" % i, p) for i, p in enumerate(new))


def test_server_append_matches_add_haplotypes(manifest, tmp_path, gpu_ctx):
    """The server's concurrent append encodes exactly like add_haplotypes."""
    case = "cfg1"
    src = os.path.join(GOLDEN, case + ".gfaz")
    raw, off, z = golden_raw(case, manifest["cases"][case])
    new = [p for p in append_cases.path_set(raw, off, int(z["n_paths"][0]), seed=12)
           if append_cases.fits(p, int(z["delta_round"][0]), int(z["layers"][0, 1]))]
    text = "".join(append_cases.p_line("srv%d" % i, p) for i, p in enumerate(new))
    ap = tmp_path / "append.gfa"
    ap.write_text(text)
    c2 = gz.add_haplotypes(gz.deserialize(src), str(ap), ctx=gpu_ctx)
    names = ["srv%d" % i for i in range(len(new))]
    want = gz.extract_path_lines(c2, names, ctx=gpu_ctx)
    with gz.Server(gz.deserialize(src), workers=2) as srv:
        srv.wait(srv.submit_append(text))
        got = [srv.wait(srv.submit_path(n))[0] for n in names]
    assert got == want


@pytest.fixture(scope="module")
def append_golden():
    with open(os.path.join(GOLDEN, "append.json")) as fh:
        meta = json.load(fh)
    return meta, np.load(os.path.join(GOLDEN, "append.npz"))


def _check_updated(mine: bytes, case, manifest, append_golden, ctx):
    meta, z = append_golden
    m = meta["cases"][case]
    if _same_zstd(manifest):
        assert hashlib.sha256(mine).hexdigest() == m["updated_gfaz_sha256"]
    else:
        pe = fmt.pre_entropy(fmt.read(mine))
        for k, v in pe.items():
            np.testing.assert_array_equal(v, z[case + ":" + k], err_msg=k)
    text = gz.gfa_text(gz.CompressedData.from_bytes(mine), ctx=ctx)
    assert hashlib.sha256(text).hexdigest() == m["updated_gfa_out_sha256"]


@pytest.mark.parametrize("case,kind", append_cases.GOLDEN_CASES)
def test_append_matches_reference_gfaz(case, kind, manifest, append_golden, tmp_path, gpu_ctx):
    """add_haplotypes on the GPU writes the reference CLI's updated .gfaz."""
    text, _, _ = append_cases.golden_append(case, kind, manifest)
    ap = tmp_path / "append.gfa"
    ap.write_text(text)
    c2 = gz.add_haplotypes(gz.deserialize(os.path.join(GOLDEN, case + ".gfaz")), str(ap), ctx=gpu_ctx)
    _check_updated(c2.to_bytes(), case, manifest, append_golden, gpu_ctx)


@pytest.mark.parametrize("case,kind", [("cfg1", "P"), ("rich", "W")])
def test_append_cli_matches_reference_gfaz(case, kind, manifest, append_golden, tmp_path, gpu_ctx):
    """The same through the `gfaz add-haplotypes` binary."""
    from gfaz_gb300.build import CLI
    text, _, _ = append_cases.golden_append(case, kind, manifest)
    ap = tmp_path / "append.gfa"
    ap.write_text(text)
    out = tmp_path / "updated.gfaz"
    r = subprocess.run([CLI, "add-haplotypes", os.path.join(GOLDEN, case + ".gfaz"), str(ap), str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _check_updated(out.read_bytes(), case, manifest, append_golden, gpu_ctx)


@pytest.mark.parametrize("case,kind", [("cfg1", "P"), ("rich", "W")])
def test_server_append_matches_reference(case, kind, manifest, append_golden, gpu_ctx):
    """The server's concurrent append of the golden set answers with the
    lines of the reference's updated container."""
    text, steps, _ = append_cases.golden_append(case, kind, manifest)
    ap_lines = text.splitlines(keepends=True)
    with gz.Server(gz.deserialize(os.path.join(GOLDEN, case + ".gfaz")), workers=2) as srv:
        srv.wait(srv.submit_append(text))
        if kind == "P":
            got = [srv.wait(srv.submit_path("app%d" % i))[0] for i in range(len(steps))]
        else:
            got = []
            for ln in ap_lines:
                f = ln.rstrip("\n").split("\t")
                key = gz.WalkLookupKey(f[1], int(f[2]), f[3], -1 if f[4] == "*" else int(f[4]),
                                       -1 if f[5] == "*" else int(f[5]))
                got.append(srv.wait(srv.submit_walk(key))[0])
    # the appended lines read back as written (the reference's decompressed
    # updated file ends with them: its digest is checked above)
    assert got == ap_lines
