"""Append encoding (add-haplotypes) against the oracle's stack encoder
(path_encoder.cpp:31-79 applied per stored layer): the encoded streams of
the appended traversals are identical for copies of stored paths, mutated
and reversed copies, random steps, long paths spanning many chunks of the
chunked pass, single-step paths, and repetitive paths whose pairings
cascade over long stretches."""
import os

import numpy as np
import pytest

import gfaz_format as fmt
import gfaz_gb300 as gz
from conftest import GOLDEN, golden_raw
from oracle import oracle

pytestmark = pytest.mark.gpu

CASES = ["cfg1", "cfg1_mini_d2_r3", "cfg1_mini_d0", "cfg1_mini_r1"]


def _p_line(name, steps):
    return "P\t%s\t%s\t*\n" % (name, ",".join("%d%s" % (abs(int(v)), "+" if v > 0 else "-") for v in steps))


def _appended(raw, off, rng):
    paths = [raw[int(off[i]):int(off[i + 1])] for i in range(len(off) - 1)]
    hi = int(np.abs(raw).max())
    out = [paths[0].copy()]
    m = paths[1 % len(paths)].copy()
    idx = rng.integers(0, len(m), max(1, len(m) // 100))
    m[idx] = rng.integers(1, hi // 2 + 1, len(idx))
    out.append(m)
    out.append(-paths[2 % len(paths)][::-1])
    out.append(np.concatenate(paths[:6]))
    out.append((rng.integers(1, hi // 2 + 1, 5000) * rng.choice([-1, 1], 5000)).astype(np.int32))
    out.append(np.array([7], np.int32))
    out.append(np.tile(paths[3 % len(paths)][:2], 6000))
    out.append(np.tile(paths[4 % len(paths)][:7], 3000))
    out.append(np.tile(np.array([5, 6], np.int32), 9000))
    return [np.asarray(p, np.int32) for p in out]


def _fits(p, delta_round, min_id):
    """Whether the delta-coded path stays below the rule id region."""
    x = p.astype(np.int64)
    for _ in range(delta_round):
        x = np.concatenate([x[:1], np.diff(x)])
    return int(np.abs(x).max()) < min_id


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
    rng = np.random.default_rng(11)
    dr = int(before["delta_round"][0])
    new = [p for p in _appended(raw, np.asarray(off, np.uint64), rng) if _fits(p, dr, int(before["layers"][0][1]))]
    assert len(new) >= 6
    ap = tmp_path / "append.gfa"
    ap.write_text("".join(_p_line("app%d" % i, p) for i, p in enumerate(new)))
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
    assert "".join(lines) == "".join(_p_line("app%d" % i, p) for i, p in enumerate(new))


def test_server_append_matches_add_haplotypes(manifest, tmp_path, gpu_ctx):
    """The server's concurrent append encodes exactly like add_haplotypes."""
    case = "cfg1"
    src = os.path.join(GOLDEN, case + ".gfaz")
    raw, off, _ = golden_raw(case, manifest["cases"][case])
    new = _appended(raw, np.asarray(off, np.uint64), np.random.default_rng(12))
    text = "".join(_p_line("srv%d" % i, p) for i, p in enumerate(new))
    ap = tmp_path / "append.gfa"
    ap.write_text(text)
    c2 = gz.add_haplotypes(gz.deserialize(src), str(ap), ctx=gpu_ctx)
    names = ["srv%d" % i for i in range(len(new))]
    want = gz.extract_path_lines(c2, names, ctx=gpu_ctx)
    with gz.Server(gz.deserialize(src), workers=2) as srv:
        srv.wait(srv.submit_append(text))
        got = [srv.wait(srv.submit_path(n))[0] for n in names]
    assert got == want
