"""Resident extraction server: every response equals the stand-alone
extraction of the same container, for a request alone and in a mix of
concurrent, interleaved and repeated requests; appends are seen by later
requests; the HBM budget bounds batches; errors keep the extraction
workflow's messages."""
import os

import pytest

import gfaz_gb300 as gz
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["tiny", "rich", "cfg1", "cfg1_mini_d2_r3"]


def _keys(c):
    paths, walks, seen = [], [], set()
    for line in gz.gfa_text(c).decode().splitlines():
        f = line.split("\t")
        if f[0] == "P":
            paths.append(f[1])
        elif f[0] == "W":
            k = (f[1], int(f[2]), f[3], -1 if f[4] == "*" else int(f[4]), -1 if f[5] == "*" else int(f[5]))
            if k not in seen:
                seen.add(k)
                walks.append(gz.WalkLookupKey(*k))
    return paths, walks


def _load(case):
    return gz.deserialize(os.path.join(GOLDEN, case + ".gfaz"))


@pytest.mark.parametrize("case", CASES)
def test_server_alone_and_in_the_mix(case, gpu_ctx):
    c = _load(case)
    paths, walks = _keys(c)
    assert paths or walks
    want_p = {n: gz.extract_path_line(c, n, ctx=gpu_ctx) for n in paths}
    want_w = [gz.extract_walk_lines(c, [k], ctx=gpu_ctx)[0] for k in walks]
    with gz.Server(c, workers=2) as srv:
        for n in paths:
            line, ms = srv.wait(srv.submit_path(n))
            assert line == want_p[n] and ms >= 0
        for k, w in zip(walks, want_w):
            assert srv.wait(srv.submit_walk(k))[0] == w
        tickets = []
        for _ in range(3):
            for n in paths:
                tickets.append(("p", n, srv.submit_path(n)))
            for i, k in enumerate(walks):
                tickets.append(("w", i, srv.submit_walk(k)))
        for kind, key, t in reversed(tickets):
            line, ms = srv.wait(t)
            assert line == (want_p[key] if kind == "p" else want_w[key])
        st = srv.stats()
        assert st["requests"] == len(paths) + len(walks) + len(tickets)
        if len(tickets) >= 16:
            assert st["max_batch"] > 1, st


def test_server_budget_limits_batches(gpu_ctx):
    c = _load("cfg1")
    paths, _ = _keys(c)
    want = gz.extract_path_lines(c, paths, ctx=gpu_ctx)
    # room for about two 22k-step paths at a time
    with gz.Server(c, hbm_budget=700_000, workers=2) as srv:
        tickets = [srv.submit_path(n) for n in paths for _ in range(2)]
        got = [srv.wait(t)[0] for t in tickets]
        assert got == [w for w in want for _ in range(2)]
        assert 1 <= srv.stats()["max_batch"] <= 2
    with gz.Server(c, hbm_budget=4096, workers=1) as srv:
        with pytest.raises(gz.GfazError, match="HBM budget"):
            srv.submit_path(paths[0])


def test_server_append_and_errors(gpu_ctx):
    c = _load("tiny")
    with gz.Server(c, workers=2) as srv:
        before = srv.submit_path("pathA")
        app = srv.submit_append("P\tpathC\t2+,4+,3-\t*\n")
        assert srv.wait(before)[0] == "P\tpathA\t1+,2+,3+\t2M,1M\n"
        assert srv.wait(app)[0] == ""
        assert srv.wait(srv.submit_path("pathC"))[0] == "P\tpathC\t2+,4+,3-\t*\n"
        assert srv.wait(srv.submit_path("pathA"))[0] == "P\tpathA\t1+,2+,3+\t2M,1M\n"
        walk_app = srv.submit_append("W\tsampleC\t0\tchr3\t*\t*\t>2>4>1\n")
        srv.wait(walk_app)
        key = gz.WalkLookupKey("sampleC", 0, "chr3", -1, -1)
        assert srv.wait(srv.submit_walk(key))[0] == "W\tsampleC\t0\tchr3\t*\t*\t>2>4>1\n"
        with pytest.raises(gz.GfazError, match="path not found: nope"):
            srv.submit_path("nope")
        with pytest.raises(gz.GfazError, match="walk not found"):
            srv.submit_walk(gz.WalkLookupKey("sampleB", 2, "chr2", -1, -1))
        bad = srv.submit_append("P\tpathA\t1+\t*\n")
        with pytest.raises(gz.GfazError, match="path name already exists or is duplicated: pathA"):
            srv.wait(bad)
        # the failed append changed nothing
        assert srv.wait(srv.submit_path("pathA"))[0] == "P\tpathA\t1+,2+,3+\t2M,1M\n"
    # the server's container is its own copy: the caller's is unchanged
    with pytest.raises(RuntimeError, match="path not found"):
        gz.extract_path_line(c, "pathC", ctx=gpu_ctx)
