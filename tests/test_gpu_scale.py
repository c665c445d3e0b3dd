"""Config-4 scale (3.6B steps, 4,320 W-lines): compression under a 24 GB
HBM budget (chunked, the stream in host memory) gives the same grammar as
the resident compression, and both equal the oracle's (encoded stream,
offsets, rulebook, id seeds), and decoding gives the input back exactly, so
positions, offsets and tile indices hold past 2^31 steps (byte offsets past
2^33).  The W text of the first and last lines equals the oracle's
formatting."""
import os

import numpy as np
import pytest

import gfaz_gb300 as gz
from gfaz_gb300 import synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu


def _host_gb():
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 2**20
    except OSError:
        pass
    return 0.0


@pytest.mark.skipif(_host_gb() < 160, reason="needs ~140 GB of host memory")
def test_cfg4_chunked_roundtrip(gpu_ctx):
    steps, off, _, meta = synthetic.cfg4_stream()
    n = len(steps)
    assert n > (1 << 31) and len(off) == 4321
    ctx = gz.Context(0)
    ctx.set_option("hbm_budget", 24 << 30)
    g = gz.encode(steps, off, ctx=ctx)
    ref = gz.encode(steps, off, ctx=gpu_ctx)
    got = g.arrays()
    for x, y in zip(got, ref.arrays()):
        np.testing.assert_array_equal(x, y)
    del ref
    want = oracle.compress(steps, off, rounds=8, delta_round=1)
    info = g.info()
    assert (info["layer_start"], info["next_id"]) == (want["layer_start"], want["next_id"])
    np.testing.assert_array_equal(got[1], want["enc_offsets"])
    assert np.array_equal(got[0], want["encoded"]), "encoded stream differs from the oracle"
    assert np.array_equal(got[2], want["rules"]), "rulebook differs from the oracle"
    del got, want
    x, xoff = g.decode()
    np.testing.assert_array_equal(xoff, off)
    assert np.array_equal(x, steps)
    del x
    # W text of the first and last walks
    for t in (0, len(off) - 2):
        a, b = int(off[t]), int(off[t + 1])
        s, h, q, st, en = meta[t]
        got = g.text(t, t + 1, mode=gz.W_LINES, names=[s], hap_indices=[h], seq_ids=[q], seq_starts=[st],
                     seq_ends=[en])
        want = oracle.format_w(steps[a:b], np.array([0, b - a], np.uint64), [s], [h], [q], [st], [en])
        assert got == want
