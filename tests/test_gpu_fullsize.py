"""Bit-exact parity at full benchmark size.

The round trip decode(encode(x)) == x holds for any lossless grammar, so it
cannot catch a rule id, sign or orientation that differs from the CPU
compressor's only at scale (table refills, the tuner's kernel variants, runs
crossing many tiles, offsets past 2^31).  These tests compare the GPU path
with the oracle (the C restatement of compression_workflow.cpp:548-700 and
path_encoder.cpp:13-84, pinned to the reference CLI's golden outputs) on
the full benchmark workloads:

* the chromosome-scale P-line workload the bench times (90 P-lines, 513M
  steps, rounds 8, delta_round 1): encoded stream, encoded offsets,
  rulebook, layer_start / next_id, stored rule columns, and the P-line text
  of every traversal (compared in pieces of a few traversals, so no 4.5 GB
  string is built twice);
* the uneven-walk workload (2,000 W-lines, 775M steps): the same, with W
  text.

The whole-genome workload (3.6B steps) is compared in test_gpu_scale.py.
Integer work: the tolerance is zero."""
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


def assert_grammar_equal(g, ref):
    """Every array the container stores before the entropy stage."""
    info = g.info()
    assert info["layer_start"] == ref["layer_start"]
    assert info["next_id"] == ref["next_id"]
    enc, eoff, rules = g.arrays()
    np.testing.assert_array_equal(eoff, ref["enc_offsets"])
    assert np.array_equal(enc, ref["encoded"]), "encoded stream differs from the oracle"
    assert np.array_equal(rules, ref["rules"]), "rulebook differs from the oracle"
    f, s = g.rule_columns()
    wf = np.zeros(len(ref["rules"]), np.int32)
    ws = np.zeros(len(ref["rules"]), np.int32)
    if len(wf):
        oracle.lib().orc_rule_columns(ref["rules"].ctypes.data, len(ref["rules"]), wf.ctypes.data, ws.ctypes.data)
    np.testing.assert_array_equal(f, wf)
    np.testing.assert_array_equal(s, ws)


def pieces(off, target_steps):
    """Consecutive traversal ranges of about target_steps steps each."""
    n = len(off) - 1
    t = 0
    while t < n:
        u = t + 1
        while u < n and int(off[u + 1] - off[t]) <= target_steps:
            u += 1
        yield t, u
        t = u


@pytest.mark.skipif(_host_gb() < 40, reason="needs ~30 GB of host memory")
def test_cfg2_full_bit_exact(gpu_ctx):
    steps, off, _ = synthetic.cfg2_stream(seed=2)
    assert len(off) - 1 == 90 and len(steps) > 500_000_000
    g = gz.encode(steps, off, rounds=8, delta_round=1, ctx=gpu_ctx)
    ref = oracle.compress(steps, off, rounds=8, delta_round=1)
    assert ref["rounds_done"] == 8
    assert_grammar_equal(g, ref)
    del ref
    names = [f"hap{i}" for i in range(len(off) - 1)]
    for a, b in pieces(off, 40_000_000):
        got = g.text(a, b, names=names[a:b], overlaps=["*"] * (b - a))
        sl = steps[int(off[a]):int(off[b])]
        want = oracle.format_p(sl, off[a:b + 1] - off[a], names[a:b], ["*"] * (b - a))
        assert got == want, f"P text of traversals {a}..{b} differs from the oracle"


@pytest.mark.skipif(_host_gb() < 60, reason="needs ~45 GB of host memory")
def test_cfg3_full_bit_exact(gpu_ctx):
    steps, off, _, meta = synthetic.cfg3_stream()
    assert len(off) - 1 == 2000 and len(steps) > 700_000_000
    g = gz.encode(steps, off, rounds=8, delta_round=1, ctx=gpu_ctx)
    ref = oracle.compress(steps, off, rounds=8, delta_round=1)
    assert_grammar_equal(g, ref)
    del ref
    samples, haps, seqids, starts, ends = (list(x) for x in zip(*meta))
    for a, b in pieces(off, 60_000_000):
        got = g.text(a, b, mode=gz.W_LINES, names=samples[a:b], hap_indices=haps[a:b], seq_ids=seqids[a:b],
                     seq_starts=starts[a:b], seq_ends=ends[a:b])
        sl = steps[int(off[a]):int(off[b])]
        want = oracle.format_w(sl, off[a:b + 1] - off[a], samples[a:b], haps[a:b], seqids[a:b], starts[a:b],
                               ends[a:b])
        assert got == want, f"W text of traversals {a}..{b} differs from the oracle"
