"""The GPU transform against the C oracle on seeded inputs: encoded streams,
rulebooks and id seeds must be identical; decoding must invert encoding;
P/W text must equal the oracle's formatter.  Edge cases follow what the
reference handles: empty and single-step traversals, runs of one candidate
pair spanning many tiles (the greedy parity carried across tiles),
palindromic pairs (b == -a), every delta_round, rounds 0/1/8."""
import numpy as np
import pytest

import gfaz_gb300 as gz
from gfaz_gb300 import synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu


def offsets_of(lengths):
    off = np.zeros(len(lengths) + 1, np.uint64)
    np.cumsum(np.asarray(lengths, np.uint64), out=off[1:])
    return off


def check_encode(steps, off, ctx, rounds=8, delta_round=1):
    steps = np.ascontiguousarray(steps, np.int32)
    off = np.ascontiguousarray(off, np.uint64)
    g = gz.encode(steps, off, rounds=rounds, delta_round=delta_round, ctx=ctx)
    ref = oracle.compress(steps, off, rounds=rounds, delta_round=delta_round)
    enc, eoff, rules = g.arrays()
    info = g.info()
    assert info["layer_start"] == ref["layer_start"]
    assert info["next_id"] == ref["next_id"]
    np.testing.assert_array_equal(eoff, ref["enc_offsets"])
    np.testing.assert_array_equal(enc, ref["encoded"])
    np.testing.assert_array_equal(rules, ref["rules"])
    # stored rule columns: delta-coded halves of the keys
    f, s = g.rule_columns()
    if len(rules):
        np.testing.assert_array_equal(np.cumsum(f.astype(np.int64)).astype(np.int64).astype(np.uint32).view(np.int32),
                                      (rules >> 32).astype(np.int32))
        np.testing.assert_array_equal(np.cumsum(s.astype(np.int64)).astype(np.int64).astype(np.uint32).view(np.int32),
                                      (rules & 0xFFFFFFFF).astype(np.uint32).view(np.int32))
    x, xoff = g.decode()
    np.testing.assert_array_equal(xoff, off)
    np.testing.assert_array_equal(x, steps)
    return g, ref


def test_random_small_alphabet(gpu_ctx):
    rng = np.random.default_rng(7)
    for trial in range(6):
        lens = rng.integers(0, 400, size=40)
        steps = rng.integers(-6, 7, size=int(lens.sum())).astype(np.int32)
        steps[steps == 0] = 1
        check_encode(steps, offsets_of(lens), gpu_ctx, rounds=8, delta_round=trial % 3)


def test_long_run_spans_many_tiles(gpu_ctx):
    # one traversal of a repeated id: deltas are 0, one candidate run of
    # ~100k positions crossing ~50 apply tiles
    steps = np.full(100_003, 5, np.int32)
    check_encode(steps, offsets_of([len(steps)]), gpu_ctx)
    # alternating runs of odd and even length across tile edges
    parts, lens = [], []
    for L in (2047, 2048, 2049, 4095, 6001, 1, 2, 3):
        parts.append(np.full(L, 9, np.int32))
        lens.append(L)
    check_encode(np.concatenate(parts), offsets_of(lens), gpu_ctx, delta_round=1)
    check_encode(np.concatenate(parts), offsets_of(lens), gpu_ctx, delta_round=0)


def test_palindromes_and_negative_ids(gpu_ctx):
    a = np.array([3, -3] * 500 + [7, -7, 7] * 300, np.int32)
    check_encode(a, offsets_of([1000, 900]), gpu_ctx, delta_round=0)
    rng = np.random.default_rng(11)
    b = rng.choice(np.array([-2**30 + 5, -17, -1, 1, 17, 2**30 - 5], np.int32), size=20000)
    check_encode(b, offsets_of([5000, 0, 1, 14999]), gpu_ctx, delta_round=0)


def test_empty_and_tiny_traversals(gpu_ctx):
    check_encode(np.zeros(0, np.int32), np.zeros(1, np.uint64), gpu_ctx)
    check_encode(np.zeros(0, np.int32), np.zeros(4, np.uint64), gpu_ctx)
    check_encode(np.array([4], np.int32), offsets_of([0, 1, 0]), gpu_ctx)
    check_encode(np.array([1, 2, 1, 2], np.int32), offsets_of([1, 1, 1, 1]), gpu_ctx)
    check_encode(np.array([1, 2, 1, 2, 1, 2], np.int32), offsets_of([2, 0, 2, 2]), gpu_ctx)


@pytest.mark.parametrize("rounds", [0, 1, 8])
@pytest.mark.parametrize("delta_round", [0, 1, 2, 3])
def test_cfg1_shape_all_params(rounds, delta_round, gpu_ctx):
    g = synthetic.cfg1(seed=17, n_backbone=4000, n_paths=7)
    steps, off = g.flat()
    check_encode(steps, off, gpu_ctx, rounds=rounds, delta_round=delta_round)


def test_many_short_identical_traversals(gpu_ctx):
    # identical content in every traversal; pairs never cross boundaries
    one = np.array([1, 2, 3, 4, 5, 6, 7, 8], np.int32)
    steps = np.tile(one, 3000)
    check_encode(steps, offsets_of([8] * 3000), gpu_ctx)
    check_encode(steps, offsets_of([3, 5] * 3000), gpu_ctx)


def test_cfg2_and_cfg3_shapes_scaled(gpu_ctx):
    steps, off, _ = synthetic.cfg2_stream(seed=5, n_segments=200_000, n_paths=8)
    check_encode(steps, off, gpu_ctx)
    steps, off, _, _ = synthetic.cfg3_stream(seed=6, n_backbone=60_000, n_walks=40, median=3000, hi=200_000)
    check_encode(steps, off, gpu_ctx)


def test_text_matches_oracle(gpu_ctx):
    g = synthetic.cfg1(seed=23, n_backbone=1500, n_paths=5)
    steps, off = g.flat()
    # include empty traversals between and after non-empty ones
    lens = list(np.diff(off.astype(np.int64)))
    lens = [0] + lens[:2] + [0, 0] + lens[2:] + [0]
    off2 = offsets_of(lens)
    gram = gz.encode(steps, off2, ctx=gpu_ctx)
    n = len(lens)
    names = [f"path{i}" for i in range(n)]
    ovs = ["*" if i % 2 else "" for i in range(n)]
    ovs[3] = "5M,2M"
    assert gram.text(0, n, names=names, overlaps=ovs) == oracle.format_p(steps, off2, names, ovs)
    samples = [f"s{i}" for i in range(n)]
    haps = list(range(n))
    seqids = [f"chr{i}" for i in range(n)]
    starts = [-1 if i % 3 == 0 else 10 * i for i in range(n)]
    ends = [-1 if i % 3 == 0 else 10 * i + 5 for i in range(n)]
    got = gram.text(0, n, mode=gz.W_LINES, names=samples, hap_indices=haps, seq_ids=seqids, seq_starts=starts,
                    seq_ends=ends)
    assert got == oracle.format_w(steps, off2, samples, haps, seqids, starts, ends)
    # a sub-range of traversals
    sub = gram.text(2, 6, names=names[2:6], overlaps=ovs[2:6])
    assert sub == oracle.format_p(steps[int(off2[2]):int(off2[6])], off2[2:7] - off2[2], names[2:6], ovs[2:6])


def test_text_large_ids_and_long_names(gpu_ctx):
    rng = np.random.default_rng(3)
    steps = rng.integers(1, 2**31 - 1, size=30000).astype(np.int32) * rng.choice([-1, 1], size=30000).astype(np.int32)
    off = offsets_of([10000, 20000])
    gram = gz.encode(steps, off, delta_round=0, ctx=gpu_ctx)
    names = ["x" * 40000, "y"]   # a prefix longer than one tile's staging buffer
    assert gram.text(0, 2, names=names, overlaps=["", ""]) == oracle.format_p(steps, off, names, ["", ""])


def test_load_grammar_decodes_oracle_output(gpu_ctx):
    steps, off, _ = synthetic.cfg2_stream(seed=9, n_segments=100_000, n_paths=5)
    ref = oracle.compress(steps, off, rounds=8, delta_round=1)
    f = np.zeros(len(ref["rules"]), np.int32)
    s = np.zeros(len(ref["rules"]), np.int32)
    oracle.lib().orc_rule_columns(ref["rules"].ctypes.data, len(ref["rules"]), f.ctypes.data, s.ctypes.data)
    g = gz.load_grammar(ref["encoded"], ref["enc_offsets"], f, s, ref["layer_start"], 1, ctx=gpu_ctx)
    x, xoff = g.decode()
    np.testing.assert_array_equal(x, steps)
    np.testing.assert_array_equal(xoff, off)


def test_count_kernels_give_same_result(gpu_ctx):
    """Every pair-count kernel (the tuner's pick, tiled, tiled with warp
    folding, flat, flat with four pairs), classification and emit from the
    count's slot references or by table probes (persistent and flat), the
    warp folding switch and the table size (load-factor tuner on and off, a
    forced first-round size too small for the pairs, so that the count
    refills and rewrites its slot references) give the same grammar."""
    steps, off, _ = synthetic.cfg2_stream(seed=4, n_segments=80_000, n_paths=6)
    a = gz.encode(steps, off, ctx=gpu_ctx).arrays()
    probe = ("slot_refs", 0)
    for opts in [[("count_kernel", 0)], [("count_kernel", 1)], [("count_kernel", 2)], [("count_kernel", 3)],
                 [("warp_dedup", 1)], [probe], [probe, ("classify_kernel", 0)], [probe, ("classify_kernel", 1)],
                 [probe, ("count_kernel", 3)], [("table_tuner", 0)], [("first_table_cap", 1 << 16)],
                 [probe, ("first_table_cap", 1 << 16)]]:
        ctx2 = gz.Context(0)
        for opt, val in opts:
            ctx2.set_option(opt, val)
        b = gz.encode(steps, off, ctx=ctx2).arrays()
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


def test_cfg3_walk_text(gpu_ctx):
    # config-3 shape: uneven walks (lognormal lengths, sigma 2) as W lines
    steps, off, _, meta = synthetic.cfg3_stream(seed=3, n_backbone=200_000, n_walks=300, median=5e3, sigma=2.0,
                                                hi=1_000_000, max_total=4_000_000)
    for dr in (1, 0):
        g, _ = check_encode(steps, off, gpu_ctx, delta_round=dr)
        n = len(off) - 1
        samples, haps, seqids, starts, ends = (list(x) for x in zip(*meta))
        got = g.text(0, n, mode=gz.W_LINES, names=samples, hap_indices=haps, seq_ids=seqids, seq_starts=starts,
                     seq_ends=ends)
        assert got == oracle.format_w(steps, off, samples, haps, seqids, starts, ends)


@pytest.mark.parametrize("delta_round", [0, 1])
def test_text_incompressible_and_long_pieces(delta_round, gpu_ctx):
    # random steps barely compress: output tiles cover more symbols than the
    # shared-memory stage holds; ids span every digit count and both signs
    rng = np.random.default_rng(31 + delta_round)
    lens = [0, 1, 5000, 0, 12_000, 3, 9000]
    steps = rng.integers(-2_000_000_000, 2_000_000_000, size=sum(lens)).astype(np.int32)
    steps[rng.integers(0, len(steps), 200)] = rng.integers(-9, 10, 200)
    off = offsets_of(lens)
    g, _ = check_encode(steps, off, gpu_ctx, delta_round=delta_round)
    n = len(lens)
    names = [f"p{i}" for i in range(n)]
    ovs = ["*"] * n
    assert g.text(0, n, names=names, overlaps=ovs) == oracle.format_p(steps, off, names, ovs)
    # a name longer than a tile's text staging: that tile writes straight to HBM
    names[2] = "n" * 40_000
    assert g.text(0, n, names=names, overlaps=ovs) == oracle.format_p(steps, off, names, ovs)


def test_tuner_decisions_file(tmp_path, monkeypatch, gpu_ctx):
    """GFAZ_TUNE_FILE: a context appends the decisions it takes and a later
    context starts from them (same grammar either way)."""
    f = tmp_path / "tune.txt"
    monkeypatch.setenv("GFAZ_TUNE_FILE", str(f))
    steps, off, _ = synthetic.cfg2_stream(seed=9, n_segments=40_000, n_paths=4)
    a = gz.encode(steps, off, ctx=gz.Context(0)).arrays()
    rows = [tuple(int(x) for x in line.split()) for line in f.read_text().splitlines()]
    assert rows and all(len(r) == 3 and r[0] in (0, 1, 2) for r in rows)
    assert any(r[0] == 2 for r in rows)  # table shrink factors from the load-factor tuner
    # force the other classification variant and tables four times smaller
    # (some then refill) for every recorded class
    f.write_text("".join("%d %d %d\n" % (k, c, (1 - v) if k == 1 else v + 2 if k == 2 else v) for k, c, v in rows))
    b = gz.encode(steps, off, ctx=gz.Context(0)).arrays()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert f.read_text().count("\n") == len(rows)  # nothing new to decide


def test_tuners_on_a_prefix(monkeypatch):
    """The tuners time their candidates on the stream's first steps
    (GFAZ_TUNE_STEPS); with a prefix far shorter than every round's stream
    the grammar is unchanged (the timed runs must not read past the prefix
    or leave their table or status behind)."""
    steps, off, _ = synthetic.cfg2_stream(seed=6, n_segments=120_000, n_paths=5)
    want = gz.encode(steps, off, ctx=gz.Context(0)).arrays()
    monkeypatch.setenv("GFAZ_TUNE_STEPS", "5000")
    for opt in (None, ("count_kernel", 0), ("classify_kernel", 0)):
        ctx = gz.Context(0)
        if opt:
            ctx.set_option(*opt)
        got = gz.encode(steps, off, ctx=ctx).arrays()
        for x, y in zip(got, want):
            np.testing.assert_array_equal(x, y)



@pytest.mark.parametrize("host_text", [0, 1])
def test_text_into_page_locked_memory(host_text):
    """P text decoded into page-locked host memory, written there by the text
    kernel on the context's low-priority stream (host_text 0) or staged in
    HBM and moved by a copy engine (1), equals the oracle's text; the steps
    decode back exactly."""
    torch = pytest.importorskip("torch")
    steps, off, _ = synthetic.cfg2_stream(seed=8, n_segments=60_000, n_paths=7)
    ctx = gz.Context(0)
    ctx.set_option("host_text", host_text)
    g = gz.encode(steps, off, ctx=ctx)
    n = len(off) - 1
    names = [f"hap{i}" for i in range(n)]
    ovs = ["*"] * n
    want = oracle.format_p(steps, off, names, ovs)
    buf = torch.zeros(len(want) + 64, dtype=torch.uint8).pin_memory()
    size = g.decode_text(0, n, names=names, overlaps=ovs, out_ptr=buf.data_ptr(), cap=buf.numel(),
                         where=gz.WHERE_HOST)
    assert size == len(want)
    assert bytes(buf[:size].numpy().tobytes()) == want
    x, xoff = g.decode()
    np.testing.assert_array_equal(x, steps)
