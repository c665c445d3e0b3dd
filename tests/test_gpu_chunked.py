"""Compression of host-resident streams in HBM-sized chunks (the config-4
mode): the grammar, the encoded streams and the serialized container are
identical to the resident compression, for chunk sizes that put chunk edges
inside traversals, between them and inside candidate runs, for every delta
round setting, and when the chunking follows from an HBM budget."""
import os

import numpy as np
import pytest

import gfaz_gb300 as gz
from conftest import GOLDEN
from gfaz_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _same(a, b):
    for x, y in zip(a.arrays(), b.arrays()):
        np.testing.assert_array_equal(x, y)
    assert a.info() == b.info()


@pytest.mark.parametrize("delta_round", [0, 1, 2])
@pytest.mark.parametrize("chunk", [2048, 3 * 2048, 37 * 2048])
def test_chunked_equals_resident(delta_round, chunk, gpu_ctx):
    steps, off, _ = synthetic.cfg2_stream(seed=7, n_segments=60_000, n_paths=5)
    want = gz.encode(steps, off, rounds=8, delta_round=delta_round, ctx=gpu_ctx)
    ctx = gz.Context(0)
    ctx.set_option("encode_chunk", chunk)
    got = gz.encode(steps, off, rounds=8, delta_round=delta_round, ctx=ctx)
    _same(got, want)
    x, xoff = got.decode()
    np.testing.assert_array_equal(x, steps)


def test_chunked_edge_cases(gpu_ctx):
    # empty and one-step traversals, traversals ending exactly on chunk
    # edges, one long run of a single pair across many chunks
    rng = np.random.default_rng(3)
    parts = [np.array([], np.int32), np.array([5], np.int32), np.full(2048, 9, np.int32),
             np.tile(np.array([4, 7], np.int32), 5000), rng.integers(1, 50, 4095).astype(np.int32),
             np.array([], np.int32), np.arange(1, 6000, dtype=np.int32)]
    steps = np.concatenate(parts)
    off = np.zeros(len(parts) + 1, np.uint64)
    off[1:] = np.cumsum([len(p) for p in parts])
    for rounds in (1, 8):
        want = gz.encode(steps, off, rounds=rounds, ctx=gpu_ctx)
        ctx = gz.Context(0)
        ctx.set_option("encode_chunk", 2048)
        _same(gz.encode(steps, off, rounds=rounds, ctx=ctx), want)


def test_budget_selects_chunks(gpu_ctx):
    steps, off, _ = synthetic.cfg2_stream(seed=8, n_segments=400_000, n_paths=6)
    n = len(steps)
    want = gz.encode(steps, off, ctx=gpu_ctx)
    ctx = gz.Context(0)
    # room for the per-tile words, the pair table and a few chunks, not for
    # the resident stream buffers
    ctx.set_option("hbm_budget", int(n * 1.1) + (64 << 20) + 16 * min(n, 1 << 24) + (8 << 20))
    got = gz.encode(steps, off, ctx=ctx)
    _same(got, want)
    ctx.set_option("hbm_budget", 1 << 20)
    with pytest.raises(gz.GfazError, match="HBM budget too small"):
        gz.encode(steps, off, ctx=ctx)


@pytest.mark.parametrize("seed,delta_round", [(8, 1), (9, 1), (8, 0), (9, 2)])
def test_budget_input_resident(seed, delta_round, gpu_ctx):
    """A budget with room for the round's input beside the per-tile arrays
    and the table, but not for resident compression: the delta pass (or
    the max |x| pass) leaves round 1's input on the device when it can,
    round 1 reads it in place (output chunks to host memory), later rounds
    run resident; the grammar is the resident one."""
    steps, off, _ = synthetic.cfg2_stream(seed=seed, n_segments=400_000, n_paths=6)
    n = len(steps)
    assert n < (1 << 24)
    want = gz.encode(steps, off, delta_round=delta_round, ctx=gpu_ctx)
    ctx = gz.Context(0)
    # fixed part (per-tile words and arrays) ~1 B/step + the first round's
    # table + 64 MB; the input adds 4 B/step; resident rounds need ~12.7
    # B/step + 64 MB and more
    ctx.set_option("hbm_budget", 8 * n + (74 << 20))
    _same(gz.encode(steps, off, delta_round=delta_round, ctx=ctx), want)


@pytest.mark.parametrize("delta_round", [0, 1])
def test_budget_input_resident_no_repeats(delta_round, gpu_ctx):
    """Round 1 reads its input in place and finds no repeated pair (every
    traversal is [t+1, 2t+3], so no pair repeats raw or delta-coded): the
    grammar has no rules and the stream is round 1's input, taken from the
    device."""
    T = 2_000_000
    t = np.arange(T, dtype=np.int64)
    steps = np.empty(2 * T, dtype=np.int32)
    steps[0::2] = t + 1
    steps[1::2] = 2 * t + 3
    off = np.arange(0, 2 * T + 1, 2, dtype=np.uint64)
    n = len(steps)
    want = gz.encode(steps, off, delta_round=delta_round, ctx=gpu_ctx)
    ctx = gz.Context(0)
    ctx.set_option("hbm_budget", 8 * n + (74 << 20))
    got = gz.encode(steps, off, delta_round=delta_round, ctx=ctx)
    _same(got, want)
    assert got.info()["num_rules"] == 0
    x, _ = got.decode()
    np.testing.assert_array_equal(x, steps)


def test_chunked_container_bytes(tmp_path, gpu_ctx):
    src = os.path.join(GOLDEN, "cfg1_mini.gfa")
    a = gz.compress_file(src, ctx=gpu_ctx)
    ctx = gz.Context(0)
    ctx.set_option("encode_chunk", 2048)
    b = gz.compress_file(src, ctx=ctx)
    pa, pb = tmp_path / "a.gfaz", tmp_path / "b.gfaz"
    gz.serialize(a, str(pa))
    gz.serialize(b, str(pb))
    assert pa.read_bytes() == pb.read_bytes()
