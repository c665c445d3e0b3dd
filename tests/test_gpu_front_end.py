"""Device GFA front end (line index, P/W field bounds and step tokens on the
GPU): the parsed graph equals the restated reference rules on the edge
cases, raises the same errors, equals the host parser on the golden inputs
and on larger numeric and named graphs (tokens across tile edges, the name
table), and file compression gives the same container through either
front end."""
import os

import numpy as np
import pytest

import gfaz_gb300 as gz
from conftest import GOLDEN
from oracle import gfa_parse
from parse_cases import CASES, ERRORS, fuzz_text, random_text
from test_parse_cpu import same_as_oracle

pytestmark = pytest.mark.gpu


def same_graph(a, b):
    assert a.header_line == b.header_line
    assert a.num_segments == b.num_segments and a.num_links == b.num_links
    assert a.num_jumps == b.num_jumps and a.num_containments == b.num_containments
    assert a.segment_names == b.segment_names and a.segment_sequences == b.segment_sequences
    assert a.path_names == b.path_names and a.path_overlaps == b.path_overlaps
    assert len(a.paths) == len(b.paths) and all(np.array_equal(x, y) for x, y in zip(a.paths, b.paths))
    assert a.walk_sample_ids == b.walk_sample_ids and a.walk_hap_indices == b.walk_hap_indices
    assert a.walk_seq_ids == b.walk_seq_ids
    assert a.walk_seq_starts == b.walk_seq_starts and a.walk_seq_ends == b.walk_seq_ends
    assert len(a.walks) == len(b.walks) and all(np.array_equal(x, y) for x, y in zip(a.walks, b.walks))


@pytest.mark.parametrize("case", sorted(CASES))
def test_device_parse_edge_cases(case, tmp_path, gpu_ctx):
    p = tmp_path / "in.gfa"
    p.write_bytes(CASES[case])
    g = gz.parse_gfa(str(p), ctx=gpu_ctx)
    same_as_oracle(g, gfa_parse.parse(CASES[case]))
    same_graph(g, gz.parse_gfa(str(p), device=False))


@pytest.mark.parametrize("case", sorted(ERRORS))
def test_device_parse_errors(case, tmp_path, gpu_ctx):
    text, msg = ERRORS[case]
    p = tmp_path / "in.gfa"
    p.write_bytes(text)
    with pytest.raises(gz.GfazError, match=msg):
        gz.parse_gfa(str(p), ctx=gpu_ctx)
    # the context stays usable after a parse error
    q = tmp_path / "ok.gfa"
    q.write_bytes(CASES["only_walks"])
    same_as_oracle(gz.parse_gfa(str(q), ctx=gpu_ctx), gfa_parse.parse(CASES["only_walks"]))


@pytest.mark.parametrize("case", ["cfg1_mini", "named", "rich", "tiny"])
def test_device_parse_golden(case, gpu_ctx):
    src = os.path.join(GOLDEN, case + ".gfa")
    same_graph(gz.parse_gfa(src, ctx=gpu_ctx), gz.parse_gfa(src, device=False))


@pytest.mark.parametrize("named", [False, True])
def test_device_parse_large(named, tmp_path, gpu_ctx):
    p = tmp_path / "big.gfa"
    p.write_bytes(random_text(seed=21 + named, n_segments=120_000, n_paths=5, n_walks=4, named=named))
    same_graph(gz.parse_gfa(str(p), ctx=gpu_ctx), gz.parse_gfa(str(p), device=False))


@pytest.mark.parametrize("case", ["cfg1_mini", "rich", "named"])
def test_compress_file_front_ends_agree(case, tmp_path, gpu_ctx):
    src = os.path.join(GOLDEN, case + ".gfa")
    host = gz.Context(0)
    host.set_option("front_end", 0)
    a, b = gz.compress_file(src, ctx=gpu_ctx), gz.compress_file(src, ctx=host)
    pa, pb = tmp_path / "a.gfaz", tmp_path / "b.gfaz"
    gz.serialize(a, str(pa))
    gz.serialize(b, str(pb))
    assert pa.read_bytes() == pb.read_bytes()


@pytest.mark.parametrize("seed", range(60))
def test_device_parse_fuzz(seed, tmp_path, gpu_ctx):
    """Random texts: the same graph, or the same error, as the host parser
    on one thread (whose first error is deterministic)."""
    p = tmp_path / "in.gfa"
    p.write_bytes(fuzz_text(seed))

    def run(**kw):
        try:
            return gz.parse_gfa(str(p), **kw), None
        except gz.GfazError as e:
            return None, str(e)
    want, werr = run(threads=1, device=False)
    got, gerr = run(ctx=gpu_ctx)
    assert gerr == werr
    if want is not None:
        same_graph(got, want)
