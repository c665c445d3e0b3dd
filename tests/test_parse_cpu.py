"""Host GFA parser (the front end's CPU path and the reference the device
front end is compared with): traversals equal the reference parser's on the
golden inputs (raw streams generated with the reference), and the edge and
error cases follow the restated rules of src/io/gfa_parser.cpp."""
import os

import numpy as np
import pytest

import gfaz_gb300 as gz
from conftest import GOLDEN, golden_raw
from oracle import gfa_parse
from parse_cases import CASES, ERRORS, fuzz_text


def same_as_oracle(g, want):
    assert g.header_line == want["header"].decode()
    assert g.num_segments == want["segments"]
    assert [n.encode() for n in g.path_names] == [p[0] for p in want["paths"]]
    assert [o.encode() for o in g.path_overlaps] == [p[1] for p in want["paths"]]
    assert [list(map(int, p)) for p in g.paths] == [p[2] for p in want["paths"]]
    ws = want["walks"]
    assert [s.encode() for s in g.walk_sample_ids] == [w[0] for w in ws]
    assert list(g.walk_hap_indices) == [w[1] for w in ws]
    assert [s.encode() for s in g.walk_seq_ids] == [w[2] for w in ws]
    assert list(g.walk_seq_starts) == [w[3] for w in ws]
    assert list(g.walk_seq_ends) == [w[4] for w in ws]
    assert [list(map(int, w)) for w in g.walks] == [w[5] for w in ws]


@pytest.mark.parametrize("case", ["cfg1_mini", "named", "rich", "tiny"])
def test_host_parse_matches_reference_streams(case, manifest):
    g = gz.parse_gfa(os.path.join(GOLDEN, case + ".gfa"), device=False)
    raw, off, _ = golden_raw(case, manifest["cases"][case])
    trav = g.paths + g.walks
    assert np.array_equal(np.concatenate(trav) if trav else np.zeros(0, np.int32), raw)
    assert np.array_equal(np.cumsum([0] + [len(t) for t in trav]), np.asarray(off, np.int64))


@pytest.mark.parametrize("case", sorted(CASES))
def test_host_parse_edge_cases(case, tmp_path):
    p = tmp_path / "in.gfa"
    p.write_bytes(CASES[case])
    same_as_oracle(gz.parse_gfa(str(p), device=False), gfa_parse.parse(CASES[case]))


@pytest.mark.parametrize("case", sorted(ERRORS))
def test_host_parse_errors(case, tmp_path):
    text, msg = ERRORS[case]
    with pytest.raises(ValueError, match=msg):
        gfa_parse.parse(text)
    p = tmp_path / "in.gfa"
    p.write_bytes(text)
    with pytest.raises(gz.GfazError, match=msg):
        gz.parse_gfa(str(p), threads=1, device=False)


def test_host_parse_missing_file(tmp_path):
    with pytest.raises(gz.GfazError, match="GFA parser error: failed to open input file"):
        gz.parse_gfa(str(tmp_path / "nope.gfa"), device=False)


@pytest.mark.parametrize("seed", range(60))
def test_host_parse_fuzz(seed, tmp_path):
    """Random texts (tests/parse_cases.fuzz_text): the host parser on one
    thread gives the restatement's traversals, or its error."""
    text = fuzz_text(seed)
    p = tmp_path / "in.gfa"
    p.write_bytes(text)
    try:
        want, werr = gfa_parse.parse(text), None
    except ValueError as e:
        want, werr = None, str(e)
    if werr is not None:
        with pytest.raises(gz.GfazError, match=werr):
            gz.parse_gfa(str(p), threads=1, device=False)
    else:
        same_as_oracle(gz.parse_gfa(str(p), threads=1, device=False), want)


@pytest.mark.parametrize("order", ["field_first", "name_first"])
def test_host_parse_link_error_order(order, tmp_path):
    """L lines are read in parallel, but errors surface in line order as in
    the sequential parser: an optional-field type clash on an earlier line
    wins over a bad segment name on a later one, and the other way round."""
    segs = "".join("S\t%d\tA\n" % i for i in range(1, 4))
    clash = "L\t1\t+\t2\t-\t0M\tXX:i:5\nL\t2\t+\t3\t-\t0M\tXX:Z:a\n"
    bad = "L\tx\t+\t3\t-\t0M\n"
    text = segs + (clash + bad if order == "field_first" else bad + clash)
    p = tmp_path / "in.gfa"
    p.write_text(text)
    msg = "Type mismatch for link tag 'XX'" if order == "field_first" else "parse_uint32: no digits"
    with pytest.raises(gz.GfazError, match=msg):
        gz.parse_gfa(str(p), device=False)


def test_host_parse_links_kept_and_counted(tmp_path):
    """Links with an unresolved end are dropped (named segments); the rest
    keep their order."""
    text = "S\ta\tA\nS\tb\tC\nL\ta\t+\tb\t-\t3M\nL\ta\t+\tzz\t-\t*\nL\tb\t-\ta\t+\t*\tRC:i:2\n"
    p = tmp_path / "in.gfa"
    p.write_text(text)
    assert gz.parse_gfa(str(p), device=False).num_links == 2
