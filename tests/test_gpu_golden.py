"""GPU path against the reference's golden outputs: .gfaz bytes, pre-entropy
streams and decompressed GFA bytes, for files written by the reference CPU
compressor and for files written by this library."""
import hashlib
import os

import numpy as np
import pytest

import gfaz_gb300 as gz
import gfaz_format
from conftest import GOLDEN, golden_input_path, golden_raw

pytestmark = pytest.mark.gpu

CASES = ["tiny", "cfg1_mini", "cfg1_mini_d0", "cfg1_mini_d2_r3", "cfg1_mini_r1", "rich", "named", "cfg1"]


def _same_zstd(manifest):
    return gfaz_format.zstd().ZSTD_versionNumber() == manifest["zstd_version"]


def _assert_container_equal(mine: bytes, ref: bytes, same_zstd: bool):
    if same_zstd:
        assert hashlib.sha256(mine).hexdigest() == hashlib.sha256(ref).hexdigest()
        return
    # another libzstd on this machine: compare every field after decoding
    a, b = gfaz_format.read(mine), gfaz_format.read(ref)
    assert a.keys() == b.keys()
    for k in a:
        va, vb = a[k], b[k]
        if isinstance(va, tuple) and len(va) == 2 and isinstance(va[1], bytes):
            assert gfaz_format.unzstd(va) == gfaz_format.unzstd(vb), k
        elif k in ("segment_optional", "link_optional"):
            assert len(va) == len(vb)
            for ca, cb in zip(va, vb):
                assert ca[:3] == cb[:3]
                for x, y in zip(ca[3], cb[3]):
                    assert gfaz_format.unzstd(x) == gfaz_format.unzstd(y), k
        elif isinstance(va, np.ndarray):
            np.testing.assert_array_equal(va, vb, err_msg=k)
        else:
            assert va == vb, k


@pytest.mark.parametrize("case", CASES)
def test_compress_file_matches_reference_gfaz(case, manifest, tmp_path, gpu_ctx):
    meta = manifest["cases"][case]
    src = golden_input_path(case, meta, tmp_path)
    c = gz.compress_file(src, rounds=meta["rounds"], threshold=2, delta_round=meta["delta_round"], threads=4,
                         ctx=gpu_ctx)
    mine = c.to_bytes()
    ref = open(os.path.join(GOLDEN, case + ".gfaz"), "rb").read()
    _assert_container_equal(mine, ref, _same_zstd(manifest))
    # pre-entropy streams
    z = np.load(os.path.join(GOLDEN, case + ".npz"))
    pe = gfaz_format.pre_entropy(gfaz_format.read(mine))
    for k in ("rules_first", "rules_second", "paths", "walks", "sequence_lengths", "walk_lengths",
              "original_path_lengths", "original_walk_lengths", "layers", "delta_round"):
        np.testing.assert_array_equal(pe[k], z[k], err_msg=k)


@pytest.mark.parametrize("case", CASES)
def test_decompress_reference_file_bytes(case, manifest, gpu_ctx):
    """CPU-written .gfaz decoded on the GPU gives the reference decompressor's
    GFA bytes."""
    meta = manifest["cases"][case]
    c = gz.deserialize(os.path.join(GOLDEN, case + ".gfaz"))
    text = gz.gfa_text(c, ctx=gpu_ctx)
    assert hashlib.sha256(text).hexdigest() == meta["gfa_out_sha256"]


def test_write_gfa_file_and_roundtrip(manifest, tmp_path, gpu_ctx):
    meta = manifest["cases"]["rich"]
    c = gz.compress_file(os.path.join(GOLDEN, "rich.gfa"), threads=2, ctx=gpu_ctx)
    out = tmp_path / "out.gfa"
    gz.write_gfa_from_compressed_data(c, str(out), ctx=gpu_ctx)
    assert hashlib.sha256(out.read_bytes()).hexdigest() == meta["gfa_out_sha256"]
    p = tmp_path / "x.gfaz"
    gz.serialize(c, str(p))
    c2 = gz.deserialize(str(p))
    assert c2.to_bytes() == c.to_bytes()


def test_decompress_data_graph(manifest, gpu_ctx):
    case = "rich"
    meta = manifest["cases"][case]
    raw, off, z = golden_raw(case, meta)
    c = gz.deserialize(os.path.join(GOLDEN, case + ".gfaz"))
    g = gz.decompress_data(c, ctx=gpu_ctx)
    npaths = int(z["n_paths"][0])
    assert len(g.paths) == npaths
    allt = g.paths + g.walks
    for t, tr in enumerate(allt):
        np.testing.assert_array_equal(tr, raw[int(off[t]):int(off[t + 1])])
    assert g.header_line.startswith("H\t")
    assert g.num_jumps == 2 and g.num_containments == 2


def test_extract_known_answers(gpu_ctx):
    """Known-answer strings of the reference CLI tests
    (tests/regression/test_cli_commands.py:114-117, 135)."""
    c = gz.deserialize(os.path.join(GOLDEN, "tiny.gfaz"))
    lines = gz.extract_path_lines(c, ["pathB", "pathA"], ctx=gpu_ctx)
    assert "".join(lines) == "P\tpathB\t1+,3-,4+\t*\nP\tpathA\t1+,2+,3+\t2M,1M\n"
    assert gz.extract_path_line(c, "pathA", ctx=gpu_ctx) == "P\tpathA\t1+,2+,3+\t2M,1M\n"
    w = gz.extract_walk_line(c, "sampleB", 1, "chr2", -1, -1, ctx=gpu_ctx)
    assert w == "W\tsampleB\t1\tchr2\t*\t*\t>1<3>4\n"
    assert gz.extract_walk_line_by_name(c, "sampleA", ctx=gpu_ctx) == "W\tsampleA\t0\tchr1\t0\t7\t>1>2>3\n"
    with pytest.raises(RuntimeError, match="Extraction workflow error: path not found: nope"):
        gz.extract_path_lines(c, ["nope"], ctx=gpu_ctx)
    with pytest.raises(RuntimeError, match="walk not found"):
        gz.extract_walk_line(c, "sampleB", 2, "chr2", -1, -1, ctx=gpu_ctx)


def test_add_haplotypes_known_answers(tmp_path, gpu_ctx):
    """Known answers of the reference CLI tests
    (tests/regression/test_cli_commands.py:157-160, 194, 201-222)."""
    c = gz.deserialize(os.path.join(GOLDEN, "tiny.gfaz"))
    ap = tmp_path / "append_paths.gfa"
    ap.write_text("H\tVN:Z:1.0\nP\tpathC\t2+,4+,3-\t*\n")
    c2 = gz.add_haplotypes(c, str(ap), ctx=gpu_ctx)
    assert gz.extract_path_line(c2, "pathC", ctx=gpu_ctx) == "P\tpathC\t2+,4+,3-\t*\n"
    # the input container is unchanged (copy semantics)
    with pytest.raises(RuntimeError, match="path not found"):
        gz.extract_path_line(c, "pathC", ctx=gpu_ctx)
    aw = tmp_path / "append_walks.gfa"
    aw.write_text("W\tsampleC\t0\tchr3\t*\t*\t>2>4>1\n")
    c3 = gz.add_haplotypes(c, str(aw), ctx=gpu_ctx)
    assert gz.extract_walk_line(c3, "sampleC", 0, "chr3", -1, -1, ctx=gpu_ctx) == \
        "W\tsampleC\t0\tchr3\t*\t*\t>2>4>1\n"
    am = tmp_path / "append_mixed.gfa"
    am.write_text("P\tpathD\t1+,2+\t*\nW\tsampleD\t0\tchr4\t*\t*\t>1>2\n")
    with pytest.raises(RuntimeError, match="mixes P-lines and W-lines"):
        gz.add_haplotypes(c, str(am), ctx=gpu_ctx)
    dup = tmp_path / "dup.gfa"
    dup.write_text("P\tpathA\t1+\t*\n")
    with pytest.raises(RuntimeError, match="path name already exists or is duplicated: pathA"):
        gz.add_haplotypes(c, str(dup), ctx=gpu_ctx)
