"""The `gfaz` binary as a drop-in for the reference CLI.

compress / decompress on the golden inputs give the reference CLI's .gfaz
bytes and decompressed GFA bytes; the reference GPU flags
(compress_command.cpp:32-45, decompress_command.cpp:34-48) are accepted
and change no byte (their refusals are checked in test_cli_cpu.py);
extract-path,
extract-walk and add-haplotypes print the known answers of the reference's
CLI tests (tests/regression/test_cli_commands.py:114-222).  Integer and
byte output: the tolerance is zero."""
import hashlib
import os
import subprocess

import pytest

import gfaz_gb300 as gz
import gfaz_format
from conftest import GOLDEN, golden_input_path
from test_gpu_golden import _assert_container_equal, _same_zstd

pytestmark = pytest.mark.gpu

CASES = ["tiny", "cfg1_mini", "cfg1_mini_d0", "cfg1_mini_d2_r3", "rich", "named", "cfg1"]


def cli(*args):
    from gfaz_gb300.build import CLI
    return subprocess.run([CLI] + [str(a) for a in args], capture_output=True, text=True)


def sha(path) -> str:
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def ok(r):
    assert r.returncode == 0, r.stdout + r.stderr
    return r


@pytest.mark.parametrize("case", CASES)
def test_cli_compress_decompress_golden(case, manifest, tmp_path, gpu_ctx):
    meta = manifest["cases"][case]
    src = golden_input_path(case, meta, tmp_path)
    out = tmp_path / "out.gfaz"
    ok(cli("compress", "-r", meta["rounds"], "-d", meta["delta_round"], src, out))
    ref = open(os.path.join(GOLDEN, case + ".gfaz"), "rb").read()
    _assert_container_equal(out.read_bytes(), ref, _same_zstd(manifest))
    dec = tmp_path / "out.gfa"
    ok(cli("decompress", out, dec))
    assert sha(dec) == meta["gfa_out_sha256"]
    # a file written by the reference compressor, decoded by this binary
    dec2 = tmp_path / "ref.gfa"
    ok(cli("decompress", "--gpu", os.path.join(GOLDEN, case + ".gfaz"), dec2))
    assert sha(dec2) == meta["gfa_out_sha256"]


def test_cli_default_output_names(manifest, tmp_path, gpu_ctx):
    src = tmp_path / "tiny.gfa"
    src.write_bytes(open(os.path.join(GOLDEN, "tiny.gfa"), "rb").read())
    ok(cli("compress", src))
    assert (tmp_path / "tiny.gfa.gfaz").exists()
    os.remove(src)
    ok(cli("decompress", tmp_path / "tiny.gfa.gfaz"))
    assert sha(src) == manifest["cases"]["tiny"]["gfa_out_sha256"]


@pytest.mark.parametrize("flags", [["--gpu", "--gpu-rolling-input-chunk-mb", "1"],
                                   ["--gpu", "--gpu-chunk-mb", "1", "--debug"],
                                   ["--gpu", "--gpu-legacy"],
                                   ["-g", "--gpu-legacy", "--gpu-chunk-mb", "1"]])
def test_cli_compress_gpu_flags_same_bytes(flags, manifest, tmp_path, gpu_ctx):
    """A 1 MiB rolling input chunk (262,144 steps) streams the 352k-step
    config-1 stream through HBM in two chunks: the same container bytes."""
    meta = manifest["cases"]["cfg1"]
    src = golden_input_path("cfg1", meta, tmp_path)
    out = tmp_path / "out.gfaz"
    r = ok(cli("compress", *flags, src, out))
    ref = open(os.path.join(GOLDEN, "cfg1.gfaz"), "rb").read()
    _assert_container_equal(out.read_bytes(), ref, _same_zstd(manifest))
    if "--debug" in flags:
        assert "Debug: on" in r.stdout
        assert r.stderr.strip()  # phase timers
    if "--gpu-legacy" in flags and "--gpu-chunk-mb" in flags:
        assert "ignored with --gpu-legacy" in r.stderr


@pytest.mark.parametrize("case", ["cfg1", "rich"])
@pytest.mark.parametrize("flags", [["--gpu", "--gpu-rolling-output-chunk-mb", "1"],
                                   ["--gpu", "--gpu-max-expanded-chunk-mb", "1", "--debug"],
                                   ["--gpu", "--gpu-legacy"], ["--legacy"], ["-s", "-j", "3"]])
def test_cli_decompress_gpu_flags_same_bytes(case, flags, manifest, tmp_path, gpu_ctx):
    meta = manifest["cases"][case]
    dec = tmp_path / "out.gfa"
    ok(cli("decompress", *flags, os.path.join(GOLDEN, case + ".gfaz"), dec))
    assert sha(dec) == meta["gfa_out_sha256"]


def test_decode_chunk_groups(manifest, gpu_ctx):
    """The writer's traversal groups (decode_chunk, in expanded steps): one
    step per group, groups smaller than one traversal, and a group holding
    everything give the reference's bytes."""
    for case in ("cfg1", "rich", "tiny"):
        c = gz.deserialize(os.path.join(GOLDEN, case + ".gfaz"))
        for chunk in (1, 5000, 30_000, 1 << 40):
            ctx = gz.Context(0)
            ctx.set_option("decode_chunk", chunk)
            text = gz.gfa_text(c, ctx=ctx)
            assert hashlib.sha256(text).hexdigest() == manifest["cases"][case]["gfa_out_sha256"], (case, chunk)
            del ctx


def test_cli_extract_and_append_known_answers(tmp_path, gpu_ctx):
    """tests/regression/test_cli_commands.py:114-222, run through this
    binary on the same fixture contents."""
    gfaz = tmp_path / "fixture.gfaz"
    ok(cli("compress", os.path.join(GOLDEN, "tiny.gfa"), gfaz))
    r = ok(cli("extract-path", gfaz, "pathB", "pathA"))
    assert r.stdout == "P\tpathB\t1+,3-,4+\t*\nP\tpathA\t1+,2+,3+\t2M,1M\n"
    r = ok(cli("extract-walk", gfaz, "sampleB", "1", "chr2", "*", "*"))
    assert r.stdout == "W\tsampleB\t1\tchr2\t*\t*\t>1<3>4\n"
    r = cli("extract-path", gfaz, "nope")
    assert r.returncode == 1 and "Error: Extraction workflow error: path not found: nope" in r.stderr

    ap = tmp_path / "append_paths.gfa"
    ap.write_text("H\tVN:Z:1.0\nP\tpathC\t2+,4+,3-\t*\n")
    upd = tmp_path / "paths_updated.gfaz"
    ok(cli("add-haplotypes", gfaz, ap, upd))
    r = ok(cli("extract-path", upd, "pathA", "pathC"))
    assert r.stdout == "P\tpathA\t1+,2+,3+\t2M,1M\nP\tpathC\t2+,4+,3-\t*\n"

    aw = tmp_path / "append_walks.gfa"
    aw.write_text("W\tsampleC\t0\tchr3\t*\t*\t>2>4>1\n")
    upd2 = tmp_path / "walks_updated.gfaz"
    ok(cli("add-haplotypes", gfaz, aw, upd2))
    r = ok(cli("extract-walk", upd2, "sampleC", "0", "chr3", "*", "*"))
    assert r.stdout == "W\tsampleC\t0\tchr3\t*\t*\t>2>4>1\n"

    am = tmp_path / "append_mixed.gfa"
    am.write_text("P\tpathD\t1+,2+\t*\nW\tsampleD\t0\tchr4\t*\t*\t>1>2\n")
    upd3 = tmp_path / "mixed_updated.gfaz"
    r = cli("add-haplotypes", gfaz, am, upd3)
    assert r.returncode != 0 and not upd3.exists()

    # default output name of add-haplotypes: <input without .gfaz>.updated.gfaz
    ok(cli("add-haplotypes", gfaz, ap))
    assert (tmp_path / "fixture.updated.gfaz").exists()
    # the reference container format throughout
    assert gfaz_format.read(str(upd))["num_links"] == 4
