"""S and L line text written on the device (full-file decompression): the
text equals the host formatting (src/io/gfa_writer.cpp:597-650,
gfa_write_utils.cpp:58-165) for segments of every length (empty, longer
than a tile), links with and without overlaps, and optional fields of each
type on some lines.  The golden full-file texts (reference output) are
checked in test_gpu_golden."""
import numpy as np
import pytest

import gfaz_gb300 as gz

pytestmark = pytest.mark.gpu


def _graph_text(seed, n_seg):
    rng = np.random.default_rng(seed)
    lens = rng.integers(1, 40, n_seg)
    lens[rng.integers(0, n_seg, 5)] = rng.integers(4000, 9000, 5)  # longer than a 4 KB tile
    lens[:3] = [5, 0, 16][:min(3, n_seg)]  # segment 2 (no optional fields) is empty
    out = ["H\tVN:Z:1.0\n"]
    for i in range(n_seg):
        seq = "".join(rng.choice(list("ACGT"), int(lens[i])))
        opt = ""
        if i % 7 == 0:
            opt += "\tLN:i:%d" % lens[i]
        if i % 11 == 0:
            opt += "\tDP:f:%.4f" % rng.random()
        if i % 13 == 0:
            opt += "\tID:Z:seg_%d" % i
        if i % 17 == 0:
            opt += "\tXA:A:G\tBB:B:i,5,-5,15"
        out.append("S\t%d\t%s%s\n" % (i + 1, seq, opt))
    for i in range(n_seg - 1):
        a, b = i + 1, int(rng.integers(1, n_seg + 1))
        ov = ["*", "0M", "%dM" % rng.integers(1, 99), "3M2I"][i % 4]
        opt = "\tRC:i:%d" % i if i % 5 == 0 else ""
        out.append("L\t%d\t%s\t%d\t%s\t%s%s\n" % (a, "+-"[i % 2], b, "-+"[i % 3 % 2], ov, opt))
    walk = rng.integers(1, n_seg + 1, 3000)
    out.append("P\tp1\t%s\t*\n" % ",".join("%d%s" % (v, "+-"[k % 2]) for k, v in enumerate(walk)))
    return "".join(out).encode()


@pytest.mark.parametrize("n_seg", [1, 5, 3000])
def test_device_static_text_equals_host(n_seg, tmp_path, gpu_ctx):
    p = tmp_path / "g.gfa"
    p.write_bytes(_graph_text(n_seg, n_seg))
    c = gz.compress_file(str(p), ctx=gpu_ctx)
    host = gz.Context(0)
    host.set_option("static_text", 0)
    dev = gz.gfa_text(c, ctx=gpu_ctx)
    assert dev == gz.gfa_text(c, ctx=host)
    # and the segments read back as written
    def segs(text):
        return [l.split(b"\t")[:3] for l in text.split(b"\n") if l.startswith(b"S")]
    assert segs(dev) == segs(p.read_bytes())
