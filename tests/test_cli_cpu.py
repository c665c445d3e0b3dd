"""The `gfaz` binary's option handling, without a GPU: the reference CLI's
GPU flags are refused in the same combinations and with the same messages
(compress_command.cpp:32-45, 108-112; decompress_command.cpp:34-48,
92-105), before any device work."""
import subprocess

import pytest


def cli(*args):
    from gfaz_gb300.build import CLI
    return subprocess.run([CLI] + [str(a) for a in args], capture_output=True, text=True)


@pytest.mark.parametrize("args,msg", [
    (["compress", "--gpu-legacy", "x.gfa"], "--gpu-rolling-input-chunk-mb and --gpu-legacy require --gpu"),
    (["compress", "--gpu-chunk-mb", "4", "x.gfa"], "--gpu-rolling-input-chunk-mb and --gpu-legacy require --gpu"),
    (["compress", "--gpu", "--gpu-chunk-mb", "0", "x.gfa"], "Invalid value for --gpu-rolling-input-chunk-mb: 0"),
    (["compress", "--gpu", "--gpu-rolling-input-chunk-mb", "4k", "x.gfa"],
     "Invalid value for --gpu-rolling-input-chunk-mb: 4k"),
    (["decompress", "--gpu-rolling-output-chunk-mb", "5", "x.gfaz"],
     "--gpu-rolling-output-chunk-mb and --gpu-legacy require --gpu"),
    (["decompress", "--gpu-legacy", "x.gfaz"], "--gpu-rolling-output-chunk-mb and --gpu-legacy require --gpu"),
    (["decompress", "--gpu", "-l", "x.gfaz"], "--legacy is the CPU legacy mode"),
    (["compress"], "No input file specified"),
])
def test_cli_flag_errors(args, msg):
    r = cli(*args)
    assert r.returncode == 1
    assert msg in r.stderr
