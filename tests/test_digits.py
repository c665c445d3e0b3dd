"""The SWAR decimal conversion used by the text kernels, checked on the
host against plain division for every value below 10^8, and their digit
count against comparisons with the powers of ten for every 32-bit value."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gfaz_gb300", "csrc")


def test_digits8_exhaustive(tmp_path):
    exe = tmp_path / "digits_check"
    cc = subprocess.run(["g++", "-O3", "-std=c++17", "-I", CSRC, os.path.join(HERE, "native", "digits_check.cpp"),
                         "-o", str(exe)], capture_output=True, text=True)
    if cc.returncode != 0:
        pytest.fail(cc.stderr)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok 100000000")
