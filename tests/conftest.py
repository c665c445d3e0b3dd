import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(TESTS, "golden")
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from gfaz_gb300.build import build
    build()
    from oracle import oracle
    oracle.build()


@pytest.fixture(scope="session")
def manifest():
    with open(os.path.join(GOLDEN, "MANIFEST.json")) as fh:
        return json.load(fh)


def golden_raw(case: str, meta: dict):
    """Raw traversals (paths then walks) and offsets of a golden case."""
    z = np.load(os.path.join(GOLDEN, case + ".npz"))
    if "raw_steps" in z:
        raw = z["raw_steps"]
    elif meta.get("input_from"):
        raw = np.load(os.path.join(GOLDEN, meta["input_from"] + ".npz"))["raw_steps"]
    else:
        from gfaz_gb300 import synthetic
        raw, _ = synthetic.cfg1(seed=1).flat()
    return raw, z["raw_offsets"], z


def golden_input_path(case: str, meta: dict, tmp_path):
    """Path of the GFA input of a golden case (regenerated when not stored)."""
    name = meta.get("input_from", case)
    p = os.path.join(GOLDEN, name + ".gfa")
    if os.path.exists(p):
        return p
    from gfaz_gb300 import synthetic
    out = os.path.join(str(tmp_path), name + ".gfa")
    with open(out, "wb") as fh:
        fh.write(synthetic.cfg1(seed=1).to_gfa())
    return out


@pytest.fixture(scope="session")
def gpu_ctx():
    import gfaz_gb300 as gz
    if not gz.has_gpu_backend():
        pytest.skip("no CUDA device")
    return gz.Context(0)
