"""Builds libgfaz_gb300.so in-tree: CUDA sources with nvcc for sm_103a only,
host C++ with g++ + OpenMP, linked into one shared library next to this
file.  No CMake; translation units compile in parallel and objects are
reused while their sources and headers are unchanged."""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgfaz_gb300.so")
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH
# -ffp-contract=off: no fused multiply-add in host floating-point code (the
# growth curve), so Arm and x86 hosts round alike.
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function", "-ffp-contract=off"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")) + glob.glob(os.path.join(CSRC, "host", "*.cpp")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
                     + glob.glob(os.path.join(CSRC, "host", "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h")))
    return cu, cpp, headers


def build(verbose: bool = False, force: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    cu, cpp, headers = _sources()
    newest_header = max((os.path.getmtime(h) for h in headers), default=0.0)
    jobs, objs = [], []
    for src in cu + cpp:
        rel = os.path.relpath(src, CSRC).replace(os.sep, "_")
        obj = os.path.join(OBJ, rel + ".o")
        objs.append(obj)
        stale = force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), newest_header)
        if not stale:
            continue
        if src.endswith(".cu"):
            cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-I", os.path.join(cuda, "include"), "-c", src, "-o", obj]
        jobs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in jobs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("libgfaz_gb300 build failed:\n" + msg)
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc, "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("libgfaz_gb300 link failed:\n" + " ".join(cmd) + "\n" + r.stdout.decode())
    build_cli()
    return LIB


CLI_SRC = os.path.join(CSRC, "cli", "gfaz_cli.cpp")
CLI = os.path.join(PKG, "gfaz")


def build_cli() -> str:
    """The `gfaz` command-line tool, a C++ client of the C ABI."""
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(CLI_SRC), os.path.getmtime(LIB)):
        return CLI
    cmd = ["g++", "-O2", "-std=c++17", CLI_SRC, "-o", CLI, "-L", PKG, "-lgfaz_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("gfaz CLI build failed:\n" + " ".join(cmd) + "\n" + r.stdout.decode())
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
