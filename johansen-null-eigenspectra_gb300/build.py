"""Builds libjne_gb300.so (the C-ABI engine) in-tree for sm_103a, and the
command-line driver jne_gb300 linked against it.

Every translation unit under csrc/ is compiled by nvcc in parallel, then linked
into one shared library next to this file.  Run as a script or call build().
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libjne_gb300.so")
CLI_SRC = os.path.join(HERE, "cli", "jne_cli.cpp")
CLI = os.path.join(HERE, "jne_gb300")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    cmd = [NVCC, *ARCH, *FLAGS, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    if verbose:
        sys.stderr.write(res.stderr)
    return obj


def _stale(srcs) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = srcs + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    deps.append(os.path.join(HERE, "..", "include", "jne.h"))
    deps.append(os.path.abspath(__file__))
    if not os.path.exists(CLI) or os.path.getmtime(CLI) < os.path.getmtime(CLI_SRC):
        return True
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force: bool = False, verbose: bool = False) -> str:
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    if not force and not _stale(srcs):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    res = subprocess.run([NVCC, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    cxx = os.environ.get("CXX", "g++")
    res = subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", CLI_SRC, "-o", CLI + ".tmp", "-L" + HERE, "-ljne_gb300",
                          "-Wl,-rpath,$ORIGIN"], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
