"""Builds ``libpmgb.so`` (the CUDA kernels + C ABI of include/pmgb.h) in-tree for sm_103a.

Each ``csrc/*.cu`` is compiled by nvcc in parallel, then linked into
``particlesimulation_gb300/libpmgb.so``.  Rebuilds only when a source or header is newer than
the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpmgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++20", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I", os.path.join(ROOT, "include"),
]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps() -> list[str]:
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(
        os.path.join(ROOT, "include", "*.h"))


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc, *NVCC_FLAGS, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


DEMOS_SRC = os.path.join(PKG, "demos", "pmgb_demos.cpp")
DEMOS_BIN = os.path.join(PKG, "pmgb_demos")


def build_demos(force: bool = False) -> str:
    """The scenario command line (demos/pmgb_demos.cpp, the reference's demos on the facade),
    linked against libpmgb.so with an rpath to this directory."""
    lib = build()
    deps = [DEMOS_SRC, lib, os.path.join(ROOT, "include", "pmgb", "pmgb.hpp")]
    if not force and os.path.exists(DEMOS_BIN) and all(
            os.path.getmtime(d) <= os.path.getmtime(DEMOS_BIN) for d in deps):
        return DEMOS_BIN
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           DEMOS_SRC, "-o", DEMOS_BIN + ".tmp", f"-L{PKG}", "-lpmgb", f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"demos build failed:\n{r.stderr}")
    os.replace(DEMOS_BIN + ".tmp", DEMOS_BIN)
    return DEMOS_BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_demos())
