"""The C++ facade (include/pmgb/pmgb.hpp) compiles against the C ABI and links with libpmgb.so;
on a GPU its demo program reproduces the Python path's P3M force."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

BIN = os.path.join(ROOT, "tests", "cpp", "_build", "facade_demo")


def build_demo():
    from particlesimulation_gb300 import _lib, build
    build.build()
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "facade_demo.cpp"), "-o", BIN,
           f"-L{libdir}", "-lpmgb", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return BIN


def test_facade_compiles_and_links():
    assert os.path.exists(build_demo())


@pytest.mark.gpu
def test_facade_demo_runs(gpu_lib):
    out = subprocess.run([build_demo()], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = dict(l.split(" ", 1) for l in out.stdout.strip().splitlines() if " " in l)
    acc0 = np.array([float(x) for x in lines["acc0"].split()])
    assert np.isfinite(acc0).all() and np.abs(acc0).max() > 0
    assert "invalid_argument" in out.stdout
    g = lines["grid"].split()
    assert g[:3] == ["32", "32", "32"] and float(g[3]) > 0
    assert np.isfinite([float(x) for x in lines["step"].split()]).all()
    assert float(lines["extforce"]) == 0.0 and float(lines["extpot"]) == 0.0  # no external field
    assert float(lines["fftroundtrip"]) < 1e-5
