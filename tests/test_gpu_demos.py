"""The reference's scenarios run end to end on the GPU through the facade: each writes the
reference's output files with one frame and one energy / momentum line per iteration
(simLength + 1), finite values, and the particle count of the scenario."""
import os
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {  # option: (particles, simLength)
    "cluster-sim-pm": (10000, 200),
    "cluster-sim-p3m": (10000, 200),
    "galaxy-sim-pm": (50000, 200),
    "galaxy-sim-p3m": (50000, 200),
    "galaxy-collision-sim-pm": (60000, 400),
}


@pytest.mark.parametrize("option", list(CASES))
def test_demo_runs_and_writes_reference_files(gpu_lib, option, tmp_path):
    from particlesimulation_gb300 import build
    exe = build.build_demos()
    r = subprocess.run([exe, option, str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    n, steps = CASES[option]
    names = sorted(os.listdir(tmp_path))
    assert names == sorted(["positions.dat", "field.dat", "energy.txt", "momentum.txt",
                            "expected_momentum.txt", "angular_momentum.txt"])
    with open(tmp_path / "positions.dat", "rb") as f:
        b = f.read()
    assert struct.unpack("<ii", b[:8]) == (n, steps + 1)
    frames = np.frombuffer(b[8:], np.float32).reshape(-1, n, 3)
    escaped = "outside the computational box" in r.stdout
    assert len(frames) == steps + 1 or escaped
    assert np.isfinite(frames).all()
    e = np.loadtxt(tmp_path / "energy.txt", ndmin=2)
    assert e.shape == (len(frames), 2) and np.isfinite(e).all()
    for name in ("momentum.txt", "expected_momentum.txt", "angular_momentum.txt"):
        assert np.loadtxt(tmp_path / name, ndmin=2).shape == (len(frames), 3)
