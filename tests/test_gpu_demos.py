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


# The PM field sweeps: (option, our file names, fixture case in tests/golden/field_sweeps.npz,
# the reference's positions.dat / field.dat of the same run, written by its own CPU code)
SWEEPS = [("anisotropy", ("positions.dat", "field.dat"), "aniso"),
          ("pm-optimal", ("positions-s2.dat", "field-s2.dat"), "optimal_s2"),
          ("assignment-schemes", ("positions-ngp.dat", "field-ngp.dat"), "ngp")]
SWEEP_FILES = {
    "anisotropy": ["positions.dat", "field.dat", "positions_offset.dat", "field_offset.dat",
                   "positions_diag.dat", "field_diag.dat"],
    "pm-optimal": ["positions-s1.dat", "field-s1.dat", "positions-s2.dat", "field-s2.dat"],
    "assignment-schemes": ["positions-tsc.dat", "field-tsc.dat", "positions-cic.dat",
                           "field-cic.dat", "positions-ngp.dat", "field-ngp.dat"],
}


def _frames(b):
    n, frames = struct.unpack("<ii", b[:8])
    return (n, frames), np.frombuffer(b[8:], np.float32).reshape(-1, n, 3)


@pytest.mark.parametrize("option,files,case", SWEEPS)
def test_field_sweep_matches_reference(gpu_lib, option, files, case, tmp_path):
    """A PM field sweep of the reference's demos (one massive particle, 399 massless tracers,
    one iteration, field recorded): exactly the reference's files, and positions and fields
    equal to the reference's own run within float rounding of the different FFTs."""
    from particlesimulation_gb300 import build
    exe = build.build_demos()
    r = subprocess.run([exe, option, str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert sorted(os.listdir(tmp_path)) == sorted(SWEEP_FILES[option])
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "field_sweeps.npz"))
    for name, kind in zip(files, ("positions", "field")):
        with open(tmp_path / name, "rb") as f:
            (h1, a) = _frames(f.read())
        (h2, b) = _frames(gold[f"{case}/{kind}"].tobytes())
        assert h1 == h2 == (400, 2), name
        if kind == "positions":
            assert np.abs(a - b).max() < 2e-6 * np.abs(b).max(), name
        else:
            for k in range(len(a)):
                rel = np.sqrt(((a[k] - b[k]) ** 2).sum() / (b[k] ** 2).sum())
                assert rel < 3e-5, (name, k, rel)
