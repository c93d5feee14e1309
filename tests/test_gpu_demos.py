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


@pytest.mark.parametrize("option,nfiles", [("pm-accuracy-no-soft", 3 + 66), ("p3m-accuracy-shapes", 3 + 84)])
def test_accuracy_scenarios(gpu_lib, option, nfiles, tmp_path):
    """The reference's accuracy scenarios (pmAccuracy on (2 Ng, 2 Ng, Ng) meshes, Ng = 30..70,
    and p3mAccuracyShapes on 128 x 128 x 64 for a = 0.2 aMul H): the reference's file names,
    one frame of 10,000 particles each; the direct-sum forces equal the FP64 oracle's at the
    sampler's positions, and a PM / P3M force file (the accelerations a run records before its
    first drift, source/pmMethod.cpp:79-85) equals the FP64 oracle's forces at the sampler's
    positions, 1e-5 RMS-normalised."""
    import particlesimulation_gb300 as P
    from conftest import rel_rms
    from oracle import oracle as O
    from particlesimulation_gb300 import build
    exe = build.build_demos()
    r = subprocess.run([exe, option, str(tmp_path)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    names = os.listdir(tmp_path)
    assert len(names) == nfiles and "positions-pp.dat" in names and "positions-pm.dat" in names
    n = 10000
    state = P.DiskSamplerLinear(42).sample((30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, n)
    mass = np.full(n, 15.0 / n, np.float32)
    pp_name = "force-pp-0.dat" if option == "pm-accuracy-no-soft" else "force-pp.dat"
    with open(tmp_path / pp_name, "rb") as f:
        (h, a) = _frames(f.read())
    assert h == (n, 1)
    want = O.port_pp_accel(state[:n].astype(np.float64), mass.astype(np.float64), 4.5e-3)
    assert rel_rms(a[0], want) < 1e-6
    with open(tmp_path / "positions-pm.dat", "rb") as f:
        (h, x) = _frames(f.read())
    assert h == (n, 1)
    if option == "pm-accuracy-no-soft":
        fname, cfg, q = "force-pm-TSC-2-point-34.dat", O.PMConfig(
            grid=(68, 68, 34), box=(60.0, 60.0, 30.0), H=60.0 / 34, DT=1.0, G=4.5e-3,
            interpolation=2, finite_diff=0, greens=0, diameter=0.0), None
    else:
        H = 60.0 / 64
        a_ = float(np.float32(0.2) * np.float32(25) * np.float32(H))
        fname = "force-p3m-TSC-4-point-S2-25.dat"
        cfg = O.PMConfig(grid=(128, 128, 64), box=(60.0, 60.0, 30.0), H=H, DT=1.0, G=4.5e-3,
                         interpolation=2, finite_diff=1, greens=2, diameter=a_)
        q = O.P3MConfig(comp_box=(60.0, 60.0, 30.0), cutoff=a_, diameter=a_, softening=0.0,
                        cloud_shape=1, use_table=0, y_sorting=0)
    with open(tmp_path / fname, "rb") as f:
        (h, fa) = _frames(f.read())
    assert h == (n, 1) and np.isfinite(fa).all()
    xs = np.ascontiguousarray(state[:n], np.float32)
    if q is None:
        ref = O.port_pm_accel(cfg, xs, np.zeros_like(xs), mass, prec=1)
    else:
        ref = O.port_p3m_accel(cfg, q, xs, np.zeros_like(xs), mass, prec=1)
        ref = ref[0] if isinstance(ref, tuple) else ref
    ref = np.asarray(ref) * (cfg.H / cfg.DT ** 2)  # code -> original units
    # the table-free short-range formula (-G/r^2 + R(r)) / r cancels in FP32 near r = a; the
    # reference's own FP32 result carries the same cancellation, so the P3M bar is 1e-4
    assert rel_rms(fa[0], ref) < (1e-5 if q is None else 1e-4), fname
