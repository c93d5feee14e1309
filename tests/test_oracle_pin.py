"""Pins the CPU oracle (oracle/port.cpp) before its results are trusted in the parity tests.

Two pins: (1) against the golden fixtures generated from the reference's own CPU code
(tests/golden/make_golden.py) - always runs; (2) directly against the reference compiled from
its sources (oracle/_ref) - runs where the reference sources exist.
"""
import numpy as np
import pytest

from conftest import load_npz, rel_rms
from oracle import oracle as O


def cfg_from(d):
    ext = tuple(float(x) for x in d["ext"]) if not np.isnan(d["ext"]).any() else ()
    return O.PMConfig(grid=tuple(int(g) for g in d["grid"]), box=tuple(float(b) for b in d["box"]),
                      H=float(d["HDTG"][0]), DT=float(d["HDTG"][1]), G=float(d["HDTG"][2]),
                      interpolation=int(d["scheme"][0]), finite_diff=int(d["scheme"][1]),
                      greens=int(d["scheme"][2]), diameter=float(d["diameter"]), ext=ext)


def p3m_from(d):
    return O.P3MConfig(comp_box=tuple(float(b) for b in d["comp_box"]), cutoff=float(d["cds"][0]),
                       diameter=float(d["cds"][1]), softening=float(d["cds"][2]),
                       cloud_shape=int(d["flags"][0]), use_table=int(d["flags"][1]),
                       y_sorting=int(d["flags"][2]))


PM = load_npz("pm_forces.npz")
P3M = load_npz("p3m_forces.npz")


@pytest.mark.parametrize("case", [c for c in PM if c != "inputs"])
def test_port_pm_matches_golden(case):
    d = PM[case]
    inp = d if "pos" in d else PM["inputs"]
    cfg = cfg_from(d)
    f32 = O.port_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"], prec=0)
    f64 = O.port_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"], prec=1)
    # the float port repeats the reference's FP32 operations (different FFT algorithm)
    assert rel_rms(f32, d["acc"]) < 2e-6
    # FP64 vs the reference's FP32: the reference's own float error (S2 shape factor
    # cancellation in FP32 dominates for S2_OPTIMAL)
    assert rel_rms(f64, d["acc"]) < 2e-5


EXACT = load_npz("p3m_exact.npz")


@pytest.mark.parametrize("case", [c for c in EXACT if c != "inputs"])
def test_port_table_free_p3m_matches_golden(case):
    """The reference's table-free short-range force without softening (shortRangeForce): the
    float port repeats it to 1e-6; the reference's own FP32 result is ~4e-5 from FP64 (its
    -G/r^2 + R(r) cancels near r = a)."""
    d = EXACT[case]
    inp = EXACT["inputs"]
    cfg, q = cfg_from(d), p3m_from(d)
    f32 = O.port_p3m_accel(cfg, q, inp["pos"], inp["vel"], inp["mass"], prec=0)
    f64 = O.port_p3m_accel(cfg, q, inp["pos"], inp["vel"], inp["mass"], prec=1)
    assert rel_rms(f32, d["acc"]) < 1e-6
    assert rel_rms(f64, d["acc"]) < 6e-5


PMACC = load_npz("pm_accuracy.npz")


@pytest.mark.parametrize("case", [c for c in PMACC if c != "inputs"])
def test_port_pm_non_power_of_two_meshes_match_golden(case):
    """Meshes of the reference's pmAccuracy scenario (2 Ng, 2 Ng, Ng) for Ng = 30, 34, 58: the
    port's mixed-length FFT against the reference (kissfft) on the same inputs."""
    d = PMACC[case]
    inp = PMACC["inputs"]
    cfg = cfg_from(d)
    f32 = O.port_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"], prec=0)
    f64 = O.port_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"], prec=1)
    assert rel_rms(f32, d["acc"]) < 1e-5
    assert rel_rms(f64, d["acc"]) < 1e-5


@pytest.mark.parametrize("case", [c for c in PM if c != "inputs" and "density" in PM[c]])
def test_port_pm_meshes_match_golden(case):
    d = PM[case]
    inp = PM["inputs"]
    cfg = cfg_from(d)
    _, dens, pot, grn = O.port_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"], prec=0,
                                        want_mesh=True)
    assert np.abs(dens - d["density"]).max() <= 1e-6 * np.abs(d["density"]).max()
    assert np.abs(grn - d["green"]).max() <= 1e-6 * np.abs(d["green"]).max() + 1e-12
    assert np.sqrt(((pot - d["potential"]) ** 2).mean()) <= 1e-5 * np.sqrt((d["potential"] ** 2).mean())


@pytest.mark.parametrize("case", [c for c in P3M if c != "inputs"])
def test_port_p3m_matches_golden(case):
    d = P3M[case]
    inp = P3M["inputs"]
    acc = O.port_p3m_accel(cfg_from(d), p3m_from(d), inp["pos"], inp["vel"], inp["mass"], prec=0)
    assert rel_rms(acc, d["acc"]) < 2e-6


@pytest.mark.parametrize("ys", [1, 0])
def test_port_cell_lists_match_golden(ys):
    d = load_npz("cell_lists.npz")
    q = O.P3MConfig(comp_box=tuple(d["q"]["comp_box"]), cutoff=float(d["q"]["cds"][0]),
                    diameter=float(d["q"]["cds"][1]))
    order, counts, dims = O.port_chaining_mesh(q, float(d["H"]), d["pos_code"], ys)
    assert dims == tuple(d[f"y{ys}"]["dims"])
    np.testing.assert_array_equal(counts, d[f"y{ys}"]["counts"])
    np.testing.assert_array_equal(order, d[f"y{ys}"]["order"])


@pytest.mark.parametrize("case", ["pm", "p3m", "escape"])
def test_port_runs_match_golden(case):
    d = load_npz("runs.npz")[case]
    q = p3m_from(d) if "flags" in d else None
    x, v, esc = O.port_run(cfg_from(d), q, d["pos"], d["vel"], d["mass"], int(d["sim_length"]),
                           prec=0)
    assert esc == bool(d["escaped"])
    scale = np.abs(d["pos_out"]).max()
    assert np.abs(x - d["pos_out"]).max() < 2e-6 * scale
    assert rel_rms(v, d["vel_out"]) < 1e-5


def test_port_sr_table_matches_golden():
    d = load_npz("misc.npz")
    H = 30.0 / 16
    for cs in (0, 1):
        for eps in (0.0, 0.5):
            q = O.P3MConfig(comp_box=(30.0,) * 3, cutoff=3 * H, diameter=3 * H, softening=eps,
                            cloud_shape=cs)
            t, _ = O.port_sr_table(q, H)
            np.testing.assert_allclose(t, d[f"cs{cs}_eps{eps}"], rtol=2e-6, atol=0)


def test_port_direct_sum_matches_reference_pp():
    d = load_npz("misc.npz")
    acc = O.port_pp_accel(d["pp_pos"], d["pp_mass"], 1.0)
    assert rel_rms(acc, d["pp_acc"]) < 1e-5


# ---------------------------------------------------------------- live reference ---
ref = pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here")


@ref
@pytest.mark.parametrize("is_,fds,gf", [(2, 0, 2), (1, 1, 1), (0, 0, 3)])
def test_port_vs_live_reference_pm(is_, fds, gf):
    rng = np.random.default_rng(7)
    n = 700
    p = rng.uniform(4, 26, (n, 3)).astype(np.float32)
    v = rng.normal(0, 0.01, (n, 3)).astype(np.float32)
    m = np.full(n, 1.0 / n, np.float32)
    H = 30.0 / 16
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0,) * 3, H=H, DT=0.05, G=1.0, interpolation=is_,
                     finite_diff=fds, greens=gf, diameter=3 * H)
    assert rel_rms(O.port_pm_accel(cfg, p, v, m, prec=0), O.ref_pm_accel(cfg, p, v, m)) < 2e-6


@ref
def test_port_vs_live_reference_p3m_and_cells():
    rng = np.random.default_rng(8)
    n = 1500
    p = np.clip(rng.normal(15, 3, (n, 3)), 4, 26).astype(np.float32)
    v = np.zeros((n, 3), np.float32)
    m = np.full(n, 1.0 / n, np.float32)
    H = 30.0 / 16
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0,) * 3, H=H, DT=0.05, G=1.0, interpolation=2,
                     finite_diff=0, greens=2, diameter=3 * H)
    q = O.P3MConfig(comp_box=(30.0,) * 3, cutoff=3 * H, diameter=3 * H, cloud_shape=1)
    assert rel_rms(O.port_p3m_accel(cfg, q, p, v, m, prec=0), O.ref_p3m_accel(cfg, q, p, v, m)) < 2e-6
    pc = (p / np.float32(H)).astype(np.float32)
    for ys in (1, 0):
        a = O.port_chaining_mesh(q, H, pc, ys)
        b = O.ref_chaining_mesh(q, H, pc, ys)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


# ---------------------------------------------------------------- run diagnostics ---
def _check_diag_vs_reference(rec, ref):
    """Energies: the reference prints them with std::to_string (6 decimals) after summing in
    float; vectors: printed with %.6e, summed in float over the particles."""
    assert rec.shape == ref.shape
    assert np.abs(rec[:, :2] - ref[:, :2]).max() < 1.5e-6
    for sl in (slice(2, 5), slice(5, 8), slice(8, 11)):
        scale = np.abs(ref[:, sl]).max()
        assert np.abs(rec[:, sl] - ref[:, sl]).max() < 1e-5 * scale


@pytest.mark.parametrize("case", ["pm_ext", "p3m", "escape"])
@pytest.mark.parametrize("prec", [0, 1])
def test_port_diagnostics_match_golden(case, prec):
    d = load_npz("diagnostics.npz")[case]
    q = p3m_from(d) if "flags" in d else None
    _, _, esc, rec = O.port_run(cfg_from(d), q, d["pos"], d["vel"], d["mass"],
                                int(d["sim_length"]), prec=prec, diagnostics=True)
    assert esc == bool(d["escaped"])
    _check_diag_vs_reference(rec, d["diag"])


@ref
def test_port_diagnostics_vs_live_reference():
    from particlesimulation_gb300 import workloads as W
    w = W.plummer_cluster(n=3000, seed=9, grid=32)
    cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=2,
                     finite_diff=1, greens=1, diameter=3 * w.H, ext=(15.0, 14.0, 16.0, 4.0, 0.3, 1.0))
    _, _, esc, ref_rec = O.ref_run(cfg, None, w.pos, w.vel, w.mass, 4, diagnostics=True)
    _, _, esc2, rec = O.port_run(cfg, None, w.pos, w.vel, w.mass, 4, prec=0, diagnostics=True)
    assert esc == esc2 and not esc
    _check_diag_vs_reference(rec, ref_rec)
