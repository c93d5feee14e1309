"""Run diagnostics on the GPU (pmgb_pm_set_diagnostics / get_diagnostics) against the
reference's recorded diagnostics (golden fixtures from its StateRecorder files) and the oracle
port's FP64 restatement of SimInfo run on the same float trajectory.

Tolerances: against the port, 1e-6 relative for the energies and 1e-6 of sum(m |u|) (times
the box size for angular momentum) for the momentum vectors (the float trajectories of the GPU and the port agree to
rounding level over these few steps; all sums are FP64 on both sides).  With an optimal
influence function the port runs in double: the reference's float Green's function holds
rounding noise at the 7 modes where the finite-difference operator vanishes, which the force
never sees but the potential energy does (about 7e-6 of it here); the GPU and the FP64 port
set those modes to zero.  Against the reference,
the bounds of its printed precision and float sums (energies 1.5e-6 absolute, vectors 1e-5 of
the largest component), as for the port in test_oracle_pin.py.
"""
import numpy as np
import pytest

from conftest import load_npz
from oracle import oracle as O
from test_gpu_p3m import make_p3m
from test_gpu_pm import make_pm
from test_oracle_pin import _check_diag_vs_reference, cfg_from, p3m_from

pytestmark = pytest.mark.gpu

DIAG = load_npz("diagnostics.npz")


def _compare(rec, ref, mass, length, rtol=1e-6):
    """Energies relative to their own size; momenta relative to sum(m |u|) ~ sqrt(2 KE M) (the
    momentum itself is a cancelling sum), angular momenta to that times the box size."""
    assert rec.shape == ref.shape, (rec.shape, ref.shape)
    for c in (0, 1, 11):
        scale = max(np.abs(ref[:, c]).max(), 1e-30)
        assert np.abs(rec[:, c] - ref[:, c]).max() <= rtol * scale, c
    p_scale = np.sqrt(2.0 * np.abs(ref[:, 1]).max() * float(np.sum(mass)))
    for sl, scale in ((slice(2, 5), p_scale), (slice(5, 8), p_scale * length),
                      (slice(8, 11), p_scale)):
        assert np.abs(rec[:, sl] - ref[:, sl]).max() <= rtol * scale, sl


def _port_prec(cfg):
    return 1 if cfg.greens in (1, 2) else 0


def _gpu_run(d, collect=True):
    cfg = cfg_from(d)
    if "flags" in d:
        pm, p3m = make_p3m(cfg, p3m_from(d), d["pos"], d["vel"], d["mass"])
        esc, steps = p3m.run(int(d["sim_length"]), collectDiagnostics=collect)
    else:
        pm = make_pm(cfg, d["pos"], d["vel"], d["mass"])
        esc, steps = pm.run(int(d["sim_length"]), collectDiagnostics=collect)
    return pm, esc, steps


@pytest.mark.parametrize("case", ["pm_ext", "p3m", "escape"])
def test_diagnostics_match_reference_and_port(gpu_lib, case):
    d = DIAG[case]
    pm, esc, steps = _gpu_run(d)
    out = pm.diagnostics()
    rec = out["records"]
    assert esc == bool(d["escaped"])
    assert out["taken"] == len(d["diag"])
    _check_diag_vs_reference(rec, d["diag"])
    q = p3m_from(d) if "flags" in d else None
    cfg = cfg_from(d)
    _, _, esc2, port = O.port_run(cfg, q, d["pos"], d["vel"], d["mass"], int(d["sim_length"]),
                                  prec=_port_prec(cfg), diagnostics=True)
    assert esc2 == esc
    _compare(rec, port, d["mass"], float(np.max(d["box"])))
    pm.close()


def test_diagnostics_at_benchmark_scale(gpu_lib):
    """The disk workload at 32,768 particles (TSC, S2, 3-cell cutoff) for 4 steps against the
    port; the external field of the reference's galaxy demos added (source/demos.cpp)."""
    from particlesimulation_gb300 import workloads as W
    w = W.disk_p3m(n=32768)
    cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=w.interpolation,
                     finite_diff=w.finite_diff, greens=w.greens, diameter=w.diameter,
                     ext=(30.0, 30.0, 30.0, 1.0, 0.2, 1.0))
    q = O.P3MConfig(comp_box=w.p3m["comp_box"], cutoff=w.p3m["cutoff"], diameter=w.p3m["diameter"],
                    cloud_shape=w.p3m["cloud_shape"])
    pm, p3m = make_p3m(cfg, q, w.pos, w.vel, w.mass)
    esc, _ = p3m.run(4, collectDiagnostics=True)
    rec = pm.diagnostics()["records"]
    _, _, esc2, port = O.port_run(cfg, q, w.pos, w.vel, w.mass, 4, prec=_port_prec(cfg),
                                  diagnostics=True)
    assert not esc and not esc2
    _compare(rec, port, w.mass, max(w.box), rtol=3e-6)
    assert np.abs(rec[:, 11]).max() > 0  # the external potential is in the record
    pm.close()


def test_run_then_advance_equals_longer_run(gpu_lib):
    """run(2) + advance(3) performs the same operations as run(5): identical records, bit for bit
    (fixed reduction order); the records are also identical run to run."""
    d = DIAG["pm_ext"]
    cfg = cfg_from(d)
    a = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    a.setDiagnostics(16)
    a.run(2)
    a.advance(3)
    ra = a.diagnostics()
    b = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    b.run(5, collectDiagnostics=True)
    rb = b.diagnostics()
    assert ra["taken"] == rb["taken"] == 6
    np.testing.assert_array_equal(ra["records"], rb["records"])
    c = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    c.run(5, collectDiagnostics=True)
    np.testing.assert_array_equal(c.diagnostics()["records"], rb["records"])
    for h in (a, b, c):
        h.close()


def test_diagnostics_enabled_after_run(gpu_lib):
    """Diagnostics turned on between run and advance: the first record needs the density of the
    last force evaluation, which is recomputed; the records then track a run that had them on
    from the start (which also rounds the masses every iteration, so to 1e-6)."""
    d = DIAG["pm_ext"]
    cfg = cfg_from(d)
    a = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    a.run(2)
    a.setDiagnostics(8)
    a.advance(3)
    ra = a.diagnostics()["records"]
    b = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    b.setDiagnostics(16)
    b.run(2)
    b.advance(3)
    rb = b.diagnostics()["records"][3:]
    assert len(ra) == 3
    ra = ra.copy()
    ra[:, 8:11] = rb[:, 8:11]  # the expected momentum starts at a different point
    _compare(ra, rb, d["mass"], float(np.max(d["box"])))
    a.close()
    b.close()


def test_capacity_and_off(gpu_lib):
    d = DIAG["pm_ext"]
    cfg = cfg_from(d)
    pm = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    pm.setDiagnostics(2)
    pm.run(5)
    out = pm.diagnostics()
    assert out["taken"] == 6 and len(out["records"]) == 2
    pm.setDiagnostics(0)
    pm.run(1)
    assert pm.diagnostics()["taken"] == 0
    with pytest.raises(ValueError):
        pm.setDiagnostics(-1)
    pm.close()
