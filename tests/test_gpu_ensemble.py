"""The batched ensemble against the same systems run one by one through PMMethod: every system
must be bit-identical (the ensemble kernels call the same device bodies; tile shapes chosen by
the autotuner do not change the arithmetic), and must agree with the FP64 oracle's force."""
import numpy as np
import pytest

from conftest import rel_rms
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _single(w, steps):
    import particlesimulation_gb300 as P
    pm = P.PMMethod(w.state, w.mass, w.box, None, w.H, w.DT, w.G, P.InterpolationScheme(w.interpolation),
                    P.FiniteDiffScheme(w.finite_diff), P.GreensFunction(w.greens), w.diameter, w.grid)
    esc, _ = pm.run(steps)
    out = pm.getParticles(units="original")
    pm.close()
    return esc, out


def test_ensemble_matches_single_runs(gpu_lib):
    from particlesimulation_gb300 import methods
    from particlesimulation_gb300 import workloads as W
    ws = W.plummer_ensemble(n_systems=6, seed=21, nmin=2000, nmax=40000)
    assert len({w.grid for w in ws}) >= 2  # uneven meshes
    ens = methods.Ensemble([W.as_system(w) for w in ws])
    tun = ens.tuning()
    assert tun["deposit_particles_per_thread"] in (1, 2, 4) and tun["x_rows_mult"] in (0, 1, 2)
    steps = 5
    esc, ms = ens.run(steps)
    assert not any(esc) and ms > 0
    for s, w in enumerate(ws):
        e1, (x1, v1, a1) = _single(w, steps)
        x, v, a = ens.getParticles(s, units="original")
        assert not e1
        np.testing.assert_array_equal(x, x1)
        np.testing.assert_array_equal(v, v1)
        np.testing.assert_array_equal(a, a1)
    ens.close()


def test_ensemble_force_matches_fp64_and_escape_is_per_system(gpu_lib):
    from particlesimulation_gb300 import methods
    from particlesimulation_gb300 import workloads as W
    ws = W.plummer_ensemble(n_systems=3, seed=5, nmin=3000, nmax=8000)
    # system 1: a few particles leave the box on the first drift
    ws[1].pos[:5, 0] = np.float32(29.95)
    ws[1].vel[:5, 0] = np.float32(50.0)
    ens = methods.Ensemble([W.as_system(w) for w in ws])
    esc, _ = ens.run(0)
    assert esc == [False, True, False]
    # the force of the initial step (run(0) ends with a force evaluation after one drift) is
    # checked against the FP64 oracle at the same positions
    for s in (0, 2):
        w = ws[s]
        x, _, a = ens.getParticles(s, units="code")
        cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=w.interpolation,
                         finite_diff=w.finite_diff, greens=w.greens, diameter=w.diameter)
        xo = (x * np.float32(w.H)).astype(np.float32)
        f64 = O.port_pm_accel(cfg, xo, np.zeros_like(xo), w.mass, prec=1)
        assert rel_rms(a, f64) < 1e-5
    ens.close()
