"""GPU parity of the PM path (through the C ABI) against the reference's outputs (golden
fixtures generated from the reference's CPU code) and the FP64 oracle port.

Tolerances (stated per test): RMS-over-particles relative force error <= 1e-5 against the
FP64 oracle and against the reference's FP32 result (the reference's own FP32 error vs FP64
is up to ~9e-6 with the S2 influence function); the density mesh is bit-exact against an
exact integer sum of the reference's float contributions.
"""
import numpy as np
import pytest

from conftest import load_npz, rel_rms
from oracle import oracle as O
from test_oracle_pin import cfg_from

pytestmark = pytest.mark.gpu

PM = load_npz("pm_forces.npz")
RUNS = load_npz("runs.npz")


def make_pm(cfg: O.PMConfig, pos, vel, mass, **kw):
    import particlesimulation_gb300 as P
    ext = None
    if cfg.ext:
        ext = P.SphRadDecrField(center=cfg.ext[:3], R=cfg.ext[3], M=cfg.ext[4], G=cfg.ext[5])
    state = np.concatenate([pos, vel]).astype(np.float32)
    return P.PMMethod(state, mass, cfg.box, ext, cfg.H, cfg.DT, cfg.G,
                      P.InterpolationScheme(cfg.interpolation), P.FiniteDiffScheme(cfg.finite_diff),
                      P.GreensFunction(cfg.greens), cfg.diameter, cfg.grid, **kw)


def gpu_pm_accel(cfg, pos, vel, mass):
    pm = make_pm(cfg, pos, vel, mass)
    pm.pmMethodStep()
    acc = pm.getParticles()[2]
    return pm, acc


@pytest.mark.parametrize("case", [c for c in PM if c != "inputs"])
def test_pm_force_matches_reference_and_fp64(gpu_lib, case):
    d = PM[case]
    inp = d if "pos" in d else PM["inputs"]
    cfg = cfg_from(d)
    pm, acc = gpu_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"])
    f64 = O.port_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"], prec=1)
    assert rel_rms(acc, f64) < 1e-5, "vs FP64 oracle"
    tol = 2e-5 if cfg.greens == 2 else 1e-5  # reference FP32 S2 shape-factor error ~9e-6
    assert rel_rms(acc, d["acc"]) < tol, "vs reference FP32"
    pm.close()


def _code_mass(cfg, mass):
    f = np.float32
    c = f(f(f(f(f(cfg.DT) * f(cfg.DT)) * f(4)) * f(np.pi)) * f(cfg.G)) / f(f(f(cfg.H) * f(cfg.H)) * f(cfg.H))
    return (f(c) * mass.astype(np.float32)).astype(np.float32)


def _tsc_w(x, t):
    f = np.float32
    if t == 1:
        a = f(0.5) + x
        return a * a
    if t == 0:
        return f(1.5) - (f(2) * x) * x
    a = f(0.5) - x
    return a * a


def exact_density(cfg, pos, mass):
    """The density as an exact (integer) sum of the reference's float contributions, converted
    like the device does: fixed point 2^k, float of the int64 sum, times 2^-k."""
    f = np.float32
    H = f(cfg.H)
    x = (pos.astype(np.float32) / H).astype(np.float32)
    m = _code_mass(cfg, mass)
    msum = np.abs(m.astype(np.float64)).sum()
    k = min(int(np.floor(62.0 - np.log2(4.0 * msum))), 100)
    scale = np.float32(2.0 ** k)
    nx, ny, nz = cfg.grid
    acc = np.zeros(nx * ny * nz, np.int64)

    def add(ix, iy, iz, w):
        q = np.rint((w * scale).astype(np.float32).astype(np.float64)).astype(np.int64)
        idx = (ix % nx) + (iy % ny) * nx + (iz % nz) * nx * ny
        np.add.at(acc, idx, q)

    if cfg.interpolation == 0:
        ii = np.round(x).astype(np.int64)  # round half away from zero for positive values
        ii = np.where(x - np.floor(x) == 0.5, np.floor(x) + 1, ii).astype(np.int64)
        add(ii[:, 0], ii[:, 1], ii[:, 2], m)
    else:
        i0 = x.astype(np.int64)
        dx = (x - i0.astype(np.float32)).astype(np.float32)
        if cfg.interpolation == 1:
            t = (f(1) - dx).astype(np.float32)
            for ox in (0, 1):
                for oy in (0, 1):
                    for oz in (0, 1):
                        wx = dx[:, 0] if ox else t[:, 0]
                        wy = dx[:, 1] if oy else t[:, 1]
                        wz = dx[:, 2] if oz else t[:, 2]
                        w = ((m * wx).astype(np.float32) * wy).astype(np.float32) * wz
                        add(i0[:, 0] + ox, i0[:, 1] + oy, i0[:, 2] + oz, w.astype(np.float32))
        else:
            d8 = (m / f(8)).astype(np.float32)
            for t1 in (-1, 0, 1):
                T1 = (d8 * _tsc_w(dx[:, 0], t1)).astype(np.float32)
                for t2 in (-1, 0, 1):
                    T2 = (T1 * _tsc_w(dx[:, 1], t2)).astype(np.float32)
                    for t3 in (-1, 0, 1):
                        T3 = (T2 * _tsc_w(dx[:, 2], t3)).astype(np.float32)
                        add(i0[:, 0] + t1, i0[:, 1] + t2, i0[:, 2] + t3, T3)
    return (acc.astype(np.float32) * np.float32(2.0 ** -k)).astype(np.float32)


@pytest.mark.parametrize("case", ["pm_is0_fd0_gf3", "pm_is1_fd0_gf0", "pm_is2_fd0_gf2"])
def test_density_bit_exact_and_deterministic(gpu_lib, case):
    d = PM[case]
    inp = PM["inputs"]
    cfg = cfg_from(d)
    pm, _ = gpu_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"])
    dens1 = pm.getGridDensity()
    pm.pmMethodStep()
    dens2 = pm.getGridDensity()
    np.testing.assert_array_equal(dens1.view(np.uint32), dens2.view(np.uint32))
    np.testing.assert_array_equal(dens1, exact_density(cfg, inp["pos"], inp["mass"]))
    # the reference accumulates in float: same values to float rounding
    assert np.abs(dens1 - d["density"]).max() <= 2e-6 * np.abs(d["density"]).max()
    pm.close()


@pytest.mark.parametrize("case", ["pm_is1_fd0_gf0", "pm_is2_fd0_gf2", "pm_is2_fd1_gf1", "pm_is0_fd0_gf3"])
def test_green_and_potential_match_fp64(gpu_lib, case):
    d = PM[case]
    inp = PM["inputs"]
    cfg = cfg_from(d)
    pm, _ = gpu_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"])
    _, _, pot64, g64 = O.port_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"], prec=1,
                                       want_mesh=True)
    nx, ny, nz = cfg.grid
    g = g64.reshape(nz, ny, nx)
    gneg = np.roll(np.flip(g, (0, 1, 2)), 1, (0, 1, 2))  # G(-k)
    want = 0.5 * (g + gneg)[:, :, : nx // 2 + 1] / (nx * ny * nz)
    got = pm.getGreensFunction()
    assert np.abs(got - want).max() <= 2e-6 * np.abs(want).max()
    pot = pm.getGridPotential()
    assert np.sqrt(((pot - pot64) ** 2).mean()) <= 1e-5 * np.sqrt((pot64 ** 2).mean())
    pm.close()


def test_pm_run_matches_reference_run(gpu_lib):
    d = RUNS["pm"]
    cfg = cfg_from(d)
    pm = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    escaped, steps = pm.run(int(d["sim_length"]))
    assert not escaped and steps == int(d["sim_length"]) + 1
    x, v, _ = pm.getParticles(units="original")
    assert np.abs(x - d["pos_out"]).max() < 2e-6 * np.abs(d["pos_out"]).max()
    assert rel_rms(v, d["vel_out"]) < 1e-5
    pm.close()


def test_escape_stops_like_reference(gpu_lib):
    d = RUNS["escape"]
    cfg = cfg_from(d)
    pm = make_pm(cfg, d["pos"], d["vel"], d["mass"])
    escaped, steps = pm.run(int(d["sim_length"]))
    assert escaped == bool(d["escaped"]) and escaped
    assert steps < int(d["sim_length"])
    x, v, _ = pm.getParticles(units="original")
    assert np.abs(x - d["pos_out"]).max() < 2e-6 * np.abs(d["pos_out"]).max()
    assert rel_rms(v, d["vel_out"]) < 1e-5
    assert pm.escapedComputationalBox()
    pm.close()


PMACC = load_npz("pm_accuracy.npz")


@pytest.mark.parametrize("case", [c for c in PMACC if c != "inputs"])
def test_pm_non_power_of_two_meshes(gpu_lib, case):
    """Meshes of the reference's pmAccuracy scenario ((2 Ng, 2 Ng, Ng), Ng = 30, 34, 58: the
    mixed-radix Poisson solve) against the reference's own forces and the FP64 oracle; 1e-5
    RMS-normalised."""
    d = PMACC[case]
    inp = PMACC["inputs"]
    cfg = cfg_from(d)
    pm, acc = gpu_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"])
    f64 = O.port_pm_accel(cfg, inp["pos"], inp["vel"], inp["mass"], prec=1)
    assert rel_rms(acc, f64) < 1e-5, "vs FP64 oracle"
    assert rel_rms(acc, d["acc"]) < 1e-5, "vs reference FP32"
    # a short run through the same path
    escaped, steps = pm.run(2)
    assert not escaped and steps == 3
    pm.close()


@pytest.mark.parametrize("dims", [(30, 60, 60), (7, 11, 13), (1, 1, 4096), (16, 16, 16), (3, 5, 97)])
def test_fft_adapter_matches_numpy(gpu_lib, dims):
    """FFTAdapter<float> (pmgb_fft3d): forward unnormalised, inverse scaled by 1/N, as the
    reference's adapters; against numpy's FFT in double, 1e-5 RMS-normalised."""
    from particlesimulation_gb300 import methods as M
    rng = np.random.default_rng(sum(dims))
    a = (rng.standard_normal(dims) + 1j * rng.standard_normal(dims)).astype(np.complex64)
    f = M.FFTAdapter(dims)
    got = f.fft(a)
    want = np.fft.fftn(a.astype(np.complex128))
    assert np.sqrt(np.mean(np.abs(got - want) ** 2) / np.mean(np.abs(want) ** 2)) < 1e-5
    back = f.ifft(got)
    assert np.sqrt(np.mean(np.abs(back - a) ** 2) / np.mean(np.abs(a) ** 2)) < 1e-5


def test_invalid_arguments_raise(gpu_lib):
    import particlesimulation_gb300 as P
    cfg = O.PMConfig(grid=(3, 32, 32), box=(30.0,) * 3, H=30 / 16)
    p = np.full((4, 3), 10.0, np.float32)
    with pytest.raises(ValueError):
        make_pm(cfg, p, p * 0, np.ones(4, np.float32))
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0,) * 3, H=30 / 16, greens=1, diameter=0.0)
    with pytest.raises(ValueError):
        make_pm(cfg, p, p * 0, np.ones(4, np.float32))


def test_periodic_blobs_force_and_determinism(gpu_lib):
    """Periodic mesh (the 256^3 workload's mode) at 64^3: forces vs the FP64 port with wrapped
    indices; two runs give bit-identical densities."""
    from particlesimulation_gb300 import workloads as W
    w = W.blobs_periodic(n=20000, seed=5, grid=64)
    cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=1,
                     finite_diff=0, greens=0, periodic=1)
    pm = make_pm(cfg, w.pos, w.vel, w.mass, periodic=True)
    pm.pmMethodStep()
    acc = pm.getParticles()[2]
    f64 = O.port_pm_accel(cfg, w.pos, w.vel, w.mass, prec=1)
    assert rel_rms(acc, f64) < 1e-5
    d1 = pm.getGridDensity()
    pm2 = make_pm(cfg, w.pos[::-1].copy(), w.vel[::-1].copy(), w.mass[::-1].copy(), periodic=True)
    pm2.pmMethodStep()
    np.testing.assert_array_equal(d1, pm2.getGridDensity())  # order-independent
    escaped, steps = pm.run(5)
    assert not escaped and steps == 6
    x, _, _ = pm.getParticles(units="code")
    assert (x >= 0).all() and (x <= 64).all()
    pm.close()
    pm2.close()


def test_large_pm_properties(gpu_lib):
    """Full-size 256^3 periodic workload (4M particles): mass conservation of the
    fixed-point deposit and bit-identical density across two force evaluations."""
    from particlesimulation_gb300 import workloads as W
    w = W.blobs_periodic()
    cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=1,
                     finite_diff=0, greens=0, periodic=1)
    pm = make_pm(cfg, w.pos, w.vel, w.mass, periodic=True)
    pm.pmMethodStep()
    d1 = pm.getGridDensity()
    pm.pmMethodStep()
    d2 = pm.getGridDensity()
    np.testing.assert_array_equal(d1.view(np.uint32), d2.view(np.uint32))
    mc = _code_mass(cfg, w.mass).astype(np.float64).sum()
    assert abs(d1.astype(np.float64).sum() - mc) < 1e-5 * mc
    acc = pm.getParticles()[2]
    assert np.isfinite(acc).all()
    pm.close()
