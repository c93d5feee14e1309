"""Generates tests/golden/*.npz from the reference's own CPU code (oracle/_ref/libpsref.so,
compiled from the reference sources by oracle/Makefile).

Run where the reference sources exist, naming the checkout:
    PSIM_REFERENCE=<reference checkout> python tests/golden/make_golden.py \
        [diagnostics|recorder|samplers|field_sweeps|pm_accuracy|p3m_exact]
(with an argument, only that fixture is rewritten).
Every case is a small seeded input; each fixture stores the inputs, the settings and the
reference's outputs (float32), so tests on a machine without the reference still compare
against the reference itself.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def inputs(seed, n, lo, hi, clustered=True):
    rng = np.random.default_rng(seed)
    if clustered:
        c = 0.5 * (lo + hi)
        p = np.concatenate([rng.normal(c, 0.08 * (hi - lo), (n // 2, 3)),
                            rng.uniform(lo, hi, (n - n // 2, 3))])
        p = np.clip(p, lo, hi)
    else:
        p = rng.uniform(lo, hi, (n, 3))
    v = rng.normal(0, 0.02, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    return p.astype(np.float32), v.astype(np.float32), m.astype(np.float32)


def pm_cases():
    H = 30.0 / 16
    out = []
    k = 0
    for is_ in (0, 1, 2):
        for fds in (0, 1):
            for gf in (0, 1, 2, 3):
                ext = (15.0, 15.0, 15.0, 3.0, 0.5, 1.0) if (k % 3 == 0) else ()
                cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                                 interpolation=is_, finite_diff=fds, greens=gf, diameter=3 * H,
                                 ext=ext)
                out.append((f"pm_is{is_}_fd{fds}_gf{gf}", cfg))
                k += 1
    # non-cubic mesh, as the reference's galaxy demos use (128 x 128 x 64 scaled down)
    cfg = O.PMConfig(grid=(32, 32, 16), box=(30.0, 30.0, 15.0), H=H, DT=0.1, G=1.0,
                     interpolation=2, finite_diff=0, greens=0, diameter=0.0)
    out.append(("pm_noncubic_tsc", cfg))
    return out


MESH_CASES = ("pm_is1_fd0_gf0", "pm_is2_fd0_gf2", "pm_is2_fd1_gf1", "pm_is0_fd0_gf3")


def diagnostics_fixture():
    """Runs with collectDiagnostics = true: the reference's recorded energy, momentum, angular
    momentum and expected momentum per iteration (StateRecorder text files), PM with an external
    field, P3M, and a run that stops on an escaped particle."""
    H = 30.0 / 16
    p, v, m = inputs(60, 900, 8.0, 22.0)
    cases = {}
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                     interpolation=1, finite_diff=0, greens=0, diameter=0.0,
                     ext=(15.0, 15.0, 15.0, 3.0, 0.5, 1.0))
    x, vv, esc, d = O.ref_run(cfg, None, p, v, m, 5, diagnostics=True)
    cases["pm_ext"] = dict(pos=p, vel=v, mass=m, diag=d, escaped=np.int32(esc),
                           sim_length=np.int32(5), **_cfg_arrays(cfg))
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                     interpolation=2, finite_diff=0, greens=2, diameter=3 * H)
    q = O.P3MConfig(comp_box=(30.0, 30.0, 30.0), cutoff=3 * H, diameter=3 * H, cloud_shape=1)
    x, vv, esc, d = O.ref_run(cfg, q, p, v, m, 3, diagnostics=True)
    cases["p3m"] = dict(pos=p, vel=v, mass=m, diag=d, escaped=np.int32(esc),
                        sim_length=np.int32(3), **_cfg_arrays(cfg), **_p3m_arrays(q))
    pe = p.copy()
    pe[:10, 0] = 29.6
    ve = v.copy()
    ve[:10, 0] = 0.05 * 30
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                     interpolation=1, finite_diff=0, greens=0, diameter=0.0)
    x, vv, esc, d = O.ref_run(cfg, None, pe, ve, m, 6, diagnostics=True)
    cases["escape"] = dict(pos=pe, vel=ve, mass=m, diag=d, escaped=np.int32(esc),
                           sim_length=np.int32(6), **_cfg_arrays(cfg))
    np.savez_compressed(os.path.join(HERE, "diagnostics.npz"),
                        **{f"{c}/{k}": a for c, dd in cases.items() for k, a in dd.items()})


def recorder_fixture():
    """The reference's StateRecorder files (raw bytes) of PM runs with collectDiagnostics and
    recordField: one with an external field, one stopped by an escaped particle."""
    import tempfile
    H = 30.0 / 16
    p, v, m = inputs(70, 800, 8.0, 22.0)
    out = {}
    cases = []
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                     interpolation=2, finite_diff=1, greens=0, diameter=0.0,
                     ext=(15.0, 15.0, 15.0, 3.0, 0.5, 1.0))
    cases.append(("ext", cfg, p, v, 5))
    pe, ve = p.copy(), v.copy()
    pe[:10, 0] = 29.6
    ve[:10, 0] = 0.05 * 30
    cfg2 = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                      interpolation=1, finite_diff=0, greens=0, diameter=0.0)
    cases.append(("escape", cfg2, pe, ve, 6))
    for name, c, pp, vv, steps in cases:
        with tempfile.TemporaryDirectory() as d:
            esc, files = O.ref_run_files(c, None, pp, vv, m, steps, d, diagnostics=True,
                                         record_field=True)
        out[name] = dict(pos=pp, vel=vv, mass=m, escaped=np.int32(esc), sim_length=np.int32(steps),
                         **_cfg_arrays(c),
                         **{f"file:{k}": np.frombuffer(b, np.uint8) for k, b in files.items()})
    np.savez_compressed(os.path.join(HERE, "recorder.npz"),
                        **{f"{c}/{k}": a for c, dd in out.items() for k, a in dd.items()})


def field_sweeps_fixture():
    """The reference's positions.dat / field.dat of three PM field sweeps of its demos
    (source/demos.cpp:109-591): a mass-1 particle with 399 massless tracers every 0.075 along x
    from (30, 30, 15), 64 x 64 x 32 mesh, box 60 x 60 x 30, H = 60/32, G = 4.5e-3, DT = 1, one
    iteration with the field recorded (the scenario command line's anisotropy,
    pm-optimal and assignment-schemes options write the same runs)."""
    import tempfile
    n = 400
    pos = np.zeros((n, 3), np.float32)
    for i in range(n):  # linearSpacing: center + i * dx * dir, in float
        pos[i] = np.float32(30) + np.float32(i) * np.float32(0.075), 30, 15
    vel = np.zeros((n, 3), np.float32)
    mass = np.zeros(n, np.float32)
    mass[0] = 1
    H = np.float32(60.0) / np.float32(32)
    out = {}
    for name, interp, fds, greens, diam in (("aniso", 2, 0, 0, 0.0), ("optimal_s2", 2, 1, 2, 4 * H),
                                              ("ngp", 0, 1, 0, 0.0)):
        cfg = O.PMConfig(grid=(64, 64, 32), box=(60.0, 60.0, 30.0), H=float(H), DT=1.0, G=4.5e-3,
                         interpolation=interp, finite_diff=fds, greens=greens, diameter=float(diam))
        with tempfile.TemporaryDirectory() as d:
            esc, files = O.ref_run_files(cfg, None, pos, vel, mass, 1, d, diagnostics=False,
                                         record_field=True)
        assert not esc
        out[name] = {"positions": np.frombuffer(files["positions.dat"], np.uint8),
                     "field": np.frombuffer(files["field.dat"], np.uint8)}
    np.savez_compressed(os.path.join(HERE, "field_sweeps.npz"),
                        **{f"{c}/{k}": a for c, dd in out.items() for k, a in dd.items()})


def samplers_fixture():
    """PlummerSampler(42) and DiskSamplerLinear(42) samples of the reference with the parameters
    of its plummerPM / galaxy demos (source/demos.cpp:361-372, 1369-1384); the disk also with
    an inner radius r0 (the galaxy-collision demo) and with 2n particles in one call (its second
    half is what a second sample() call of the same sampler returns)."""
    n = 5000
    out = {
        "plummer": O.ref_sample_plummer(42, (30, 30, 30), 2.0, 15.0, 1.0, 4.5e-3, n),
        "disk": O.ref_sample_disk_linear(42, (30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, n),
        "disk_r0": O.ref_sample_disk_linear(7, (30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, n, 3.0),
        "disk_2n": O.ref_sample_disk_linear(42, (30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, 2 * n),
    }
    np.savez_compressed(os.path.join(HERE, "samplers.npz"), **out)


def main():
    assert O.build_ref(), "set PSIM_REFERENCE to the reference checkout"
    os.makedirs(HERE, exist_ok=True)
    # ---- PM forces (single pmMethodStep after unit conversion and Green's function)
    p, v, m = inputs(10, 600, 3.0, 27.0)
    cases = {}
    for name, cfg in pm_cases():
        lo_hi = (3.0, 12.0) if cfg.grid[2] == 16 else (3.0, 27.0)
        pp, vv, mm = (p, v, m) if cfg.grid[2] == 32 else inputs(11, 600, *lo_hi)
        acc, dens, pot, grn = O.ref_pm_accel(cfg, pp, vv, mm, want_mesh=True)
        d = dict(acc=acc, **_cfg_arrays(cfg))
        if cfg.grid[2] != 32:
            d.update(pos=pp, vel=vv, mass=mm)
        if name in MESH_CASES:  # meshes for a few cases only (fixture size)
            d.update(density=dens, potential=pot, green=grn)
        cases[name] = d
    cases["inputs"] = dict(pos=p, vel=v, mass=m)
    np.savez_compressed(os.path.join(HERE, "pm_forces.npz"),
                        **{f"{c}/{k}": a for c, d in cases.items() for k, a in d.items()})
    # ---- P3M forces
    H = 30.0 / 16
    p, v, m = inputs(20, 3000, 4.0, 26.0)
    cases = {}
    for cs, gf in ((0, 1), (1, 2)):
        for table in (1, 0):
            for ys in (1, 0):
                cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                                 interpolation=2, finite_diff=0, greens=gf, diameter=3 * H)
                q = O.P3MConfig(comp_box=(30.0, 30.0, 30.0), cutoff=3 * H, diameter=3 * H,
                                softening=0.0 if table else 0.2, cloud_shape=cs, use_table=table,
                                y_sorting=ys)
                acc = O.ref_p3m_accel(cfg, q, p, v, m)
                cases[f"p3m_cs{cs}_t{table}_y{ys}"] = dict(acc=acc, **_cfg_arrays(cfg),
                                                           **_p3m_arrays(q))
    cases["inputs"] = dict(pos=p, vel=v, mass=m)
    np.savez_compressed(os.path.join(HERE, "p3m_forces.npz"),
                        **{f"{c}/{k}": a for c, d in cases.items() for k, a in d.items()})
    # ---- chaining-mesh cell lists (code-unit positions), including exact y ties
    rng = np.random.default_rng(30)
    pc = rng.uniform(0, 16, (4000, 3)).astype(np.float32)
    pc[:400, 1] = np.float32(7.25)                     # many equal y values
    pc[400:440] = pc[440:480]                          # duplicated particles
    q = O.P3MConfig(comp_box=(30.0, 30.0, 30.0), cutoff=3 * H, diameter=3 * H)
    cl = {}
    for ys in (1, 0):
        order, counts, dims = O.ref_chaining_mesh(q, H, pc, ys)
        cl[f"y{ys}/order"] = order
        cl[f"y{ys}/counts"] = counts
        cl[f"y{ys}/dims"] = np.array(dims, np.int32)
    np.savez_compressed(os.path.join(HERE, "cell_lists.npz"), pos_code=pc, H=np.float32(H),
                        **{f"q/{k}": a for k, a in _p3m_arrays(q).items()}, **cl)
    # ---- short runs (run(simLength) from the reference, final state in original units)
    p, v, m = inputs(40, 800, 8.0, 22.0)
    runs = {}
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                     interpolation=1, finite_diff=0, greens=0, diameter=0.0)
    x, vv, esc = O.ref_run(cfg, None, p, v, m, 4)
    runs["pm"] = dict(pos=p, vel=v, mass=m, pos_out=x, vel_out=vv, escaped=np.int32(esc),
                      sim_length=np.int32(4), **_cfg_arrays(cfg))
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                     interpolation=2, finite_diff=0, greens=2, diameter=3 * H)
    q = O.P3MConfig(comp_box=(30.0, 30.0, 30.0), cutoff=3 * H, diameter=3 * H, cloud_shape=1)
    x, vv, esc = O.ref_run(cfg, q, p, v, m, 3)
    runs["p3m"] = dict(pos=p, vel=v, mass=m, pos_out=x, vel_out=vv, escaped=np.int32(esc),
                       sim_length=np.int32(3), **_cfg_arrays(cfg), **_p3m_arrays(q))
    # escape: particles pushed out of the box by a strong external field pointing outwards
    pe = p.copy()
    pe[:10, 0] = 29.6
    ve = v.copy()
    ve[:10, 0] = 0.05 * 30
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                     interpolation=1, finite_diff=0, greens=0, diameter=0.0)
    x, vv, esc = O.ref_run(cfg, None, pe, ve, m, 6)
    runs["escape"] = dict(pos=pe, vel=ve, mass=m, pos_out=x, vel_out=vv, escaped=np.int32(esc),
                          sim_length=np.int32(6), **_cfg_arrays(cfg))
    np.savez_compressed(os.path.join(HERE, "runs.npz"),
                        **{f"{c}/{k}": a for c, d in runs.items() for k, a in d.items()})
    # ---- SR force table and FP32 direct sum
    t = {}
    for cs in (0, 1):
        for eps in (0.0, 0.5):
            qq = O.P3MConfig(comp_box=(30.0,) * 3, cutoff=3 * H, diameter=3 * H, softening=eps,
                             cloud_shape=cs)
            t[f"cs{cs}_eps{eps}"] = O.ref_sr_table(qq, H)[0]
    pp, _, mm = inputs(50, 300, 0.0, 10.0)
    t["pp_pos"] = pp
    t["pp_mass"] = mm
    t["pp_acc"] = O.ref_pp_accel(pp, mm, 1.0, 0.0)
    np.savez_compressed(os.path.join(HERE, "misc.npz"), **t)
    print("golden fixtures written to", HERE)


def p3m_exact_fixture():
    """The reference's table-free short-range force (useSRForceTable = false, softening 0:
    shortRangeForce, source/p3mMethod.cpp:220-238) on the P3M inputs of p3m_forces.npz: S1 and
    S2 shapes, y-sorted and unsorted chaining mesh, and a diameter below the cutoff (a = 2H,
    re = 3H, so pairs at a <= r < re feel the pure Newtonian remainder)."""
    H = 30.0 / 16
    p, v, m = inputs(20, 3000, 4.0, 26.0)
    cases = {"inputs": dict(pos=p, vel=v, mass=m)}
    for cs, gf in ((0, 1), (1, 2)):
        for ys in (1, 0):
            for amul in (3.0, 2.0):
                cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.1, G=1.0,
                                 interpolation=2, finite_diff=0, greens=gf, diameter=amul * H)
                q = O.P3MConfig(comp_box=(30.0, 30.0, 30.0), cutoff=3 * H, diameter=amul * H,
                                softening=0.0, cloud_shape=cs, use_table=0, y_sorting=ys)
                acc = O.ref_p3m_accel(cfg, q, p, v, m)
                cases[f"exact_cs{cs}_y{ys}_a{int(amul)}"] = dict(acc=acc, **_cfg_arrays(cfg),
                                                                 **_p3m_arrays(q))
    np.savez_compressed(os.path.join(HERE, "p3m_exact.npz"),
                        **{f"{c}/{k}": a for c, dd in cases.items() for k, a in dd.items()})


def pm_accuracy_fixture():
    """The reference's PM forces on the meshes of its accuracy scenario pmAccuracy
    (source/demos.cpp:361-428): a linear disk from DiskSamplerLinear(42) (centre (30, 30, 15),
    rb 3, mb 60, rd 15, md 15, thickness 0.3, G 4.5e-3; 2,000 particles here), effective box
    60 x 60 x 30, meshes (2 Ng, 2 Ng, Ng) for Ng = 30, 34, 58 (not powers of two: factors 2, 3,
    5, 17, 29), H = 60 / Ng, DT 1, discrete-Laplacian Green's function, every interpolation and
    difference scheme at Ng = 30."""
    n = 2000
    st = O.ref_sample_disk_linear(42, np.array([30, 30, 15], np.float32), 3.0, 60.0, 15.0, 15.0,
                                  0.3, 4.5e-3, n)
    pos, vel = st[:n].astype(np.float32), st[n:].astype(np.float32)
    mass = np.full(n, 15.0 / n, np.float32)
    cases = {"inputs": dict(pos=pos, vel=vel, mass=mass)}
    combos = [(30, is_, fds) for is_ in (0, 1, 2) for fds in (0, 1)] + [(34, 2, 0), (58, 1, 1)]
    for ng, is_, fds in combos:
        cfg = O.PMConfig(grid=(2 * ng, 2 * ng, ng), box=(60.0, 60.0, 30.0), H=60.0 / ng, DT=1.0,
                         G=4.5e-3, interpolation=is_, finite_diff=fds, greens=0, diameter=0.0)
        acc = O.ref_pm_accel(cfg, pos, vel, mass)
        acc = acc[0] if isinstance(acc, tuple) else acc
        cases[f"ng{ng}_is{is_}_fd{fds}"] = dict(acc=np.asarray(acc, np.float32), **_cfg_arrays(cfg))
    np.savez_compressed(os.path.join(HERE, "pm_accuracy.npz"),
                        **{f"{c}/{k}": a for c, dd in cases.items() for k, a in dd.items()})


def _cfg_arrays(cfg):
    return dict(grid=np.array(cfg.grid, np.int32), box=np.array(cfg.box, np.float32),
                HDTG=np.array([cfg.H, cfg.DT, cfg.G], np.float32),
                scheme=np.array([cfg.interpolation, cfg.finite_diff, cfg.greens], np.int32),
                diameter=np.float32(cfg.diameter),
                ext=np.array(cfg.ext if cfg.ext else [np.nan] * 6, np.float32))


def _p3m_arrays(q):
    return dict(comp_box=np.array(q.comp_box, np.float32),
                cds=np.array([q.cutoff, q.diameter, q.softening], np.float32),
                flags=np.array([q.cloud_shape, q.use_table, q.y_sorting], np.int32))


if __name__ == "__main__":
    if sys.argv[1:] == ["diagnostics"]:
        diagnostics_fixture()
    elif sys.argv[1:] == ["recorder"]:
        recorder_fixture()
    elif sys.argv[1:] == ["samplers"]:
        samplers_fixture()
    elif sys.argv[1:] == ["field_sweeps"]:
        field_sweeps_fixture()
    elif sys.argv[1:] == ["pm_accuracy"]:
        pm_accuracy_fixture()
    elif sys.argv[1:] == ["p3m_exact"]:
        p3m_exact_fixture()
    else:
        main()
        diagnostics_fixture()
        recorder_fixture()
        samplers_fixture()
        field_sweeps_fixture()
        pm_accuracy_fixture()
        p3m_exact_fixture()
