"""GPU parity of the P3M path (chaining mesh + short-range pair pass) through the C ABI.

Cell lists are compared bit for bit with the reference's ChainingMesh (golden fixtures, exact
y ties and duplicated particles included).  Forces: RMS relative error <= 1e-5 against the FP64
oracle and against the reference's FP32 result, on small cases and, at the full 262,144-particle
disk workload, on a 1,500-particle subsample (FP64 PM + brute-force short-range sum).
"""
import numpy as np
import pytest

from conftest import load_npz, rel_rms
from oracle import oracle as O
from test_gpu_pm import make_pm
from test_oracle_pin import cfg_from, p3m_from

pytestmark = pytest.mark.gpu

P3M = load_npz("p3m_forces.npz")


def make_p3m(cfg, q, pos, vel, mass):
    import particlesimulation_gb300 as P
    pm = make_pm(cfg, pos, vel, mass)
    p3m = P.P3MMethod(pm, q.comp_box, q.cutoff, q.diameter, cfg.H, q.softening,
                      P.CloudShape(q.cloud_shape), bool(q.use_table), bool(q.y_sorting))
    return pm, p3m


@pytest.mark.parametrize("case", [c for c in P3M if c != "inputs"])
def test_p3m_force_matches_reference_and_fp64(gpu_lib, case):
    d = P3M[case]
    inp = P3M["inputs"]
    cfg, q = cfg_from(d), p3m_from(d)
    pm, p3m = make_p3m(cfg, q, inp["pos"], inp["vel"], inp["mass"])
    p3m.force()
    acc = pm.getParticles()[2]
    f64 = O.port_p3m_accel(cfg, q, inp["pos"], inp["vel"], inp["mass"], prec=1)
    assert rel_rms(acc, f64) < 1e-5, "vs FP64 oracle"
    # the direct (table-free) S1/S2 formulas lose ~1.5e-5 to FP32 cancellation in the reference
    tol = 1e-5 if q.use_table else 3e-5
    assert rel_rms(acc, d["acc"]) < tol, "vs reference FP32"
    p3m.close()
    pm.close()


EXACT = load_npz("p3m_exact.npz")


@pytest.mark.parametrize("case", [c for c in EXACT if c != "inputs"])
def test_p3m_table_free_force(gpu_lib, case):
    """useSRForceTable = false without softening: the slotted pass's exact mode (Newton part
    from rsqrt, R(r)/r from a 499-segment table) against the FP64 oracle and the reference's
    FP32 result.  Without the table's cap at r -> 0 the close pairs' 1/r^2 magnifies the float
    rounding of the code-unit positions: the reference's own FP32 result is 3.8e-5 (RMS-
    normalised) from FP64 on these inputs, so the bars are 6e-5 vs FP64 and 3e-5 vs the
    reference's FP32 result."""
    d = EXACT[case]
    inp = EXACT["inputs"]
    cfg, q = cfg_from(d), p3m_from(d)
    pm, p3m = make_p3m(cfg, q, inp["pos"], inp["vel"], inp["mass"])
    p3m.force()
    acc = pm.getParticles()[2].copy()
    f64 = O.port_p3m_accel(cfg, q, inp["pos"], inp["vel"], inp["mass"], prec=1)
    assert rel_rms(acc, f64) < 6e-5, "vs FP64 oracle"
    assert rel_rms(acc, d["acc"]) < 3e-5, "vs reference FP32"
    p3m.force()
    np.testing.assert_array_equal(acc, pm.getParticles()[2])  # deterministic
    p3m.close()
    pm.close()


@pytest.mark.parametrize("ys", [1, 0])
def test_cell_lists_bit_exact(gpu_lib, ys):
    d = load_npz("cell_lists.npz")
    H = float(d["H"])
    pc = d["pos_code"]
    n = len(pc)
    q = O.P3MConfig(comp_box=tuple(float(b) for b in d["q"]["comp_box"]),
                    cutoff=float(d["q"]["cds"][0]), diameter=float(d["q"]["cds"][1]),
                    cloud_shape=1, y_sorting=ys)
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0,) * 3, H=H, DT=0.1, G=1.0, interpolation=2,
                     finite_diff=0, greens=0)
    pm, p3m = make_p3m(cfg, q, pc * np.float32(H), np.zeros_like(pc), np.full(n, 1.0 / n, np.float32))
    pm.setParticles(pc, np.zeros_like(pc), units="code")  # the fixture's code-unit positions
    p3m.force()
    order, counts, dims = p3m.getCellLists()
    assert dims == tuple(d[f"y{ys}"]["dims"])
    np.testing.assert_array_equal(counts, d[f"y{ys}"]["counts"])
    np.testing.assert_array_equal(order, d[f"y{ys}"]["order"])
    # twice in a row (the particles are now in sorted order: ties must still go by index)
    p3m.force()
    order2, counts2, _ = p3m.getCellLists()
    np.testing.assert_array_equal(order2, d[f"y{ys}"]["order"])
    p3m.close()
    pm.close()


def test_sr_table_matches_reference(gpu_lib):
    d = load_npz("misc.npz")
    H = 30.0 / 16
    for cs in (0, 1):
        for eps in (0.0, 0.5):
            q = O.P3MConfig(comp_box=(30.0,) * 3, cutoff=3 * H, diameter=3 * H, softening=eps,
                            cloud_shape=cs)
            cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0,) * 3, H=H)
            p = np.full((2, 3), 15.0, np.float32)
            pm, p3m = make_p3m(cfg, q, p, p * 0, np.ones(2, np.float32))
            t, _ = p3m.getSRForceTable()
            np.testing.assert_allclose(t, d[f"cs{cs}_eps{eps}"], rtol=2e-6, atol=0)
            p3m.close()
            pm.close()


def test_p3m_run_matches_reference_run(gpu_lib):
    d = load_npz("runs.npz")["p3m"]
    cfg, q = cfg_from(d), p3m_from(d)
    pm, p3m = make_p3m(cfg, q, d["pos"], d["vel"], d["mass"])
    escaped, steps = p3m.run(int(d["sim_length"]))
    assert not escaped and steps == int(d["sim_length"]) + 1
    x, v, _ = pm.getParticles(units="original")
    assert np.abs(x - d["pos_out"]).max() < 2e-6 * np.abs(d["pos_out"]).max()
    assert rel_rms(v, d["vel_out"]) < 1e-5
    p3m.close()
    pm.close()


def test_p3m_full_size_disk(gpu_lib):
    """The 262,144-particle disk + bulge workload (128^3, TSC, S2, cutoff 3H): size-independent
    properties of the cell lists on the whole system, forces on a subsample vs FP64."""
    from particlesimulation_gb300 import workloads as W
    w = W.disk_p3m()
    cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=w.interpolation,
                     finite_diff=w.finite_diff, greens=w.greens, diameter=w.diameter)
    q = O.P3MConfig(comp_box=w.p3m["comp_box"], cutoff=w.p3m["cutoff"], diameter=w.p3m["diameter"],
                    softening=0.0, cloud_shape=1)
    pm, p3m = make_p3m(cfg, q, w.pos, w.vel, w.mass)
    p3m.force()
    acc = pm.getParticles()[2]
    order, counts, dims = p3m.getCellLists()
    # cell lists: a permutation of the particles inside the mesh, grouped by cell, y ascending,
    # ties by index
    xc = (w.pos / np.float32(w.H)).astype(np.float32)
    HC = np.float32(np.float32(w.box[0] / dims[0]) / np.float32(w.H))
    cell = (xc / HC).astype(np.int64)
    flat = cell[:, 0] + cell[:, 1] * dims[0] + cell[:, 2] * dims[0] * dims[1]
    expect = np.lexsort((np.arange(w.n), xc[:, 1], flat))
    np.testing.assert_array_equal(order, expect)
    np.testing.assert_array_equal(counts, np.bincount(flat, minlength=int(np.prod(dims))))
    # forces on a subsample vs FP64 (PM for all + brute-force short range for the targets)
    rng = np.random.default_rng(0)
    idx = np.sort(rng.choice(w.n, 1500, replace=False)).astype(np.int32)
    f64 = O.port_p3m_accel_targets(cfg, q, w.pos, w.vel, w.mass, idx, prec=1)
    assert rel_rms(acc[idx], f64) < 1e-5
    p3m.close()
    pm.close()


def test_p3m_dense_cluster_heavy_units(gpu_lib):
    """A cluster dense enough that some units of the table pass are heavy (taken by whole CTAs,
    their candidate chunks split over the CTA's warps) or medium: forces on a subsample vs the
    FP64 oracle, and two evaluations bit-identical (the warps' partial sums are added in a fixed
    order)."""
    rng = np.random.default_rng(11)
    H = 30.0 / 32
    n = 40000
    pos = np.concatenate([rng.normal(15.0, 0.6, (n // 2, 3)), rng.normal(15.0, 2.5, (n // 4, 3)),
                          rng.uniform(4.0, 26.0, (n - n // 2 - n // 4, 3))])
    pos = np.clip(pos, 4.0, 26.0).astype(np.float32)
    vel = rng.normal(0, 0.01, (n, 3)).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    cfg = O.PMConfig(grid=(32, 32, 32), box=(30.0, 30.0, 30.0), H=H, DT=0.05, G=1.0,
                     interpolation=2, finite_diff=0, greens=2, diameter=3 * H)
    q = O.P3MConfig(comp_box=(30.0, 30.0, 30.0), cutoff=3 * H, diameter=3 * H, softening=0.0,
                    cloud_shape=1)
    pm, p3m = make_p3m(cfg, q, pos, vel, mass)
    p3m.force()
    acc1 = pm.getParticles()[2].copy()
    order, counts, dims = p3m.getCellLists()
    assert counts.max() >= 1024  # units against this cell cost at least the heavy minimum
    p3m.force()
    acc2 = pm.getParticles()[2]
    np.testing.assert_array_equal(acc1, acc2)
    idx = np.sort(rng.choice(n, 1200, replace=False)).astype(np.int32)
    f64 = O.port_p3m_accel_targets(cfg, q, pos, vel, mass, idx, prec=1)
    assert rel_rms(acc1[idx], f64) < 1e-5
    p3m.close()
    pm.close()


def _sym_case(n, table, seed, grid=64, spread=(0.6, 2.5)):
    rng = np.random.default_rng(seed)
    H = 30.0 / (grid // 2)
    pos = np.concatenate([rng.normal(15.0, spread[0], (n // 2, 3)), rng.normal(15.0, spread[1], (n // 4, 3)),
                          rng.uniform(4.0, 26.0, (n - n // 2 - n // 4, 3))])
    pos = np.clip(pos, 4.0, 26.0).astype(np.float32)
    vel = rng.normal(0, 0.01, (n, 3)).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    cfg = O.PMConfig(grid=(grid,) * 3, box=(30.0,) * 3, H=H, DT=0.05, G=1.0,
                     interpolation=2, finite_diff=0, greens=2, diameter=3 * H)
    q = O.P3MConfig(comp_box=(30.0,) * 3, cutoff=3 * H, diameter=3 * H, softening=0.0,
                    cloud_shape=1, use_table=table)
    return cfg, q, pos, vel, mass


@pytest.mark.parametrize("table,n,grid,sub", [(1, 20000, 64, 3), (0, 20000, 64, 3), (1, 40000, 64, 4),
                                              (0, 60000, 64, 4), (1, 60000, 32, 5), (0, 60000, 32, 5)])
def test_symmetric_pass_matches_one_sided(gpu_lib, table, n, grid, sub):
    """The pair pass's symmetric part (light sub-column pairs evaluated once, each side into a
    slot of its own, summed in a fixed order): it takes a large share of the pairs here, its
    forces equal the one-sided pass's to float rounding and the FP64 oracle's within the parity
    bar, and two evaluations are bit-identical (every slot has one writer).  With 3 x 3, 4 x 4
    and 5 x 5 sub-columns per cell (10^3 cells of 20, 40 or 60 particles on average, 5^3 of 480)."""
    from conftest import err_stats
    cfg, q, pos, vel, mass = _sym_case(n, table, seed=21, grid=grid)
    pm, p3m = make_p3m(cfg, q, pos, vel, mass)
    on, _ = p3m.symmetric()
    assert on
    assert p3m.subColumns() == sub
    p3m.force()
    acc_sym = pm.getParticles()[2].copy()
    units = p3m.symmetric()[1]
    assert units > 50, units
    p3m.force()
    np.testing.assert_array_equal(acc_sym, pm.getParticles()[2])
    p3m.setSymmetric(False)
    p3m.force()
    acc_one = pm.getParticles()[2].copy()
    assert p3m.symmetric() == (False, 0)
    st = err_stats(acc_sym, acc_one)
    assert st["rms"] < 1e-6 and st["median"] < 1e-6, st
    rng = np.random.default_rng(5)
    idx = np.sort(rng.choice(len(pos), 1500, replace=False)).astype(np.int32)
    f64 = O.port_p3m_accel_targets(cfg, q, pos, vel, mass, idx, prec=1)
    e_sym, e_one = rel_rms(acc_sym[idx], f64), rel_rms(acc_one[idx], f64)
    if table:
        assert e_sym < 1e-5 and e_one < 1e-5
    else:
        # the exact formula's 1/r^2 on the cluster's close pairs magnifies the float rounding of
        # the positions for both passes alike (the parity bar of the formula is in
        # test_p3m_table_free_force); the symmetric pass must not add to it
        assert e_sym <= 1.01 * e_one + 1e-7, (e_sym, e_one)
    p3m.close()
    pm.close()


@pytest.mark.parametrize("grid,n,ysort,sub", [(64, 20000, 1, 3), (64, 40000, 1, 4), (32, 30000, 1, 5),
                                              (32, 30000, 0, 1)])
def test_subcolumns_per_cell_and_cell_lists(gpu_lib, grid, n, ysort, sub):
    """Sub-columns per cell axis: 5 where the particles average at least 96 per chaining-mesh cell,
    4 from 32, else 3, 1 for the reference's unsorted lists; the cell lists handed out are the
    reference's whole-cell lists either way (vs the oracle's ChainingMesh fill, bit for bit)."""
    cfg, q, pos, vel, mass = _sym_case(n, 1, seed=31, grid=grid)
    q = O.P3MConfig(comp_box=q.comp_box, cutoff=q.cutoff, diameter=q.diameter, softening=0.0,
                    cloud_shape=1, use_table=1, y_sorting=ysort)
    pm, p3m = make_p3m(cfg, q, pos, vel, mass)
    assert p3m.subColumns() == sub
    pc = (pos / np.float32(cfg.H)).astype(np.float32)
    pm.setParticles(pc, np.zeros_like(pc), units="code")  # the same code-unit positions as the oracle's
    p3m.force()
    order, counts, dims = p3m.getCellLists()
    o_ref, c_ref, d_ref = O.port_chaining_mesh(q, cfg.H, pc, ysort)
    assert dims == d_ref
    if ysort:
        nc = int(np.prod(dims))
        assert sub == (5 if n >= 96 * nc else 4 if n >= 32 * nc else 3)
    np.testing.assert_array_equal(counts, c_ref)
    np.testing.assert_array_equal(order, o_ref)
    p3m.close()
    pm.close()


def test_symmetric_pass_run_bit_identical(gpu_lib):
    """A multi-step P3M run with the symmetric part on: repeated runs from the same state give
    bit-identical particles, and the end state stays within float rounding of the one-sided
    run's."""
    cfg, q, pos, vel, mass = _sym_case(30000, 1, seed=23, grid=32, spread=(1.0, 3.0))
    outs = []
    for sym in (True, True, False):
        pm, p3m = make_p3m(cfg, q, pos, vel, mass)
        p3m.setSymmetric(sym)
        escaped, steps = p3m.run(5)
        assert not escaped and steps == 6
        outs.append(pm.getParticles(units="original")[0].copy())
        p3m.close()
        pm.close()
    np.testing.assert_array_equal(outs[0], outs[1])
    assert np.abs(outs[0] - outs[2]).max() < 1e-5 * np.abs(outs[2]).max()


def test_symmetric_pass_only_where_it_applies(gpu_lib):
    """The symmetric part needs equal masses and y-sorted sub-columns: with unequal masses
    the pass lists no symmetric unit (and still matches the FP64 oracle), with unsorted cell
    lists the handle has no symmetric slots at all."""
    cfg, q, pos, vel, mass = _sym_case(20000, 1, seed=27, grid=32)
    rng = np.random.default_rng(28)
    mass = (mass * rng.uniform(0.5, 1.5, len(mass))).astype(np.float32)
    pm, p3m = make_p3m(cfg, q, pos, vel, mass)
    p3m.force()
    assert p3m.symmetric() == (True, 0)
    idx = np.sort(rng.choice(len(pos), 800, replace=False)).astype(np.int32)
    f64 = O.port_p3m_accel_targets(cfg, q, pos, vel, mass, idx, prec=1)
    assert rel_rms(pm.getParticles()[2][idx], f64) < 1e-5
    p3m.close()
    pm.close()
    import particlesimulation_gb300 as P
    cfg, q, pos, vel, mass = _sym_case(20000, 1, seed=27, grid=32)
    pm = make_pm(cfg, pos, vel, mass)
    p3m = P.P3MMethod(pm, q.comp_box, q.cutoff, q.diameter, cfg.H, q.softening,
                      P.CloudShape(q.cloud_shape), True, False)
    p3m.setSymmetric(True)
    p3m.force()
    assert p3m.symmetric() == (False, 0)
    p3m.close()
    pm.close()
