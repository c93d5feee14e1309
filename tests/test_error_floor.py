"""What sets plain P3M's force error against the Newtonian direct sum (CPU, FP64 oracle).

On the disk + bulge workload (128^3 mesh, H = 60/64, S2 particles, a = cutoff = 3H; 65,536
particles here, same generator as the benchmark's 1,048,576) the median per-particle relative
error of the reference's P3M against an FP64 direct sum is several percent.  Taking the
reference's choices away one at a time, in FP64 so that only the method is measured:

  * the short-range force table (500 entries, linear in r^2 with spacing re^2/499, F(0) = 0;
    source/p3mMethod.cpp:240-245, 275-294) against the exact short-range formula of the same
    reference (shortRangeForce, 220-238, useSRForceTable = false);
  * the TSC stencil centred on the cell below the particle (offsets in [0, 1),
    source/pmMethod.cpp:250-270, 312-331) against the standard TSC centred on the nearest mesh
    point (interpolation = 3 in the oracle port, a deviation from the reference);
  * the 2-point finite difference against the 4-point one.

Each removal lowers the median error; what remains (about 1 % at the full size) is the mesh
force's own anisotropy at r ~ a and the padded (periodic 2L) box's images and background, which
no short-range closure can remove.  So a target of 1e-3 against the direct sum is below the
floor of P3M at this mesh and cutoff."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def disk():
    from particlesimulation_gb300 import workloads as W
    w = W.disk_p3m(n=65536, seed=7)
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(w.n, 1024, replace=False)).astype(np.int32)
    app = O.port_pp_accel(w.pos.astype(np.float64), w.mass.astype(np.float64), w.G, idx=idx)
    return w, idx, app


def _median_err(disk, interpolation, finite_diff, table):
    w, idx, app = disk
    cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=interpolation,
                     finite_diff=finite_diff, greens=2, diameter=3 * w.H)
    q = O.P3MConfig(comp_box=w.p3m["comp_box"], cutoff=3 * w.H, diameter=3 * w.H, softening=0.0,
                    cloud_shape=1, use_table=table, y_sorting=1)
    a = O.port_p3m_accel_targets(cfg, q, w.pos, w.vel, w.mass, idx, prec=1) * (w.H / w.DT ** 2)
    return float(np.median(np.linalg.norm(a - app, axis=1) / np.linalg.norm(app, axis=1)))


def test_error_floor_decomposition(disk):
    e_ref = _median_err(disk, 2, 0, 1)        # the reference's configuration
    e_exact_sr = _median_err(disk, 2, 0, 0)   # exact short-range formula
    e_centred = _median_err(disk, 3, 0, 0)    # + centred TSC
    e_fd4 = _median_err(disk, 3, 1, 0)        # + 4-point difference
    print(f"median relative force error vs FP64 direct sum: reference {e_ref:.4f}, exact SR "
          f"{e_exact_sr:.4f}, + centred TSC {e_centred:.4f}, + 4-point FD {e_fd4:.4f}")
    assert e_exact_sr < 0.9 * e_ref
    assert e_centred < 0.9 * e_exact_sr
    assert e_fd4 < 0.9 * e_centred
    assert e_fd4 > 1e-3  # the floor left is still above a 1e-3 target
