"""Seeded synthetic inputs and the run settings of the benchmark / parity workloads.

No dataset is involved anywhere: every workload is generated here from a seed
(numpy PCG64), so the CUDA path, the oracle and the CPU baseline all get identical float32
arrays.  State layout follows the reference's constructors: N positions then N velocities.

  plummer_cluster   PM, 16,384-particle Plummer sphere, 64^3, CIC                (C0)
  disk_p3m          P3M, 262,144-particle exponential disk + Plummer bulge, 128^3,
                    TSC, S2 shapes, cutoff 3 mesh cells                           (C1)
  blobs_periodic    PM, 4,194,304 particles uniform + 64 Gaussian blobs, periodic
                    256^3, CIC                                                    (C2)
  disk_p3m_1m       C1's generator at 1,048,576 particles, exact short-range formula
                    (learned closure)                                             (C4)
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def _iso_dirs(rng, n):
    phi = rng.uniform(0.0, 2 * np.pi, n)
    cth = rng.uniform(-1.0, 1.0, n)
    sth = np.sqrt(1 - cth * cth)
    return np.stack([sth * np.cos(phi), sth * np.sin(phi), cth], axis=1)


def plummer(rng, n, M=1.0, a=1.0, G=1.0, rmax=10.0):
    """Plummer sphere positions (inverse CDF, radius truncated at rmax) and isotropic
    velocities from its distribution function (speed fraction q drawn from
    q^2 (1 - q^2)^(7/2) by rejection), following the reference's PlummerSampler
    (source/plummerSampler.cpp:11-83; it clamps r at rMax, as here)."""
    u = rng.uniform(1e-12, 1.0, n)
    r = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    r = np.minimum(r, rmax)
    pos = r[:, None] * _iso_dirs(rng, n)
    q = np.empty(n)
    todo = np.arange(n)
    while len(todo):
        x = rng.uniform(0, 1, len(todo))
        y = rng.uniform(0, 0.1, len(todo))
        ok = y < x * x * (1 - x * x) ** 3.5
        q[todo[ok]] = x[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2 * G * M / np.sqrt(r * r + a * a))
    vel = (q * vesc)[:, None] * _iso_dirs(rng, n)
    return pos, vel


def disk_bulge(rng, n, M=1.0, G=1.0, rd=3.0, z0=0.3, rb=0.5, fbulge=0.1, rdmax=25.0,
               disp=0.05):
    """Exponential disk (surface density ~ exp(-R/rd), vertical sech^2(z/z0)) holding 1-fbulge
    of the mass plus a Plummer bulge of scale rb; disk particles get the circular velocity of
    the enclosed mass (spherical approximation) plus `disp` Gaussian dispersion per component,
    bulge particles the Plummer distribution function of the bulge."""
    nb = int(round(fbulge * n))
    nd = n - nb
    # disk radius: inverse of 1 - (1 + R/rd) exp(-R/rd) by bisection on a table
    Rt = np.linspace(0, rdmax, 200001)
    cdf = 1 - (1 + Rt / rd) * np.exp(-Rt / rd)
    cdf /= cdf[-1]
    R = np.interp(rng.uniform(0, 1, nd), cdf, Rt)
    ph = rng.uniform(0, 2 * np.pi, nd)
    zu = rng.uniform(-0.999, 0.999, nd)
    z = z0 * np.arctanh(zu)
    pd = np.stack([R * np.cos(ph), R * np.sin(ph), z], axis=1)
    Md, Mb = (1 - fbulge) * M, fbulge * M
    r3 = np.sqrt(R * R + z * z)
    menc = Md * (1 - (1 + R / rd) * np.exp(-R / rd)) + Mb * r3 ** 3 / (r3 * r3 + rb * rb) ** 1.5
    vc = np.sqrt(G * menc / np.maximum(r3, 1e-6))
    vd = np.stack([-vc * np.sin(ph), vc * np.cos(ph), np.zeros(nd)], axis=1)
    vd += disp * vc[:, None] * rng.standard_normal((nd, 3))
    pb, vb = plummer(rng, nb, M=Mb, a=rb, G=G, rmax=10 * rb)
    return np.concatenate([pd, pb]), np.concatenate([vd, vb])


def uniform_blobs(rng, n, nblobs=64, smin=0.01, smax=0.05):
    """Half the particles uniform in [0,1)^3, half in Gaussian blobs (centres uniform, sigma
    log-uniform in [smin, smax]), wrapped periodically; zero initial velocities."""
    nu = n // 2
    nb = n - nu
    pu = rng.uniform(0, 1, (nu, 3))
    centres = rng.uniform(0, 1, (nblobs, 3))
    sig = np.exp(rng.uniform(np.log(smin), np.log(smax), nblobs))
    which = rng.integers(0, nblobs, nb)
    pb = centres[which] + sig[which, None] * rng.standard_normal((nb, 3))
    pos = np.mod(np.concatenate([pu, pb]), 1.0)
    return pos, np.zeros_like(pos)


@dataclass
class Workload:
    """Inputs plus PMMethod / P3MMethod settings (the reference's constructor arguments)."""
    name: str
    pos: np.ndarray
    vel: np.ndarray
    mass: np.ndarray
    grid: tuple
    box: tuple
    H: float
    DT: float
    G: float
    interpolation: int
    finite_diff: int
    greens: int
    diameter: float
    steps: int
    periodic: bool = False
    p3m: dict | None = None  # comp_box, cutoff, diameter, softening, cloud_shape, table, ysort
    extra: dict = field(default_factory=dict)

    @property
    def n(self):
        return len(self.mass)

    @property
    def state(self):
        return np.concatenate([self.pos, self.vel]).astype(np.float32)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def plummer_cluster(n=16384, seed=0, grid=64):
    """C0: Plummer (M=1, a=1, G=1, r <= 10) centred in a side-30 box; mesh of twice the box
    (the reference's isolation by padding, H = 30 / (grid/2)); CIC, 2-point FD, discrete
    Laplacian; dt = 0.01, 100 steps."""
    rng = np.random.default_rng(seed)
    p, v = plummer(rng, n)
    box = 30.0
    return Workload("plummer_cluster", _f32(p + box / 2), _f32(v), _f32(np.full(n, 1.0 / n)),
                    (grid,) * 3, (box,) * 3, box / (grid // 2), 0.01, 1.0, 1, 0, 0, 0.0, 100)


def disk_p3m(n=262144, seed=1, grid=128, cutoff_cells=3.0, table=1):
    """C1: disk + bulge in a side-60 box, mesh 128^3 of twice the box (H = 60/64), TSC,
    S2-optimal influence function with particle diameter = cutoff = 3 H, plain P3M with the
    500-entry table (table = 0: the exact short-range formula, useSRForceTable = false) and
    y-sorted chaining mesh; dt = 0.005, 200 steps."""
    rng = np.random.default_rng(seed)
    p, v = disk_bulge(rng, n)
    box = 60.0
    H = box / (grid // 2)
    a = 3.0 * H
    return Workload("disk_p3m", _f32(p + box / 2), _f32(v), _f32(np.full(n, 1.0 / n)),
                    (grid,) * 3, (box,) * 3, H, 0.005, 1.0, 2, 0, 2, a, 200,
                    p3m=dict(comp_box=(box,) * 3, cutoff=cutoff_cells * H, diameter=a,
                             softening=0.0, cloud_shape=1, table=table, ysort=1))


def blobs_periodic(n=4194304, seed=2, grid=256):
    """C2: uniform + 64 Gaussian blobs in the periodic unit cube, 256^3 mesh (H = 1/256), CIC,
    2-point FD, discrete Laplacian, total mass 1, G = 1; dt = 1e-3, 50 steps."""
    rng = np.random.default_rng(seed)
    p, v = uniform_blobs(rng, n)
    return Workload("blobs_periodic", _f32(p), _f32(v), _f32(np.full(n, 1.0 / n)),
                    (grid,) * 3, (1.0,) * 3, 1.0 / grid, 1e-3, 1.0, 1, 0, 0, 0.0, 50,
                    periodic=True)


def disk_p3m_1m(n=1048576, seed=4, grid=128, cutoff_cells=3.0, table=0):
    """C4: C1's generator at 1,048,576 particles, the learned closure's workload.  By default
    with the exact short-range formula (the reference's useSRForceTable = false): the 500-entry
    table's error on close pairs (F(0) = 0, linear in r^2) sits in every residual the closure
    is trained on and is larger than the closure's own error; table = 1 keeps the table."""
    w = disk_p3m(n=n, seed=seed, grid=grid, cutoff_cells=cutoff_cells, table=table)
    w.name = "disk_p3m_1m"
    return w


def plummer_ensemble(n_systems=64, seed=3, nmin=4096, nmax=131072, steps=100):
    """C3: independent Plummer systems as plummer_cluster (M=1, a=1, G=1, r <= 10, box 30,
    CIC, 2-point, discrete Laplacian, dt 0.01), N log-uniform in [nmin, nmax], mesh the power of
    two in {32, 64, 128} nearest to 2 N^(1/3); returns a list of Workloads."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_systems):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        target = 2.0 * n ** (1.0 / 3.0)
        grid = min((32, 64, 128), key=lambda g: abs(np.log2(g) - np.log2(target)))
        w = plummer_cluster(n=n, seed=int(rng.integers(1 << 31)), grid=grid)
        w.name = f"plummer_ensemble[{s}]"
        w.steps = steps
        out.append(w)
    return out


def as_system(w: Workload) -> dict:
    """PMMethod arguments of a workload, as particlesimulation_gb300.methods.Ensemble takes them."""
    return dict(state=w.state, masses=w.mass, box=w.box, H=w.H, DT=w.DT, G=w.G,
                interpolation=w.interpolation, finite_diff=w.finite_diff, greens=w.greens,
                diameter=w.diameter, grid=w.grid, periodic=w.periodic)


WORKLOADS = {
    "plummer_cluster": plummer_cluster,
    "disk_p3m": disk_p3m,
    "blobs_periodic": blobs_periodic,
    "disk_p3m_1m": disk_p3m_1m,
}
