"""ctypes front-end of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Loads ``oracle/_build/liboracle.so`` (the port, ``port_*``) and, when it was built,
``oracle/_ref/libpsref.so`` (the reference's own CPU code, ``ref_*``).  Both are declared in
``oracle/oracle_api.h``.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
legs import this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpsref.so")


class PMParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("box_x", C.c_float), ("box_y", C.c_float), ("box_z", C.c_float),
        ("H", C.c_float), ("DT", C.c_float), ("G", C.c_float),
        ("is_", C.c_int), ("fds", C.c_int), ("gf", C.c_int),
        ("diameter", C.c_float),
        ("ext_kind", C.c_int),
        ("ext_cx", C.c_float), ("ext_cy", C.c_float), ("ext_cz", C.c_float),
        ("ext_R", C.c_float), ("ext_M", C.c_float), ("ext_G", C.c_float),
        ("periodic", C.c_int),
    ]


class P3MParams(C.Structure):
    _fields_ = [
        ("comp_x", C.c_float), ("comp_y", C.c_float), ("comp_z", C.c_float),
        ("cutoff", C.c_float), ("diameter", C.c_float), ("softening", C.c_float),
        ("cloud_shape", C.c_int), ("use_table", C.c_int), ("y_sorting", C.c_int),
    ]


@dataclass
class PMConfig:
    """Arguments of the reference's PMMethod constructor plus the grid size."""
    grid: tuple = (32, 32, 32)
    box: tuple = (30.0, 30.0, 30.0)
    H: float = 30.0 / 16
    DT: float = 1.0
    G: float = 1.0
    interpolation: int = 1   # 0 NGP, 1 CIC, 2 TSC
    finite_diff: int = 0     # 0 TWO_POINT, 1 FOUR_POINT
    greens: int = 0          # 0 DISCRETE_LAPLACIAN, 1 S1_OPTIMAL, 2 S2_OPTIMAL, 3 POOR_MAN
    diameter: float = 0.0
    ext: tuple = ()          # () or (cx, cy, cz, R, M, G) for sphRadDecrField
    periodic: int = 0

    def c(self) -> PMParams:
        p = PMParams()
        p.nx, p.ny, p.nz = self.grid
        p.box_x, p.box_y, p.box_z = self.box
        p.H, p.DT, p.G = self.H, self.DT, self.G
        p.is_, p.fds, p.gf = self.interpolation, self.finite_diff, self.greens
        p.diameter = self.diameter
        if self.ext:
            p.ext_kind = 1
            p.ext_cx, p.ext_cy, p.ext_cz, p.ext_R, p.ext_M, p.ext_G = self.ext
        p.periodic = self.periodic
        return p


@dataclass
class P3MConfig:
    """Arguments of the reference's P3MMethod constructor."""
    comp_box: tuple = (30.0, 30.0, 30.0)
    cutoff: float = 3.0
    diameter: float = 3.0
    softening: float = 0.0
    cloud_shape: int = 1     # 0 S1, 1 S2
    use_table: int = 1
    y_sorting: int = 1

    def c(self) -> P3MParams:
        q = P3MParams()
        q.comp_x, q.comp_y, q.comp_z = self.comp_box
        q.cutoff, q.diameter, q.softening = self.cutoff, self.diameter, self.softening
        q.cloud_shape, q.use_table, q.y_sorting = self.cloud_shape, self.use_table, self.y_sorting
        return q


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def build_port() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def build_ref() -> bool:
    """Compile the reference CPU path from its sources (the checkout named by the PSIM_REFERENCE
    environment variable); False where it is not set or the sources are absent."""
    ref = os.environ.get("PSIM_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "source")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={ref}"], check=True)
    return True


_port = None
_ref = None


def port() -> C.CDLL:
    global _port
    if _port is None:
        build_port()  # incremental (make)
        _port = C.CDLL(PORT_SO)
    return _port


def ref_available() -> bool:
    if not os.path.exists(REF_SO):
        return False
    try:
        ref()
        return True
    except OSError:
        return False


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_SO)
    return _ref


def _state(pos, vel):
    return _f32(np.concatenate([np.asarray(pos).reshape(-1, 3), np.asarray(vel).reshape(-1, 3)]))


# ---------------------------------------------------------------- reference ---
def ref_pm_accel(cfg: PMConfig, pos, vel, mass, want_mesh=False):
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    acc = np.zeros((n, 3), np.float32)
    L = int(np.prod(cfg.grid))
    dens = np.zeros(L, np.float32) if want_mesh else None
    pot = np.zeros(L, np.float32) if want_mesh else None
    grn = np.zeros(L, np.float32) if want_mesh else None
    fp = C.POINTER(C.c_float)
    rc = ref().ref_pm_accel(C.byref(cfg.c()), n, _ptr(st, C.c_float), _ptr(m, C.c_float),
                            _ptr(acc, C.c_float),
                            _ptr(dens, C.c_float) if want_mesh else fp(),
                            _ptr(pot, C.c_float) if want_mesh else fp(),
                            _ptr(grn, C.c_float) if want_mesh else fp())
    assert rc == 0
    return (acc, dens, pot, grn) if want_mesh else acc


def ref_p3m_accel(cfg: PMConfig, q: P3MConfig, pos, vel, mass):
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    acc = np.zeros((n, 3), np.float32)
    rc = ref().ref_p3m_accel(C.byref(cfg.c()), C.byref(q.c()), n, _ptr(st, C.c_float),
                             _ptr(m, C.c_float), _ptr(acc, C.c_float))
    assert rc == 0
    return acc


def _read_ref_diagnostics(d):
    """The text files StateRecorder writes with collectDiagnostics (reference
    source/stateRecorder.cpp:63-107) as an (R, 12) array in the PMGB_DIAG_* layout; column 11
    (the external part of the potential energy) is not recorded by the reference: NaN."""
    def load(name, cols):
        a = np.loadtxt(os.path.join(d, name), ndmin=2)
        return a.reshape(-1, cols)
    e = load("energy.txt", 2)
    p = load("momentum.txt", 3)
    la = load("angular_momentum.txt", 3)
    pe = load("expected_momentum.txt", 3)
    out = np.full((len(e), 12), np.nan)
    out[:, 0:2] = e
    out[:, 2:5] = p
    out[:, 5:8] = la
    out[:, 8:11] = pe
    return out


def ref_run(cfg: PMConfig, q: P3MConfig | None, pos, vel, mass, sim_length, diagnostics=False):
    """PMMethod::run / P3MMethod::run of the compiled reference; with diagnostics=True also
    returns the recorded energy / momentum records (see _read_ref_diagnostics)."""
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    out = np.zeros((2 * n, 3), np.float32)
    esc = C.c_int(0)
    diag = None
    with tempfile.TemporaryDirectory() as d:
        if q is None:
            rc = ref().ref_pm_run(C.byref(cfg.c()), n, _ptr(st, C.c_float), _ptr(m, C.c_float),
                                  sim_length, d.encode(), _ptr(out, C.c_float), C.byref(esc),
                                  int(diagnostics))
        else:
            rc = ref().ref_p3m_run(C.byref(cfg.c()), C.byref(q.c()), n, _ptr(st, C.c_float),
                                   _ptr(m, C.c_float), sim_length, d.encode(),
                                   _ptr(out, C.c_float), C.byref(esc), int(diagnostics))
        if rc == 0 and diagnostics:
            diag = _read_ref_diagnostics(d)
    assert rc == 0
    if diagnostics:
        return out[:n], out[n:], bool(esc.value), diag
    return out[:n], out[n:], bool(esc.value)


def ref_run_files(cfg: PMConfig, q: P3MConfig | None, pos, vel, mass, sim_length, outdir,
                  diagnostics=False, record_field=False):
    """run(StateRecorder(outdir), sim_length, diagnostics, record_field) of the compiled
    reference, leaving its output files in outdir; returns (escaped, {file name: bytes})."""
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    out = np.zeros((2 * n, 3), np.float32)
    esc = C.c_int(0)
    flags = (1 if diagnostics else 0) | (2 if record_field else 0)
    if q is None:
        rc = ref().ref_pm_run(C.byref(cfg.c()), n, _ptr(st, C.c_float), _ptr(m, C.c_float),
                              sim_length, outdir.encode(), _ptr(out, C.c_float), C.byref(esc), flags)
    else:
        rc = ref().ref_p3m_run(C.byref(cfg.c()), C.byref(q.c()), n, _ptr(st, C.c_float),
                               _ptr(m, C.c_float), sim_length, outdir.encode(),
                               _ptr(out, C.c_float), C.byref(esc), flags)
    assert rc == 0
    files = {}
    for name in sorted(os.listdir(outdir)):
        with open(os.path.join(outdir, name), "rb") as f:
            files[name] = f.read()
    return bool(esc.value), files


def ref_chaining_mesh(q: P3MConfig, H, pos_code, y_sorting=1):
    n = len(pos_code)
    pc = _f32(pos_code)
    dims = np.zeros(3, np.int32)
    ref().ref_chaining_mesh(C.byref(q.c()), C.c_float(H), n, _ptr(pc, C.c_float), y_sorting,
                            C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), _ptr(dims, C.c_int))
    order = np.zeros(n, np.int32)
    counts = np.zeros(int(np.prod(dims)), np.int32)
    ref().ref_chaining_mesh(C.byref(q.c()), C.c_float(H), n, _ptr(pc, C.c_float), y_sorting,
                            _ptr(order, C.c_int), _ptr(counts, C.c_int), _ptr(dims, C.c_int))
    return order[: counts.sum()], counts, tuple(int(d) for d in dims)


def ref_pp_accel(pos, mass, G, eps=0.0):
    n = len(mass)
    p, m = _f32(pos), _f32(mass)
    acc = np.zeros((n, 3), np.float32)
    ref().ref_pp_accel(n, _ptr(p, C.c_float), _ptr(m, C.c_float), C.c_float(G), C.c_float(eps),
                       _ptr(acc, C.c_float))
    return acc


def ref_sr_table(q: P3MConfig, H):
    t = np.zeros(500, np.float32)
    d2 = C.c_float(0)
    ref().ref_sr_table(C.byref(q.c()), C.c_float(H), _ptr(t, C.c_float), C.byref(d2))
    return t, d2.value


# --------------------------------------------------------------------- port ---
def port_pm_accel(cfg: PMConfig, pos, vel, mass, prec=1, want_mesh=False):
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    acc = np.zeros((n, 3), np.float64)
    L = int(np.prod(cfg.grid))
    dp = C.POINTER(C.c_double)
    dens = np.zeros(L) if want_mesh else None
    pot = np.zeros(L) if want_mesh else None
    grn = np.zeros(L) if want_mesh else None
    rc = port().port_pm_accel(prec, C.byref(cfg.c()), n, _ptr(st, C.c_float), _ptr(m, C.c_float),
                              _ptr(acc, C.c_double),
                              _ptr(dens, C.c_double) if want_mesh else dp(),
                              _ptr(pot, C.c_double) if want_mesh else dp(),
                              _ptr(grn, C.c_double) if want_mesh else dp())
    assert rc == 0
    return (acc, dens, pot, grn) if want_mesh else acc


def port_p3m_accel(cfg: PMConfig, q: P3MConfig, pos, vel, mass, prec=1, nthreads=None,
                   want_sr=False):
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    acc = np.zeros((n, 3), np.float64)
    sr = np.zeros((n, 3), np.float64)
    rc = port().port_p3m_accel(prec, C.byref(cfg.c()), C.byref(q.c()), n, _ptr(st, C.c_float),
                               _ptr(m, C.c_float), _ptr(acc, C.c_double), _ptr(sr, C.c_double),
                               nthreads or os.cpu_count())
    assert rc == 0
    return (acc, sr) if want_sr else acc


def port_run(cfg: PMConfig, q: P3MConfig | None, pos, vel, mass, sim_length, prec=1,
             nthreads=None, diagnostics=False):
    """The port's run loop; with diagnostics=True also returns the (R, 12) FP64 records of the
    reference's collectDiagnostics (layout of include/pmgb.h's PMGB_DIAG_*)."""
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    out = np.zeros((2 * n, 3), np.float64)
    esc = C.c_int(0)
    cap = sim_length + 1 if diagnostics else 0
    diag = np.zeros((max(cap, 1), 12), np.float64)
    cnt = C.c_int(0)
    dptr = _ptr(diag, C.c_double) if diagnostics else C.POINTER(C.c_double)()
    if q is None:
        rc = port().port_pm_run(prec, C.byref(cfg.c()), n, _ptr(st, C.c_float), _ptr(m, C.c_float),
                                sim_length, _ptr(out, C.c_double), C.byref(esc), dptr, cap,
                                C.byref(cnt))
    else:
        rc = port().port_p3m_run(prec, C.byref(cfg.c()), C.byref(q.c()), n, _ptr(st, C.c_float),
                                 _ptr(m, C.c_float), sim_length, _ptr(out, C.c_double),
                                 C.byref(esc), nthreads or os.cpu_count(), dptr, cap, C.byref(cnt))
    assert rc == 0
    if diagnostics:
        return out[:n], out[n:], bool(esc.value), diag[: min(cnt.value, cap)].copy()
    return out[:n], out[n:], bool(esc.value)


def port_chaining_mesh(q: P3MConfig, H, pos_code, y_sorting=1):
    n = len(pos_code)
    pc = _f32(pos_code)
    dims = np.zeros(3, np.int32)
    port().port_chaining_mesh(C.byref(q.c()), C.c_float(H), n, _ptr(pc, C.c_float), y_sorting,
                              C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), _ptr(dims, C.c_int))
    order = np.zeros(n, np.int32)
    counts = np.zeros(int(np.prod(dims)), np.int32)
    port().port_chaining_mesh(C.byref(q.c()), C.c_float(H), n, _ptr(pc, C.c_float), y_sorting,
                              _ptr(order, C.c_int), _ptr(counts, C.c_int), _ptr(dims, C.c_int))
    return order[: counts.sum()], counts, tuple(int(d) for d in dims)


def port_pp_accel(pos, mass, G, idx=None, eps=0.0, periodic_L=0.0, nthreads=None):
    """FP64 direct sum on the targets ``idx`` (all particles if None)."""
    p = np.ascontiguousarray(pos, np.float64)
    m = np.ascontiguousarray(mass, np.float64)
    n = len(m)
    idx = np.arange(n, dtype=np.int32) if idx is None else np.ascontiguousarray(idx, np.int32)
    acc = np.zeros((len(idx), 3), np.float64)
    port().port_pp_accel(n, _ptr(p, C.c_double), _ptr(m, C.c_double), C.c_double(G),
                         C.c_double(eps), len(idx), _ptr(idx, C.c_int), C.c_double(periodic_L),
                         _ptr(acc, C.c_double), nthreads or os.cpu_count())
    return acc


def port_p3m_accel_targets(cfg: PMConfig, q: P3MConfig, pos, vel, mass, idx, prec=1,
                           nthreads=None):
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    idx = np.ascontiguousarray(idx, np.int32)
    acc = np.zeros((len(idx), 3), np.float64)
    rc = port().port_p3m_accel_targets(prec, C.byref(cfg.c()), C.byref(q.c()), n,
                                       _ptr(st, C.c_float), _ptr(m, C.c_float), len(idx),
                                       _ptr(idx, C.c_int), _ptr(acc, C.c_double),
                                       nthreads or os.cpu_count())
    assert rc == 0
    return acc


def port_sr_table(q: P3MConfig, H):
    t = np.zeros(500, np.float32)
    d2 = C.c_float(0)
    port().port_sr_table(C.byref(q.c()), C.c_float(H), _ptr(t, C.c_float), C.byref(d2))
    return t, d2.value


def port_time_steps(cfg: PMConfig, q: P3MConfig | None, pos, vel, mass, steps, nthreads,
                    pair_stride=1, fill_stride=1):
    """Seconds per step of the port in float: dict(est, pm, cells, pair_sampled, wall).

    pair_stride S: only every S-th particle (by index) is an i-particle of the pair pass (its
    time is scaled by S in ``est``); fill_stride F: the reference's y-sorting insertion sort runs
    on every F-th particle and its time is scaled by F^2 (``cells`` is the scaled figure).
    ``wall`` is the time the sampled steps actually took, per step."""
    n = len(mass)
    st, m = _state(pos, vel), _f32(mass)
    out = np.zeros(4, np.float64)
    wall = C.c_double(0)
    rc = port().port_time_steps2(C.byref(cfg.c()), C.byref(q.c()) if q is not None else None, n,
                                 _ptr(st, C.c_float), _ptr(m, C.c_float), steps, nthreads,
                                 pair_stride, fill_stride, _ptr(out, C.c_double), C.byref(wall))
    assert rc == 0
    return dict(est=out[0], pm=out[1], cells=out[2], pair_sampled=out[3],
                wall=wall.value / max(steps, 1))


# ----------------------------------------------------------------- samplers ---
def ref_sample_plummer(seed, center, a, r_max, M, G, n):
    out = np.zeros((2 * n, 3), np.float32)
    c = _f32(center)
    ref().ref_sample_plummer(C.c_uint(seed), _ptr(c, C.c_float), C.c_float(a), C.c_float(r_max),
                             C.c_float(M), C.c_float(G), n, _ptr(out, C.c_float))
    return out


def ref_sample_disk_linear(seed, center, rb, mb, rd, md, thickness, G, n, r0=0.0):
    out = np.zeros((2 * n, 3), np.float32)
    c = _f32(center)
    ref().ref_sample_disk_linear(C.c_uint(seed), _ptr(c, C.c_float), C.c_float(rb), C.c_float(mb),
                                 C.c_float(rd), C.c_float(md), C.c_float(thickness), C.c_float(G), n,
                                 C.c_float(r0), _ptr(out, C.c_float))
    return out


def minstd_uniforms(seed, count, offset=0):
    """The float uniforms std::uniform_real_distribution<float>(0, 1) draws from
    std::default_random_engine(seed) in libstdc++ (minstd_rand0; generate_canonical<float, 24>
    takes one engine value per number): u = float(x - 1) / float(2^31 - 2), below 1."""
    m, a = 2147483647, 16807
    x = seed % m or 1
    x = x * pow(a, offset, m) % m
    out = np.empty(count, np.float32)
    for k in range(count):
        x = x * a % m
        u = np.float32(np.float32(x - 1) / np.float32(2147483646.0))
        out[k] = u if u < 1 else np.nextafter(np.float32(1), np.float32(0))
    return out
