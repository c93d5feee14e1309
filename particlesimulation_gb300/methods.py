"""Python mirror of the reference's PM / P3M call surface over the C ABI (include/pmgb.h).

Names, argument order and meaning follow the reference (include/pmMethod.h:12-46,
include_gpu/PMMethodGPU.h:12-55, include/p3mMethod.h:11-31, include/pmConfig.h:3-5,
include/greensFunctions.h:7).  The differences are the ones a device path needs: the grid is
given by its point counts (as PMMethodGPU takes it) and the external field is a description
(``SphRadDecrField``) instead of a host callback.  Errors: invalid arguments raise ValueError
(the reference throws std::invalid_argument), device failures raise PMGBError; an escaped
particle stops ``run`` like the reference's loop break and is reported by its return value.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import UNITS_CODE, UNITS_ORIGINAL, check, lib


class InterpolationScheme(enum.IntEnum):
    NGP = 0
    CIC = 1
    TSC = 2


class FiniteDiffScheme(enum.IntEnum):
    TWO_POINT = 0
    FOUR_POINT = 1


class GreensFunction(enum.IntEnum):
    DISCRETE_LAPLACIAN = 0
    S1_OPTIMAL = 1
    S2_OPTIMAL = 2
    POOR_MAN = 3


class CloudShape(enum.IntEnum):
    S1 = 0
    S2 = 1


@dataclass(frozen=True)
class SphRadDecrField:
    """sphRadDecrField(pos, center, R, M, G) (reference source/externalFields.cpp:4-15)."""
    center: tuple
    R: float
    M: float
    G: float


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


class PMMethod:
    """PMMethodGPU(state, masses, effectiveBoxSize, externalField, externalPotential, H, DT, G,
    is, fds, gFunc, particleDiameter, gridPoints) on the GB300 path.  ``state`` holds the N
    positions followed by the N velocities (original units)."""

    def __init__(self, state, masses, effectiveBoxSize, externalField, H, DT, G,
                 interpolation: InterpolationScheme, finiteDiff: FiniteDiffScheme,
                 greensFunction: GreensFunction, particleDiameter, gridPoints,
                 sortInterval: int = 0, periodic: bool = False):
        masses = _f32(masses).reshape(-1)
        n = len(masses)
        state = _f32(state, (2 * n, 3))
        cfg = _lib.PMConfigC()
        cfg.grid[:] = [int(g) for g in gridPoints]
        cfg.box[:] = [float(b) for b in effectiveBoxSize]
        cfg.H, cfg.DT, cfg.G = float(H), float(DT), float(G)
        cfg.interpolation, cfg.finite_diff, cfg.greens = int(interpolation), int(finiteDiff), int(greensFunction)
        cfg.particle_diameter = float(particleDiameter)
        if externalField is not None:
            cfg.ext.kind = 1
            cfg.ext.center[:] = [float(c) for c in externalField.center]
            cfg.ext.R, cfg.ext.M, cfg.ext.G = externalField.R, externalField.M, externalField.G
        cfg.sort_interval = int(sortInterval)
        cfg.periodic = int(bool(periodic))
        self._cfg = cfg
        self.N = n
        self.H, self.DT, self.G = float(H), float(DT), float(G)
        self.gridPoints = tuple(int(g) for g in gridPoints)
        h = C.c_void_p()
        check(lib().pmgb_pm_create(C.byref(cfg), n, _fp(state), _fp(masses), C.byref(h)))
        self._h = h
        self._p3m = None

    # -- lifecycle --
    def close(self):
        if getattr(self, "_h", None):
            if self._p3m is not None:
                self._p3m.close()
            check(lib().pmgb_pm_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- reference surface --
    def getH(self):
        return self.H

    def getDT(self):
        return self.DT

    def getG(self):
        return self.G

    def initGreensFunction(self):
        check(lib().pmgb_pm_init_greens_function(self._h))

    def pmMethodStep(self):
        check(lib().pmgb_pm_method_step(self._h))

    def run(self, simLength: int, collectDiagnostics: bool = False, stateRecorder=None,
            recordField: bool = False):
        """PMMethod::run: returns (escaped, steps_done).  collectDiagnostics records the
        reference's per-iteration diagnostics (read them with ``diagnostics()``); it turns them
        on with room for this run if they are off or too small.  With a ``StateRecorder`` the
        run writes the reference's output files (positions every iteration, the field with
        recordField, energy / momentum lines with collectDiagnostics) and flushes them."""
        if collectDiagnostics:
            self._ensure_diagnostics(int(simLength) + 1)
        done = C.c_int(0)
        if stateRecorder is not None:
            rc = check(lib().pmgb_pm_run_recorded(self._h, stateRecorder._h, int(simLength),
                                                  int(bool(collectDiagnostics)), int(bool(recordField)),
                                                  C.byref(done)))
        else:
            rc = check(lib().pmgb_pm_run(self._h, int(simLength), C.byref(done)))
        return rc == _lib.PMGB_EESCAPED, done.value

    # -- run diagnostics (SimInfo) --
    def setDiagnostics(self, capacity: int):
        """Record up to ``capacity`` diagnostics records during run / advance (0 = off)."""
        check(lib().pmgb_pm_set_diagnostics(self._h, int(capacity)))
        self._diag_cap = int(capacity)

    def _ensure_diagnostics(self, capacity: int):
        if getattr(self, "_diag_cap", 0) < capacity:
            self.setDiagnostics(capacity)

    def diagnostics(self):
        """The records taken so far as a dict of float64 arrays (original units): potential_energy,
        kinetic_energy, momentum (R, 3), angular_momentum (R, 3), expected_momentum (R, 3),
        external_potential_energy; ``records`` is the raw (R, 12) array and ``taken`` the
        number of records taken (more than R if some were dropped for lack of capacity)."""
        cap = getattr(self, "_diag_cap", 0)
        rec = np.zeros((max(cap, 1), _lib.DIAG_WIDTH), np.float64)
        cnt = C.c_int(0)
        check(lib().pmgb_pm_get_diagnostics(self._h, rec.ctypes.data_as(C.POINTER(C.c_double)),
                                            cap, C.byref(cnt)))
        rec = rec[: min(cnt.value, cap)].copy()
        return dict(records=rec, taken=cnt.value, potential_energy=rec[:, 0],
                    kinetic_energy=rec[:, 1], momentum=rec[:, 2:5], angular_momentum=rec[:, 5:8],
                    expected_momentum=rec[:, 8:11], external_potential_energy=rec[:, 11])

    def advance(self, nSteps: int):
        """nSteps more iterations of run()'s loop body (drift, force, kick), continuing from the
        state run() or a previous advance left.  Returns (escaped, steps_done, device_ms)."""
        done = C.c_int(0)
        ms = C.c_float(0)
        rc = check(lib().pmgb_pm_advance(self._h, int(nSteps), C.byref(done), C.byref(ms)))
        return rc == _lib.PMGB_EESCAPED, done.value, ms.value

    def getParticles(self, units: str = "code", pos=None, vel=None, acc=None):
        """(positions, velocities, accelerations), each (N, 3) float32 in original index order.
        Caller-provided (e.g. pinned) float32 output arrays are filled in place."""
        n = self.N
        pos = np.zeros((n, 3), np.float32) if pos is None else pos
        vel = np.zeros((n, 3), np.float32) if vel is None else vel
        acc = np.zeros((n, 3), np.float32) if acc is None else acc
        for a in (pos, vel, acc):
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != 3 * n:
                raise ValueError("output arrays must be contiguous float32 of shape (N, 3)")
        u = UNITS_ORIGINAL if units == "original" else UNITS_CODE
        check(lib().pmgb_pm_get_particles(self._h, _fp(pos), _fp(vel), _fp(acc), u))
        return pos, vel, acc

    def setParticles(self, pos, vel, units: str = "original"):
        n = self.N
        u = UNITS_ORIGINAL if units == "original" else UNITS_CODE
        check(lib().pmgb_pm_set_particles(self._h, _fp(_f32(pos, (n, 3))), _fp(_f32(vel, (n, 3))), u))

    def kernelLaunches(self) -> int:
        """Kernels this process has launched through the library so far."""
        c = C.c_longlong(0)
        check(lib().pmgb_kernel_launches(C.byref(c)))
        return int(c.value)

    def escapedComputationalBox(self) -> bool:
        e = C.c_int(0)
        check(lib().pmgb_pm_escaped(self._h, C.byref(e)))
        return bool(e.value)

    def totalExternalForceOrigUnits(self):
        """PMMethod::totalExternalForceOrigUnits (reference source/pmMethod.cpp:158-162)."""
        f = np.zeros(3, np.float32)
        check(lib().pmgb_pm_total_external_force(self._h, _fp(f)))
        return f

    def getIntegerStepVelocities(self, units: str = "code"):
        """Particle::integerStepVelocity as the last setIntegerStepVelocities(pm) set it."""
        u = np.zeros((self.N, 3), np.float32)
        check(lib().pmgb_pm_get_integer_step_velocities(
            self._h, _fp(u), UNITS_ORIGINAL if units == "original" else UNITS_CODE))
        return u

    def getGridDensity(self):
        nx, ny, nz = self.gridPoints
        d = np.zeros(nx * ny * nz, np.float32)
        check(lib().pmgb_pm_get_density(self._h, _fp(d)))
        return d

    def getGridPotential(self):
        nx, ny, nz = self.gridPoints
        d = np.zeros(nx * ny * nz, np.float32)
        check(lib().pmgb_pm_get_potential(self._h, _fp(d)))
        return d

    def getGreensFunction(self):
        """Influence function as applied: (nz, ny, nx//2+1), symmetrised, times 1/(nx ny nz)."""
        nx, ny, nz = self.gridPoints
        g = np.zeros(nz * ny * (nx // 2 + 1), np.float32)
        check(lib().pmgb_pm_get_greens_function(self._h, _fp(g)))
        return g.reshape(nz, ny, nx // 2 + 1)

    def stageTimes(self):
        t = np.zeros(5, np.float32)
        check(lib().pmgb_pm_stage_times(self._h, _fp(t)))
        return dict(zip(["sort", "deposit", "poisson", "interpolation", "pair"], t.tolist()))

    def stream(self) -> int:
        """The handle's CUDA stream (cudaStream_t as an integer)."""
        s = C.c_void_p()
        check(lib().pmgb_pm_get_stream(self._h, C.byref(s)))
        return int(s.value or 0)


class PlummerSampler:
    """PlummerSampler(seed) (reference include/plummerSampler.h): ``sample(center, a, rMax, M,
    G, n)`` returns the (2n, 3) state (positions, velocities), drawn on the GPU from the
    reference's own random stream; successive calls continue the stream as the reference's
    engine does."""

    def __init__(self, seed: int = 0):
        self.seed = int(seed)
        self.draws = 0

    def sample(self, center, a, rMax, M, G, n: int):
        out = np.zeros((2 * int(n), 3), np.float32)
        c = _f32(center).reshape(3)
        check(lib().pmgb_sample_plummer(C.c_uint(self.seed), C.c_ulonglong(self.draws), _fp(c), a, rMax,
                                        M, G, int(n), _fp(out)))
        self.draws += 6 * int(n)
        return out


class DiskSamplerLinear:
    """DiskSamplerLinear(seed) (reference include/diskSamplerLinear.h): ``sample(center, rb, mb,
    rd, md, thickness, G, n, r0=0)`` as PlummerSampler.sample."""

    def __init__(self, seed: int = 0):
        self.seed = int(seed)
        self.draws = 0

    def sample(self, center, rb, mb, rd, md, thickness, G, n: int, r0: float = 0.0):
        out = np.zeros((2 * int(n), 3), np.float32)
        c = _f32(center).reshape(3)
        check(lib().pmgb_sample_disk_linear(C.c_uint(self.seed), C.c_ulonglong(self.draws), _fp(c), rb, mb,
                                            rd, md, thickness, G, int(n), r0, _fp(out)))
        self.draws += 3 * int(n)
        return out


class StateRecorder:
    """StateRecorder(particlesCnt, framesCnt, outputDirPath, positionsFile, energyFile,
    momentumFile, expectedMomentumFile, angularMomentumFile, fieldFile) (reference
    include/stateRecorder.h:10-21): the reference's output files, written from device frame
    buffers by a host thread.  An empty file name leaves that output out.  ``withField``
    reserves device room for recordField frames."""

    def __init__(self, particlesCnt: int, framesCnt: int, outputDirPath,
                 positionsFile="positions.dat", energyFile="energy.txt",
                 momentumFile="momentum.txt", expectedMomentumFile="expected_momentum.txt",
                 angularMomentumFile="angular_momentum.txt", fieldFile="field.dat",
                 withField: bool = True):
        names = (C.c_char_p * 6)(*[str(x).encode() for x in (
            positionsFile, energyFile, momentumFile, expectedMomentumFile, angularMomentumFile,
            fieldFile)])
        h = C.c_void_p()
        check(lib().pmgb_recorder_create(int(particlesCnt), int(framesCnt), str(outputDirPath).encode(),
                                         names, int(bool(withField)), C.byref(h)))
        self._h = h
        self.outputDirPath = str(outputDirPath)

    def flush(self) -> str:
        buf = C.create_string_buffer(4096)
        check(lib().pmgb_recorder_flush(self._h, buf, 4096))
        return buf.value.decode()

    def framesWritten(self) -> int:
        c = C.c_longlong(0)
        check(lib().pmgb_recorder_frames_written(self._h, C.byref(c)))
        return int(c.value)

    def close(self):
        if getattr(self, "_h", None):
            check(lib().pmgb_recorder_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FFTAdapter:
    """FFTAdapter<float> (reference include/FFTAdapter.h:6-15): 3D complex-to-complex FFT of
    complex64 arrays shaped (nz, ny, nx) (x fastest, the reference's mesh layout), any lengths;
    ``ifft`` is scaled by 1/N like the reference's adapters (source/FFTWAdapter.cpp:34-43).
    ``dims`` is (nz, ny, nx), as the reference passes it to FFTWAdapter / KissFFTAdapter
    (source/demos.cpp:758)."""

    def __init__(self, dims):
        self.dims = tuple(int(d) for d in dims)

    def _run(self, a, inverse, out=None):
        nz, ny, nx = self.dims
        a = np.ascontiguousarray(a, np.complex64).reshape(nz, ny, nx)
        res = np.empty_like(a) if out is None else out
        check(lib().pmgb_fft3d(nx, ny, nz, a.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)),
                               res.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)),
                               1 if inverse else 0))
        return res

    def fft(self, a, out=None):
        return self._run(a, False, out)

    def ifft(self, a, out=None):
        return self._run(a, True, out)


LEAPFROG_HALF_KICK, LEAPFROG_DRIFT, LEAPFROG_KICK, LEAPFROG_INTEGER_STEP = range(4)


def _leapfrog(op, target, dt):
    """A leapfrog operation on a PMMethod's device particles, or on a dict of (N, 3) float32
    arrays {'position', 'velocity', 'acceleration', 'integerStepVelocity'} (updated in place)."""
    if isinstance(target, PMMethod):
        check(lib().pmgb_pm_leapfrog(target._h, op, C.c_float(dt)))
        return target
    arr = {k: _f32(target[k], (-1, 3)) for k in ("position", "velocity", "acceleration")}
    n = len(arr["velocity"])
    u = np.zeros((n, 3), np.float32)
    check(lib().pmgb_leapfrog(op, n, _fp(arr["position"]), _fp(arr["velocity"]),
                              _fp(arr["acceleration"]), _fp(u), C.c_float(dt)))
    target.update(arr)
    if op == LEAPFROG_INTEGER_STEP:
        target["integerStepVelocity"] = u
    return target


def setHalfStepVelocities(particles, dt: float = 1.0):
    """v += 0.5 dt a (reference source/leapfrog.cpp:5-8), on the device."""
    return _leapfrog(LEAPFROG_HALF_KICK, particles, dt)


def setIntegerStepVelocities(particles, dt: float = 1.0):
    """u = v + 0.5 dt a (reference source/leapfrog.cpp:10-15), on the device."""
    return _leapfrog(LEAPFROG_INTEGER_STEP, particles, dt)


def updateVelocities(particles, dt: float = 1.0):
    """v += dt a (reference source/leapfrog.cpp:17-20), on the device."""
    return _leapfrog(LEAPFROG_KICK, particles, dt)


def updatePositions(particles, dt: float = 1.0):
    """x += dt v (reference source/leapfrog.cpp:22-24), on the device."""
    return _leapfrog(LEAPFROG_DRIFT, particles, dt)


def direct_sum_fp64(pos, masses, G, idx, eps=0.0, periodic_L=0.0):
    """FP64 direct-sum accelerations of the targets ``idx`` on the GPU (ppMethod's force,
    reference source/ppMethod.cpp:23-36): (len(idx), 3) float64, same units as the inputs."""
    pos = _f32(pos, (-1, 3))
    m = _f32(masses).reshape(-1)
    idx = np.ascontiguousarray(idx, np.int32).reshape(-1)
    acc = np.zeros((len(idx), 3), np.float64)
    check(lib().pmgb_direct_sum_fp64(len(m), _fp(pos), _fp(m), float(G), float(eps), len(idx),
                                     idx.ctypes.data_as(C.POINTER(C.c_int)), float(periodic_L),
                                     acc.ctypes.data_as(C.POINTER(C.c_double))))
    return acc


def fp32_peak_tflops() -> float:
    """Measured FP32 FMA throughput of the current GPU (TFLOP/s)."""
    t = C.c_float(0)
    check(lib().pmgb_fp32_peak_probe(C.byref(t)))
    return float(t.value)


class P3MMethod:
    """P3MMethod(pm, compBoxSize, cutoffRadius, particleDiameter, H, softeningLength,
    cloudShape, useSRForceTable, enableYSorting) on the GB300 path; borrows ``pm``."""

    def __init__(self, pm: PMMethod, compBoxSize, cutoffRadius, particleDiameter, H,
                 softeningLength, cloudShape: CloudShape, useSRForceTable: bool = True,
                 enableYSorting: bool = True):
        if abs(float(H) - pm.H) > 0:
            raise ValueError("P3MMethod H must equal the PM method's H")
        cfg = _lib.P3MConfigC()
        cfg.comp_box[:] = [float(b) for b in compBoxSize]
        cfg.cutoff = float(cutoffRadius)
        cfg.particle_diameter = float(particleDiameter)
        cfg.softening = float(softeningLength)
        cfg.cloud_shape = int(cloudShape)
        cfg.use_table = int(bool(useSRForceTable))
        cfg.y_sorting = int(bool(enableYSorting))
        h = C.c_void_p()
        check(lib().pmgb_p3m_create(pm._h, C.byref(cfg), C.byref(h)))
        self._h = h
        self.pm = pm
        pm._p3m = self

    def close(self):
        if getattr(self, "_h", None):
            check(lib().pmgb_p3m_destroy(self._h))
            self._h = None
            self.pm._p3m = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def force(self):
        """pmMethodStep + calculateShortRangeForces + correctAccelerations."""
        check(lib().pmgb_p3m_force(self._h))

    def run(self, simLength: int, collectDiagnostics: bool = False, stateRecorder=None,
            recordField: bool = False):
        """P3MMethod::run: returns (escaped, steps_done); diagnostics and recorder as
        PMMethod.run (read the diagnostics with ``pm.diagnostics()``)."""
        if stateRecorder is not None:
            return self.pm.run(simLength, collectDiagnostics, stateRecorder, recordField)
        if collectDiagnostics:
            self.pm._ensure_diagnostics(int(simLength) + 1)
        done = C.c_int(0)
        rc = check(lib().pmgb_p3m_run(self._h, int(simLength), C.byref(done)))
        return rc == _lib.PMGB_EESCAPED, done.value

    def getCellLists(self):
        """(order, counts, (Mx, My, Mz)) of the last force evaluation."""
        dims = (C.c_int * 3)()
        ip = C.POINTER(C.c_int)
        check(lib().pmgb_p3m_get_cell_lists(self._h, ip(), ip(), dims))
        mx, my, mz = dims[0], dims[1], dims[2]
        counts = np.zeros(mx * my * mz, np.int32)
        order = np.zeros(self.pm.N, np.int32)
        check(lib().pmgb_p3m_get_cell_lists(self._h, order.ctypes.data_as(ip),
                                            counts.ctypes.data_as(ip), dims))
        return order[: counts.sum()], counts, (mx, my, mz)

    def advance(self, nSteps: int):
        return self.pm.advance(nSteps)

    def setPairCounting(self, enable: bool):
        check(lib().pmgb_p3m_set_pair_counting(self._h, int(bool(enable))))

    def setSymmetric(self, enable: bool):
        """Evaluate the light sub-column pairs once (on by default where it applies)."""
        check(lib().pmgb_p3m_set_symmetric(self._h, int(bool(enable))))

    def symmetric(self):
        """(switch on, sub-column pairs the last force evaluation took once)."""
        e, u = C.c_int(0), C.c_uint(0)
        check(lib().pmgb_p3m_get_symmetric(self._h, C.byref(e), C.byref(u)))
        return bool(e.value), int(u.value)

    def subColumns(self) -> int:
        """Sub-columns per cell axis of the pair pass (1, or 3 to 5; fixed at creation)."""
        s = C.c_int(0)
        check(lib().pmgb_p3m_get_subcolumns(self._h, C.byref(s)))
        return int(s.value)

    def pairCount(self) -> int:
        """Ordered pairs within the cutoff in the last force evaluation."""
        c = C.c_ulonglong(0)
        check(lib().pmgb_p3m_pair_count(self._h, C.byref(c)))
        return int(c.value)

    def getSRForceTable(self):
        t = np.zeros(500, np.float32)
        d2 = C.c_float(0)
        check(lib().pmgb_p3m_get_sr_table(self._h, _fp(t), C.byref(d2)))
        return t, d2.value


class LearnedClosure:
    """Learned short-range closure over a PM handle (no counterpart in the reference): the
    full-cutoff pair pass of P3M (plain P3M, the judge and fallback) and a reduced-cutoff pair
    pass whose missing residual an MLP predicts (include/pmgb.h, pmgb_closure_*)."""

    FULL, LEARNED, REDUCED_ONLY = 0, 1, 2

    def __init__(self, pm: PMMethod, compBoxSize, cutoffRadius, particleDiameter,
                 softeningLength, cloudShape: CloudShape, reducedCutoff, capacity=0, seed=0,
                 useSRForceTable: bool = True, enableYSorting: bool = True):
        cfg = _lib.P3MConfigC()
        cfg.comp_box[:] = [float(b) for b in compBoxSize]
        cfg.cutoff = float(cutoffRadius)
        cfg.particle_diameter = float(particleDiameter)
        cfg.softening = float(softeningLength)
        cfg.cloud_shape = int(cloudShape)
        cfg.use_table = int(bool(useSRForceTable))
        cfg.y_sorting = int(bool(enableYSorting))
        h = C.c_void_p()
        check(lib().pmgb_closure_create(pm._h, C.byref(cfg), C.c_float(reducedCutoff), int(capacity),
                                        C.c_ulonglong(seed), C.byref(h)))
        self._h = h
        self.pm = pm
        pm._p3m = self

    def close(self):
        if getattr(self, "_h", None):
            check(lib().pmgb_closure_destroy(self._h))
            self._h = None
            self.pm._p3m = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setMode(self, mode: int):
        check(lib().pmgb_closure_set_mode(self._h, int(mode)))

    def mode(self) -> int:
        m = C.c_int(0)
        check(lib().pmgb_closure_get_mode(self._h, C.byref(m)))
        return m.value

    def collect(self, stride: int = 1) -> int:
        total = C.c_int(0)
        check(lib().pmgb_closure_collect(self._h, int(stride), C.byref(total)))
        return total.value

    def train(self, epochs: int, batch: int = 4096, lr: float = 2e-3) -> float:
        loss = C.c_float(0)
        check(lib().pmgb_closure_train(self._h, int(epochs), int(batch), C.c_float(lr), C.byref(loss)))
        return float(loss.value)

    def params(self):
        n = lib().pmgb_closure_param_count()
        p = np.zeros(n, np.float32)
        check(lib().pmgb_closure_get_params(self._h, _fp(p), n))
        return p

    def setParams(self, p):
        p = _f32(p).reshape(-1)
        check(lib().pmgb_closure_set_params(self._h, _fp(p), len(p)))

    def judge(self, stride: int = 1) -> float:
        e = C.c_float(0)
        check(lib().pmgb_closure_judge(self._h, int(stride), C.byref(e)))
        return float(e.value)

    def run(self, nSteps: int, bound: float, judgeInterval: int, judgeStride: int = 1):
        """(escaped, steps_done, fallback_step or -1, device_ms)"""
        done, fb, ms = C.c_int(0), C.c_int(-1), C.c_float(0)
        rc = check(lib().pmgb_closure_run(self._h, int(nSteps), C.c_float(bound), int(judgeInterval),
                                          int(judgeStride), C.byref(done), C.byref(fb), C.byref(ms)))
        return rc == _lib.PMGB_EESCAPED, done.value, fb.value, ms.value

    def force(self):
        check(lib().pmgb_pm_method_step(self.pm._h))

    def features(self):
        n = self.pm.N
        x = np.zeros((n, 67), np.float32)
        s = np.zeros(n, np.float32)
        check(lib().pmgb_closure_features(self._h, _fp(x), _fp(s)))
        return x, s

    def scales(self):
        c = C.c_float(0)
        d = (C.c_int * 3)()
        check(lib().pmgb_closure_scales(self._h, C.byref(c), d))
        return float(c.value), (d[0], d[1], d[2])


class Ensemble:
    """Independent PM systems advanced together, one launch per stage (pmgb_ensemble_*).
    `systems` is a list of dicts with the PMMethod arguments: state, masses, box, H, DT, G,
    interpolation, finite_diff, greens, diameter, grid, periodic (optional)."""

    def __init__(self, systems):
        S = len(systems)
        cfgs = (_lib.PMConfigC * S)()
        counts = (C.c_int * S)()
        self._keep = []
        sp = (C.POINTER(C.c_float) * S)()
        mp = (C.POINTER(C.c_float) * S)()
        self.N = []
        for s, d in enumerate(systems):
            m = _f32(d["masses"]).reshape(-1)
            st = _f32(d["state"], (2 * len(m), 3))
            self._keep += [m, st]
            c = cfgs[s]
            c.grid[:] = [int(g) for g in d["grid"]]
            c.box[:] = [float(b) for b in d["box"]]
            c.H, c.DT, c.G = float(d["H"]), float(d["DT"]), float(d["G"])
            c.interpolation, c.finite_diff, c.greens = int(d["interpolation"]), int(d["finite_diff"]), int(d["greens"])
            c.particle_diameter = float(d.get("diameter", 0.0))
            c.periodic = int(bool(d.get("periodic", False)))
            counts[s] = len(m)
            sp[s] = _fp(st)
            mp[s] = _fp(m)
            self.N.append(len(m))
        h = C.c_void_p()
        check(lib().pmgb_ensemble_create(S, cfgs, counts, sp, mp, C.byref(h)))
        self._h = h
        self.S = S

    def close(self):
        if getattr(self, "_h", None):
            check(lib().pmgb_ensemble_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, simLength: int):
        """(escaped flags per system, device ms)"""
        esc = (C.c_int * self.S)()
        ms = C.c_float(0)
        check(lib().pmgb_ensemble_run(self._h, int(simLength), esc, C.byref(ms)))
        return [bool(e) for e in esc], float(ms.value)

    def advance(self, nSteps: int) -> float:
        ms = C.c_float(0)
        check(lib().pmgb_ensemble_advance(self._h, int(nSteps), C.byref(ms)))
        return float(ms.value)

    def getParticles(self, system: int, units: str = "code"):
        n = self.N[system]
        pos, vel, acc = (np.zeros((n, 3), np.float32) for _ in range(3))
        u = UNITS_ORIGINAL if units == "original" else UNITS_CODE
        check(lib().pmgb_ensemble_get_particles(self._h, int(system), _fp(pos), _fp(vel), _fp(acc), u))
        return pos, vel, acc

    def tuning(self):
        ppt, mult = C.c_int(0), C.c_int(0)
        t = np.zeros(6, np.float32)
        check(lib().pmgb_ensemble_tuning(self._h, C.byref(ppt), C.byref(mult), _fp(t)))
        return {"deposit_particles_per_thread": ppt.value, "x_rows_mult": mult.value,
                "candidate_ms": t.tolist()}


def mlp_param_count() -> int:
    return int(lib().pmgb_closure_param_count())


def mlp_eval(params, x):
    """The closure MLP (our tensor-core kernels) on host inputs x (n, 67) -> (n, 3)."""
    p = _f32(params).reshape(-1)
    x = _f32(x).reshape(-1, 67)
    y = np.zeros((len(x), 3), np.float32)
    check(lib().pmgb_mlp_eval(_fp(p), len(x), _fp(x), _fp(y)))
    return y


def tc_wait_probe(arrive, spins):
    """Status code of the tensor-core kernels' bounded mbarrier wait on a barrier that gets its
    arrival (arrive=True) or never does: PMGB_OK or PMGB_ETIMEOUT (returned, not raised)."""
    return lib().pmgb_tc_wait_probe(1 if arrive else 0, int(spins))


def mlp_gradients(params, x, t):
    """Gradient of mean_rows |MLP(x) - t|^2 w.r.t. the parameters, by our training kernels."""
    p = _f32(params).reshape(-1)
    x = _f32(x).reshape(-1, 67)
    t = _f32(t).reshape(-1, 3)
    g = np.zeros_like(p)
    loss = C.c_float(0)
    check(lib().pmgb_mlp_gradients(_fp(p), len(x), _fp(x), _fp(t), _fp(g), C.byref(loss)))
    return g, float(loss.value)
