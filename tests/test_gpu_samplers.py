"""GPU samplers against the reference's PlummerSampler / DiskSamplerLinear output (golden
fixture tests/golden/samplers.npz).  The random stream is the reference's, so each particle is
the reference's particle: positions and velocities agree to float rounding of the libm
functions (relative 1e-5 for 99.9 % of the particles, 1e-3 for all: the velocity of a Plummer
particle comes from a Newton solve stopped at |dx| <= 1e-3, where one extra or missing iteration
on either side moves the result by at most the square of that step); a second sample() call
continues the stream exactly as a single call of twice the size."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

S = np.load(os.path.join(GOLDEN, "samplers.npz"))


def _close(a, b):
    scale = np.maximum(np.abs(b), 1e-3 * np.abs(b).max(axis=0))
    rel = (np.abs(a - b) / scale).max(axis=1)
    assert np.quantile(rel, 0.999) < 1e-5, np.quantile(rel, 0.999)
    assert rel.max() < 1e-3, rel.max()


def test_plummer_matches_reference(gpu_lib):
    import particlesimulation_gb300 as P
    s = P.PlummerSampler(42).sample((30, 30, 30), 2.0, 15.0, 1.0, 4.5e-3, 5000)
    _close(s[:5000], S["plummer"][:5000])
    _close(s[5000:], S["plummer"][5000:])


def test_disk_linear_matches_reference(gpu_lib):
    import particlesimulation_gb300 as P
    n = 5000
    s = P.DiskSamplerLinear(42).sample((30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, n)
    _close(s, S["disk"])
    s7 = P.DiskSamplerLinear(7).sample((30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, n, 3.0)
    _close(s7, S["disk_r0"])


def test_second_call_continues_the_stream(gpu_lib):
    import particlesimulation_gb300 as P
    n = 5000
    smp = P.DiskSamplerLinear(42)
    a = smp.sample((30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, n)
    b = smp.sample((30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, n)
    both = P.DiskSamplerLinear(42).sample((30, 30, 15), 3.0, 60.0, 15.0, 15.0, 0.3, 4.5e-3, 2 * n)
    np.testing.assert_array_equal(np.concatenate([a[:n], b[:n]]), both[:2 * n])
    np.testing.assert_array_equal(np.concatenate([a[n:], b[n:]]), both[2 * n:])
    _close(both, S["disk_2n"])
    p = P.PlummerSampler(3)
    big = p.sample((0, 0, 0), 1.0, 10.0, 1.0, 1.0, 1_000_000)  # large N on the device
    assert np.isfinite(big).all() and np.abs(big[:1_000_000]).max() <= 10.0 + 1e-4
