"""The random stream of the reference's samplers, modelled in oracle.minstd_uniforms (libstdc++'s
std::default_random_engine = minstd_rand0 through uniform_real_distribution<float>), pinned
against the reference's own DiskSamplerLinear output (golden fixture): the disk's z coordinate
is a pure function of the third number drawn for each particle, so it must match bit for bit."""
import os

import numpy as np

from conftest import GOLDEN
from oracle import oracle as O


def _z(u, cz=15.0, thickness=0.3):
    f = np.float32
    return (f(cz) + (f(thickness) / f(2)) * (f(2) * u - f(1))).astype(np.float32)


def test_minstd_stream_matches_reference_disk_z():
    d = np.load(os.path.join(GOLDEN, "samplers.npz"))
    n = 5000
    u = O.minstd_uniforms(42, 3 * n)
    np.testing.assert_array_equal(_z(u[2::3]), d["disk"][:n, 2])
    # the second half of a 2n sample = a second sample() call: the stream continues
    u2 = O.minstd_uniforms(42, 3 * n, offset=3 * n)
    np.testing.assert_array_equal(_z(u2[2::3]), d["disk_2n"][n:2 * n, 2])
    u7 = O.minstd_uniforms(7, 3 * n)
    np.testing.assert_array_equal(_z(u7[2::3]), d["disk_r0"][:n, 2])
