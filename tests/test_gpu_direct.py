"""The FP64 direct sum on the GPU (pmgb_direct_sum_fp64, ppMethod's force restated in double)
against the oracle's CPU FP64 direct sum (oracle/port.cpp port_pp_accel): the yardstick of every
force error report has to be right itself.  Tolerance 1e-12 relative (both FP64, different
summation orders)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("periodic", [0.0, 1.0])
def test_direct_sum_matches_cpu_oracle(gpu_lib, periodic):
    from particlesimulation_gb300 import methods as M
    rng = np.random.default_rng(7)
    n = 20000
    pos = (rng.uniform(0, 1, (n, 3)) if periodic else rng.normal(10, 2, (n, 3))).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, n).astype(np.float32) / n
    idx = np.sort(rng.choice(n, 777, replace=False)).astype(np.int32)
    for eps in (0.0, 0.05):
        got = M.direct_sum_fp64(pos, mass, 1.3, idx, eps=eps, periodic_L=periodic)
        want = O.port_pp_accel(pos.astype(np.float64), mass.astype(np.float64), 1.3, idx=idx,
                               eps=eps, periodic_L=periodic)
        err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
        assert err.max() < 1e-12


def test_direct_sum_rejects_bad_targets(gpu_lib):
    from particlesimulation_gb300 import methods as M
    pos = np.zeros((4, 3), np.float32)
    with pytest.raises(ValueError):
        M.direct_sum_fp64(pos, np.ones(4, np.float32), 1.0, np.array([0, 4], np.int32))
