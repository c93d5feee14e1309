"""The stepper surface of the reference (include/leapfrog.h:6-12, source/leapfrog.cpp:5-24) and
PMMethod::totalExternalForceOrigUnits (source/pmMethod.cpp:158-162) through the C ABI.

The leapfrog operations repeat the reference's float arithmetic (0.5f * dt * a, then the add),
so they are compared bit for bit with the same float32 operations in numpy; the external force
is an FP64 sum on the device, compared with numpy's FP64 sum to 1e-6 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

f32 = np.float32


def _ref_op(op, p, v, a, dt):
    dt = f32(dt)
    half = f32(f32(0.5) * dt)
    if op == "half":
        return p, (v + half * a).astype(f32), None
    if op == "drift":
        return (p + dt * v).astype(f32), v, None
    if op == "kick":
        return p, (v + dt * a).astype(f32), None
    return p, v, (v + half * a).astype(f32)


@pytest.mark.parametrize("op", ["half", "drift", "kick", "integer"])
def test_leapfrog_on_host_arrays_bit_exact(gpu_lib, op):
    import particlesimulation_gb300 as P
    rng = np.random.default_rng(5)
    n = 1001
    parts = {k: rng.standard_normal((n, 3)).astype(f32) for k in ("position", "velocity", "acceleration")}
    want = _ref_op(op, parts["position"], parts["velocity"], parts["acceleration"], 0.37)
    fn = {"half": P.setHalfStepVelocities, "drift": P.updatePositions, "kick": P.updateVelocities,
          "integer": P.setIntegerStepVelocities}[op]
    got = fn({k: v.copy() for k, v in parts.items()}, 0.37)
    np.testing.assert_array_equal(got["position"], want[0])
    np.testing.assert_array_equal(got["velocity"], want[1])
    if op == "integer":
        np.testing.assert_array_equal(got["integerStepVelocity"], want[2])


def _pm_with_field(n=3000):
    import particlesimulation_gb300 as P
    rng = np.random.default_rng(9)
    pos = rng.uniform(8, 22, (n, 3)).astype(f32)
    vel = rng.normal(0, 0.01, (n, 3)).astype(f32)
    mass = rng.uniform(0.5, 1.5, n).astype(f32) / n
    ext = P.SphRadDecrField(center=(15.0, 15.0, 15.0), R=3.0, M=0.5, G=1.0)
    pm = P.PMMethod(np.concatenate([pos, vel]), mass, (30.0,) * 3, ext, 30 / 16, 0.1, 1.0,
                    P.InterpolationScheme.CIC, P.FiniteDiffScheme.TWO_POINT,
                    P.GreensFunction.DISCRETE_LAPLACIAN, 0.0, (32, 32, 32))
    return pm, pos, mass, ext


def test_leapfrog_on_handle_state_bit_exact(gpu_lib):
    import particlesimulation_gb300 as P
    pm, _, _, _ = _pm_with_field()
    pm.pmMethodStep()
    x, v, a = pm.getParticles(units="code")
    P.setIntegerStepVelocities(pm)
    np.testing.assert_array_equal(pm.getIntegerStepVelocities(), _ref_op("integer", x, v, a, 1.0)[2])
    P.setHalfStepVelocities(pm)
    x1, v1, _ = pm.getParticles(units="code")
    np.testing.assert_array_equal(v1, _ref_op("half", x, v, a, 1.0)[1])
    P.updatePositions(pm)
    x2, v2, _ = pm.getParticles(units="code")
    np.testing.assert_array_equal(x2, _ref_op("drift", x1, v1, a, 1.0)[0])
    P.updateVelocities(pm, 0.5)
    _, v3, _ = pm.getParticles(units="code")
    np.testing.assert_array_equal(v3, _ref_op("kick", x2, v2, a, 0.5)[1])
    pm.close()


def test_total_external_force(gpu_lib):
    pm, _, mass, ext = _pm_with_field()
    x, _, _ = pm.getParticles(units="original")
    c = np.asarray(ext.center, np.float64)
    d = x.astype(np.float64) - c
    r = np.linalg.norm(d, axis=1)
    GM = ext.G * ext.M
    g = np.where(r > ext.R, -GM / r ** 2, -(GM / ext.R ** 3) * r * (4 - 3 * r / ext.R))
    want = ((mass.astype(np.float64) * g / r)[:, None] * d).sum(0)
    got = pm.totalExternalForceOrigUnits()
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()
    pm.close()
