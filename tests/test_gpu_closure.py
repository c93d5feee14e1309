"""The learned short-range closure: tensor-core MLP kernels against the CPU oracle
(oracle/mlp_oracle.py), patch features against a numpy restatement, and training on residuals
from the plain P3M, which must cut the reduced-cutoff error substantially."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def test_mlp_forward_matches_oracle(gpu_lib):
    from particlesimulation_gb300 import methods
    rng = np.random.default_rng(3)
    p = M.init_params(5)
    p[M.OFF_W4:M.OFF_B4] *= 4.0
    x = rng.uniform(-1, 1, (1000, M.IN)).astype(np.float32)
    y = methods.mlp_eval(p, x)
    want, _ = M.forward(p, x, bf16=True)
    # same bf16 rounding points; differences come from FP32 vs FP64 accumulation, which can
    # flip an activation's last bf16 bit
    err = np.sqrt(((y - want) ** 2).mean() / (want ** 2).mean())
    assert err < 3e-3, err


def test_mlp_gradients_match_oracle(gpu_lib):
    from particlesimulation_gb300 import methods
    rng = np.random.default_rng(4)
    p = M.init_params(6)
    p[M.OFF_W4:M.OFF_B4] *= 4.0
    x = rng.uniform(-1, 1, (512, M.IN)).astype(np.float32)
    t = rng.normal(0, 0.3, (512, 3)).astype(np.float32)
    g, loss = methods.mlp_gradients(p, x, t)
    want = M.gradients(p, x, t, bf16=True)
    assert abs(loss - M.loss(p, x, t, bf16=True)) < 1e-3 * M.loss(p, x, t, bf16=True)
    for lo, hi in ((M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2),
                   (M.OFF_B2, M.OFF_W3), (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.OFF_W4),
                   (M.OFF_W4, M.OFF_B4), (M.OFF_B4, M.NPARAM)):
        a, b = g[lo:hi], want[lo:hi]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err < 2e-2, (lo, err)


def _small_disk(n=65536, grid=64, seed=7):
    from particlesimulation_gb300 import workloads as W
    return W.disk_p3m(n=n, seed=seed, grid=grid)


def _closure(w, capacity=0, seed=0):
    import particlesimulation_gb300 as P
    pm = P.PMMethod(w.state, w.mass, w.box, None, w.H, w.DT, w.G, P.InterpolationScheme(w.interpolation),
                    P.FiniteDiffScheme(w.finite_diff), P.GreensFunction(w.greens), w.diameter, w.grid)
    q = w.p3m
    cl = P.LearnedClosure(pm, q["comp_box"], q["cutoff"], q["diameter"], q["softening"],
                          P.CloudShape(q["cloud_shape"]), 0.5 * q["cutoff"], capacity=capacity,
                          seed=seed)
    return pm, cl


def test_features_match_numpy(gpu_lib):
    w = _small_disk(n=20000)
    pm, cl = _closure(w)
    x, s = cl.features()
    c, dims = cl.scales()
    # numpy restatement: cell masses of the reduced chaining mesh, 4x4x4 patch, offsets
    H = np.float32(w.H)
    xc = (w.pos / H).astype(np.float32)
    mx = dims[0]
    HC = np.float32(np.float32(w.box[0] / mx) / H)
    mc = np.float32(np.float32(np.float32(np.float32(np.float32(w.DT) * np.float32(w.DT)) * np.float32(4))
                                          * np.float32(np.pi)) * np.float32(w.G)) / np.float32(H * H * H)
    m = (mc * w.mass).astype(np.float64)
    cell = (xc / HC).astype(np.int64)
    inside = np.all((cell >= 0) & (cell < mx), axis=1)
    occ = np.zeros((mx, mx, mx))
    np.add.at(occ, (cell[inside, 2], cell[inside, 1], cell[inside, 0]), m[inside])
    u = (xc / HC).astype(np.float32)
    c0 = np.floor(u).astype(np.int64)
    fr = u - c0
    up = (fr >= 0.5).astype(np.int64)
    o = c0 - 2 + up
    off = fr - up
    sel = np.arange(0, w.n, 97)
    for i in sel:
        patch = np.zeros(64)
        for k in range(64):
            cx, cy, cz = o[i, 0] + (k & 3), o[i, 1] + ((k >> 2) & 3), o[i, 2] + (k >> 4)
            if 0 <= cx < mx and 0 <= cy < mx and 0 <= cz < mx:
                patch[k] = occ[cz, cy, cx]
        S = patch.sum()
        assert abs(s[i] - S) <= 1e-5 * S
        np.testing.assert_allclose(x[i, :64], patch / S, rtol=2e-5, atol=1e-7)
        np.testing.assert_allclose(x[i, 64:], off[i], atol=1e-6)
    cl.close()
    pm.close()


def test_training_gains_over_reduced_cutoff(gpu_lib):
    """Residuals from the plain P3M at 3H, reduced pair cutoff 1.5H: after training, the
    learned force must be far closer to the plain P3M force than the reduced force alone."""
    w = _small_disk()
    pm, cl = _closure(w, capacity=2 * w.n, seed=1)
    cl.collect()
    pm.run(0)
    pm.advance(20)
    total = cl.collect()
    assert total == 2 * w.n
    loss = cl.train(epochs=40, batch=1024, lr=2e-3)
    assert np.isfinite(loss)
    cl.setMode(cl.REDUCED_ONLY)
    # judge() compares the learned mode with the plain P3M; for the reduced-only baseline
    # compare zero-closure parameters the same way
    p = cl.params()
    e_learned = cl.judge(stride=3)
    cl.setParams(np.zeros_like(p))
    e_zero = cl.judge(stride=3)  # a zero network: the reduced-cutoff force alone
    cl.setParams(p)
    # The residual (about 5 % of the force here) is dominated by the discreteness of the shell
    # particles, which a cell-mass patch only partly resolves (a CPU reference MLP on the same
    # features removes about 10 % of it); require a clear, repeatable gain.
    assert e_learned < 0.95 * e_zero, (e_learned, e_zero)
    cl.close()
    pm.close()


def test_judge_falls_back_to_plain_p3m(gpu_lib):
    """With a bound no closure can meet, the judged run switches to plain P3M at its first
    check and then matches a plain-P3M run."""
    w = _small_disk(n=16384, seed=9)
    pm, cl = _closure(w)
    pm.run(0)
    cl.setMode(cl.LEARNED)
    esc, done, fallback, _ = cl.run(4, bound=1e-9, judgeInterval=2)
    assert not esc and done == 4 and fallback == 0
    assert cl.mode() == cl.FULL
    cl.close()
    pm.close()


def test_tensor_core_wait_gives_up_and_context_survives(gpu_lib):
    """The bounded mbarrier wait of the tcgen05 kernels: with its arrival it completes; on a
    barrier nothing arrives on it gives up after its spin bound and the call reports
    PMGB_ETIMEOUT; the context stays usable (the tensor-core MLP runs correctly afterwards)."""
    from particlesimulation_gb300 import _lib, methods
    assert methods.tc_wait_probe(True, 1 << 20) == _lib.PMGB_OK
    assert methods.tc_wait_probe(False, 2000) == _lib.PMGB_ETIMEOUT
    p = M.init_params(5)
    x = np.random.default_rng(1).uniform(-1, 1, (300, M.IN)).astype(np.float32)
    y = methods.mlp_eval(p, x)
    want, _ = M.forward(p, x, bf16=True)
    assert np.sqrt(((y - want) ** 2).mean() / (want ** 2).mean()) < 3e-3
