import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: long-running")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library (built in-tree if missing).  GPU tests fail if it cannot load."""
    from particlesimulation_gb300 import build
    build.build()
    from particlesimulation_gb300 import _lib
    return _lib.lib()


def load_npz(name):
    d = np.load(os.path.join(GOLDEN, name))
    out = {}
    for k in d.files:
        if "/" in k:
            case, key = k.split("/", 1)
            out.setdefault(case, {})[key] = d[k]
        else:
            out[k] = d[k]
    return out


def rel_rms(a, b):
    """RMS over particles of |a - b|, relative to the RMS of |b| (the force-error measure used
    throughout: per-particle relative errors blow up where |F| is tiny)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum(-1).mean() / (b ** 2).sum(-1).mean()))


def err_stats(a, b):
    """Per-particle relative force errors |a - b| / |b|: median and max, next to the
    RMS-normalised figure of rel_rms."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(a - b, axis=-1)
    r = np.linalg.norm(b, axis=-1)
    e = d / np.maximum(r, 1e-300)
    return {"rms": rel_rms(a, b), "median": float(np.median(e)), "max": float(e.max())}
