"""The allocation-free cell-list entry point (pmgb_chaining_mesh_fill_noalloc) against the
allocating one (a P3M handle's pmgb_p3m_get_cell_lists).

It serves callers that cannot allocate device memory at the call site: hosts that hand this
library buffers out of their own fixed pool, or step loops that must not call cudaMalloc.  The
caller owns inputs and outputs (here allocated by torch, standing in for such a host); the
entry point itself only uses its fixed scratch arrays.  Cell lists are integer data, so the
comparison is exact, as for the other cell-list tests.  Two calls in a row with different
inputs check that nothing from one call leaks into the next.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _allocating_cell_lists(pos_code, H, comp_box, cutoff, ysort):
    import particlesimulation_gb300 as P
    n = len(pos_code)
    pm = P.PMMethod(np.concatenate([pos_code * np.float32(H), np.zeros_like(pos_code)]),
                    np.full(n, 1.0 / n, np.float32), comp_box, None, H, 0.1, 1.0,
                    P.InterpolationScheme.CIC, P.FiniteDiffScheme.TWO_POINT,
                    P.GreensFunction.DISCRETE_LAPLACIAN, 0.0, (32, 32, 32))
    p3m = P.P3MMethod(pm, comp_box, cutoff, cutoff, H, 0.0, P.CloudShape.S2,
                      enableYSorting=bool(ysort))
    pm.setParticles(pos_code, np.zeros_like(pos_code), units="code")
    p3m.force()
    out = p3m.getCellLists()
    p3m.close()
    pm.close()
    return out


def _noalloc_cell_lists(lib, pos_code, H, comp_box, cutoff, ysort):
    import torch
    from particlesimulation_gb300 import _lib
    cfg = _lib.P3MConfigC()
    cfg.comp_box[:] = list(comp_box)
    cfg.cutoff = cutoff
    cfg.particle_diameter = cutoff
    cfg.cloud_shape = 1
    cfg.use_table = 1
    cfg.y_sorting = ysort
    n = len(pos_code)
    mx = int(np.float32(comp_box[0]) / np.float32(cutoff))
    d_pos = torch.from_numpy(np.ascontiguousarray(pos_code, np.float32)).cuda()
    d_order = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    d_counts = torch.full((mx ** 3,), -7, dtype=torch.int32, device="cuda")
    dims = (C.c_int * 3)()
    torch.cuda.synchronize()
    rc = lib.pmgb_chaining_mesh_fill_noalloc(C.c_void_p(d_pos.data_ptr()), n, C.byref(cfg),
                                             C.c_float(H), C.c_void_p(d_order.data_ptr()),
                                             C.c_void_p(d_counts.data_ptr()), dims, None)
    assert rc == 0, lib.pmgb_last_error()
    torch.cuda.synchronize()
    counts = d_counts.cpu().numpy()
    return d_order.cpu().numpy()[: counts.sum()], counts, (dims[0], dims[1], dims[2])


@pytest.mark.parametrize("ysort", [1, 0])
def test_noalloc_cell_lists_match_allocating_entry_point(gpu_lib, ysort):
    H = 30.0 / 16
    comp_box = (30.0, 30.0, 30.0)
    cutoff = 3 * H
    rng = np.random.default_rng(11)
    inputs = []
    a = rng.uniform(0, 16, (5000, 3)).astype(np.float32)
    a[:300, 1] = np.float32(7.25)  # exact y ties
    inputs.append(a)
    b = np.clip(rng.normal(8, 2.5, (3000, 3)), 0, 15.99).astype(np.float32)
    inputs.append(b)
    for pos in inputs:  # two calls in a row, different sizes and contents
        want = _allocating_cell_lists(pos, H, comp_box, cutoff, ysort)
        got = _noalloc_cell_lists(gpu_lib, pos, H, comp_box, cutoff, ysort)
        assert got[2] == want[2]
        np.testing.assert_array_equal(got[1], want[1])
        np.testing.assert_array_equal(got[0], want[0])


def test_noalloc_rejects_oversized_input(gpu_lib):
    from particlesimulation_gb300 import _lib
    cfg = _lib.P3MConfigC()
    cfg.comp_box[:] = [30.0, 30.0, 30.0]
    cfg.cutoff = 30.0 / 16 * 3
    dims = (C.c_int * 3)()
    rc = gpu_lib.pmgb_chaining_mesh_fill_noalloc(C.c_void_p(16), 262145, C.byref(cfg),
                                                 C.c_float(30.0 / 16), C.c_void_p(16),
                                                 C.c_void_p(16), dims, None)
    assert rc == _lib.PMGB_EINVAL
    assert b"262144" in gpu_lib.pmgb_last_error()
