"""The allocation-free cell-list entry point (pmgb_chaining_mesh_fill_noalloc) against the
allocating one (a P3M handle's pmgb_p3m_get_cell_lists).

It serves callers that cannot allocate device memory at the call site: hosts that hand this
library buffers out of their own fixed pool, or step loops that must not call cudaMalloc.  The
caller owns inputs and outputs (here allocated by torch, standing in for such a host); the
entry point itself only uses its fixed scratch arrays: after the first call on a device the
free device memory is unchanged across a call.  Cell lists are integer data, so the comparison
is exact, as for the other cell-list tests.  Two calls in a row with different inputs check that
nothing from one call leaks into the next.  This file is collected last.
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


def _noalloc_cell_lists(lib, pos_code, H, comp_box, cutoff, ysort, check_free=False):
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
    ncells = int(np.prod([int(np.float32(b) / np.float32(cutoff)) for b in comp_box]))
    d_pos = torch.from_numpy(np.ascontiguousarray(pos_code, np.float32).reshape(-1, 3)).cuda()
    d_order = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    d_counts = torch.full((ncells,), -7, dtype=torch.int32, device="cuda")
    dims = (C.c_int * 3)()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = lib.pmgb_chaining_mesh_fill_noalloc(C.c_void_p(d_pos.data_ptr()), n, C.byref(cfg),
                                             C.c_float(H), C.c_void_p(d_order.data_ptr()),
                                             C.c_void_p(d_counts.data_ptr()), dims, None)
    assert rc == 0, lib.pmgb_last_error()
    torch.cuda.synchronize()
    if check_free:  # after the first call on this device nothing more is allocated
        assert torch.cuda.mem_get_info()[0] == free0
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
    for k, pos in enumerate(inputs):  # two calls in a row, different sizes and contents
        want = _allocating_cell_lists(pos, H, comp_box, cutoff, ysort)
        got = _noalloc_cell_lists(gpu_lib, pos, H, comp_box, cutoff, ysort, check_free=k > 0)
        assert got[2] == want[2]
        np.testing.assert_array_equal(got[1], want[1])
        np.testing.assert_array_equal(got[0], want[0])


def test_noalloc_non_cubic_box_outside_particles_and_empty_input(gpu_lib):
    """A non-cubic box (Mx, My, Mz differ, so the x + y Mx + z Mx My cell index matters), some
    particles outside the chaining mesh (beyond the box, not listed: the counts sum to the
    particles inside), and an empty input (every count 0), each against the allocating entry
    point where it has one."""
    H = 30.0 / 16
    comp_box = (30.0, 22.5, 15.0)
    cutoff = 3 * H
    rng = np.random.default_rng(12)
    pos = rng.uniform(0, 15.9, (4000, 3)).astype(np.float32)
    pos[:, 1] *= np.float32(0.75)
    pos[:, 2] *= np.float32(0.5)
    pos[::37, 0] = np.float32(16.5)   # beyond the box in x (code units, box 16)
    pos[5::41, 2] = np.float32(8.5)   # beyond the box in z (box 8)
    # the first call on a device loads the scratch: make it before the memory checks (this
    # test may run alone in a fresh process)
    _noalloc_cell_lists(gpu_lib, pos[:10], H, comp_box, cutoff, 1)
    for ysort in (1, 0):
        want = _allocating_cell_lists(pos, H, comp_box, cutoff, ysort)
        got = _noalloc_cell_lists(gpu_lib, pos, H, comp_box, cutoff, ysort, check_free=True)
        assert got[2] == want[2] and len(set(got[2])) == 3
        np.testing.assert_array_equal(got[1], want[1])
        np.testing.assert_array_equal(got[0], want[0])
        inside = ((pos[:, 0] < 16) & (pos[:, 1] < 12) & (pos[:, 2] < 8)).sum()
        assert got[1].sum() == inside < len(pos)
    empty = _noalloc_cell_lists(gpu_lib, np.zeros((0, 3), np.float32), H, comp_box, cutoff, 1,
                                check_free=True)
    assert len(empty[0]) == 0 and (empty[1] == 0).all()


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
