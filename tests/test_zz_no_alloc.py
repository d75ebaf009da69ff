"""amr_copy_boundaries_noalloc: the ghost fill for callers that cannot let the library allocate.

Such callers (an application that owns a fixed device-memory budget, or a time-critical loop
that must not block on cudaMalloc) get the same ghost fill as amr_copy_boundaries, staged in a
fixed array compiled into the library instead of an allocated buffer.  This test calls it through
the C ABI and checks it against amr_copy_boundaries bit for bit (the tolerance the ghost-fill tests
use), on two calls in a row, so the second call runs on an array that still holds the first
call's contents.  It lives in its own file, collected last, and needs nothing from other tests.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _case(am, n, p, tree):
    import torch
    o = am.Octree(64)
    cases.TREES[tree](o)
    st = o.state()
    used = st["used_slots"]
    xyz = cases.cell_coordinates(st["positions"], used, n, p, 100.0)
    f_old = cases.smooth_field(xyz, 100.0, 1, 11)
    f_new = cases.smooth_field(xyz, 100.0, 1, 12)
    bd = torch.from_numpy(st["boundaries"][: used * 6].view(np.int64)).cuda()
    return st, used, f_old, f_new, bd


@pytest.mark.parametrize("n,p,tree", [(16, 3, "uneven"), (28, 2, "bssn")])
def test_noalloc_ghost_fill_matches_allocating_entry_point(am, cuda, n, p, tree):
    import torch
    lib = am.load()
    cfg = am.Config(n, p, 100.0)
    st, used, f_old, f_new, bd = _case(am, n, p, tree)
    md = st["max_depth"]
    # two calls in a row with different substeps and modes
    for substep, only_new in ((0, 0), ((1 << md) - 1, 1)):
        a_old, a_new = torch.from_numpy(f_old).cuda(), torch.from_numpy(f_new).cuda()
        b_old, b_new = torch.from_numpy(f_old).cuda(), torch.from_numpy(f_new).cuda()
        assert lib.amr_copy_boundaries(ctypes.byref(cfg), a_old.data_ptr(), a_new.data_ptr(), bd.data_ptr(), used,
                                       substep, md, only_new, None) == 0
        assert lib.amr_copy_boundaries_noalloc(ctypes.byref(cfg), b_old.data_ptr(), b_new.data_ptr(), bd.data_ptr(),
                                               used, substep, md, only_new, None) == 0
        torch.cuda.synchronize()
        for a, b in ((a_old, b_old), (a_new, b_new)):
            x, y = a.cpu().numpy(), b.cpu().numpy()
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
        assert not np.array_equal(a_new.cpu().numpy(), f_new) or substep != 0


def test_noalloc_rejects_cases_beyond_its_array(am, cuda):
    import torch
    lib = am.load()
    cfg = am.Config(16, 3, 100.0)
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    bd = torch.zeros(16, dtype=torch.int64, device="cuda")
    # 1366 slots of 16^3 stage 1366 * 2 * 3 * 16^2 floats, more than the array's 2^21: rejected
    # before anything is launched (the dummy buffers are never touched)
    assert lib.amr_copy_boundaries_noalloc(ctypes.byref(cfg), dummy.data_ptr(), dummy.data_ptr(), bd.data_ptr(), 1366,
                                           0, 3, 1, None) == am.ERR_CAPACITY
    assert lib.amr_copy_boundaries_noalloc(None, dummy.data_ptr(), dummy.data_ptr(), bd.data_ptr(), 1, 0, 0, 1,
                                           None) == am.ERR_INVALID
