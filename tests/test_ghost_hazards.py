"""CPU check of the property the GPU ghost fill is built on: a fill reads no ghost cell that it
writes, except the innermost layer of the three lower faces.

The library writes every other ghost cell in place during the interpolation pass and stages only
those innermost lower layers (adaptivemesh_gb300/csrc/kernels_amr.cu, k_ghost_fill).  That gives
the pre-fill-state result only if no interpolation reads a cell written in place.  Here the cells
written in place are poisoned with NaN and the oracle's fill (which reads the unmodified fields
of the reference's formula, AMR.h:701-762) runs over them: a NaN in any written value would mean
such a read.  Trees: the reference's own octrees from the host fixture; every substep."""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

import cases
from conftest import GOLDEN

CONFIGS = [(16, 3), (28, 2), (32, 3), (8, 2)]


def _inner_lower_layers(used: int, n: int, p: int) -> np.ndarray:
    t = n + 2 * p
    m = np.zeros((used, t, t, t), bool)          # [slot, z, y, x]
    inn = slice(p, p + n)
    m[:, inn, inn, p - 1] = True
    m[:, inn, p - 1, inn] = True
    m[:, p - 1, inn, inn] = True
    return m.reshape(-1)


@pytest.mark.parametrize("n,p", CONFIGS)
@pytest.mark.parametrize("tree", ["wave", "uneven", "bssn", "uniform2"])
def test_fill_reads_no_cell_written_in_place(orc, n, p, tree):
    hg = np.load(os.path.join(GOLDEN, "host_golden.npz"))
    pos, bd = hg[f"tree/{tree}/positions"], hg[f"tree/{tree}/boundaries"]
    used, md = int(hg[f"tree/{tree}/scalars"][3]), int(hg[f"tree/{tree}/scalars"][1])
    xyz = cases.cell_coordinates(pos, used, n, p, 100.0)
    f_old = cases.smooth_field(xyz, 100.0, 1, 11)
    f_new = cases.smooth_field(xyz, 100.0, 1, 12)
    oc = orc.cfg(n, p, 100.0)
    staged = _inner_lower_layers(used, n, p)
    checked = 0
    for s in range(1 << md):
        written = cases.ghost_write_mask(bd, used, n, p, md, s)
        in_place = written & ~staged
        for only_new in (0, 1):
            po, pn = f_old.copy(), f_new.copy()
            pn[in_place] = np.nan
            if not only_new:
                po[in_place] = np.nan
            orc.lib().orc_copy_boundaries(ctypes.byref(oc), orc.P(po), orc.P(pn), orc.P(bd), used, s, md, only_new)
            assert not np.isnan(pn[written]).any(), f"substep {s}: a fill read a cell written in place (new)"
            if not only_new:
                assert not np.isnan(po[written]).any(), f"substep {s}: a fill read a cell written in place (old)"
            checked += int(written.sum())
    if tree != "wave" or n != 8:
        assert checked > 0
