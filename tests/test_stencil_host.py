"""Host-side arithmetic of the fused BSSN pass (k_stencil_bssn), checked on the CPU.

The compute threads' cells must cover a tile's cells once each.  At 16/3 a warp takes rows ty and
ty + 8 of the 22-float padded rows (176 floats = 16 banks apart), so every shared-memory access of
the warp falls on 32 distinct banks.  At 28/2 the padded row is 32 floats, so a cell's bank is fixed
by its x alone: every warp of 32 row-major cells has 4 lanes in 2-way conflicts, as measured (a
layout with rows padded to 36 floats removes them, but its extra 22 KB of shared memory made the
pass slower).  The taps (+-P along each axis, the mixed partials' +-1 diagonals) stay inside the
copied padded rows, and the ring, barriers and per-thread tables fit in one CTA's shared memory.
"""
from __future__ import annotations

import numpy as np
import pytest

SMEM_LIMIT = 232448   # bytes of dynamic shared memory one CTA may use (sm_100 family)


def shape(n: int, p: int) -> dict:
    """StencilShape<N, P, SK_BSSN> (kernels_stencil.cu)."""
    t = n + 2 * p
    ty = n // 2 if n * n > 1024 - 32 else n
    rows = ty + 2 * p
    r = 2 * p + 2
    cells = n * ty
    ring = 6 * r * rows * t * 4
    bars = r * 8 * 2
    tables = 19 * cells * 4
    return dict(T=t, TY=ty, ROWS=rows, R=r, CELLS=cells, CW=(cells + 31) // 32, SMEM=ring + bars + tables)


def cell_of_thread(n: int, t: int):
    """The compute thread's tile cell (x, ty) in k_stencil_bssn (kernels_stencil.cu)."""
    return t % n, (((t // n) >> 1) | (((t // n) & 1) << 3)) if n == 16 else t // n


def conflicted_lanes(n: int, p: int) -> list[int]:
    """Per compute warp, the lanes beyond the first on their bank (same for every tap offset)."""
    s = shape(n, p)
    out = []
    for w in range(s["CW"]):
        lanes = [t for t in range(32 * w, 32 * w + 32) if t < s["CELLS"]]
        banks = [((y + p) * s["T"] + x + p) % 32 for x, y in (cell_of_thread(n, t) for t in lanes)]
        out.append(len(lanes) - len(set(banks)))
    return out


@pytest.mark.parametrize("n,p", [(16, 3), (28, 2), (32, 3), (8, 2)])
def test_threads_cover_the_tile(n, p):
    s = shape(n, p)
    cells = [cell_of_thread(n, t) for t in range(s["CELLS"])]
    assert len(set(cells)) == s["CELLS"]
    assert all(0 <= x < n and 0 <= y < s["TY"] for x, y in cells)


def test_bank_conflicts_per_warp():
    assert conflicted_lanes(16, 3) == [0] * 8      # rows y and y + 8: conflict-free
    assert conflicted_lanes(32, 3) == [0] * 16     # one 32-cell row per warp
    assert set(conflicted_lanes(28, 2)[:-1]) == {4}   # 28 distinct x among 32 lanes


@pytest.mark.parametrize("n,p", [(16, 3), (28, 2), (32, 3), (8, 2)])
def test_taps_stay_in_the_copied_rows(n, p):
    s = shape(n, p)
    for x in (0, n - 1):
        for y in (0, s["TY"] - 1):
            for dx in range(-p, p + 1):
                for dy in range(-p, p + 1):
                    assert 0 <= x + p + dx < s["T"] and 0 <= y + p + dy < s["ROWS"]


@pytest.mark.parametrize("n,p", [(16, 3), (28, 2), (32, 3), (8, 2)])
def test_ring_fits_and_slots_are_aligned(n, p):
    s = shape(n, p)
    assert s["SMEM"] <= SMEM_LIMIT, (n, p, s["SMEM"])
    assert (s["ROWS"] * s["T"] * 4) % 16 == 0   # every slot's bulk copy starts on 16 bytes
    # two CTAs per SM at 16^3 (the launch bounds ask for them)
    if n == 16:
        assert 2 * (s["SMEM"] + 1024) <= 233472
