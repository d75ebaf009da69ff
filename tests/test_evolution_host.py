"""Host-side arithmetic behind the evolution's kernels, checked on the CPU.

* The ghost fill's same-depth copies map a face cell index k to its coordinates by multiplying
  with ceil(2^21 / e) and shifting, in place of two integer divisions: exact for every extent e and
  index k the padded edges up to 38 produce.
* The ghost fill's interpolating faces stage a source box and two intermediate stages in shared
  memory, sized by the launcher from (n, p, t) alone: on seeded random octrees, the nested puncture
  tree and the uneven tree, at 8^3, 16^3 and 32^3, every face with a coarser source needs at most
  that much, and the stencil's base cell grows with the ghost cell's coordinate along every axis
  (the kernel takes the box from the first and the last cell).
* Random octrees built one batch per level have the slots of the same adds made one at a time.
"""
from __future__ import annotations

import numpy as np
import pytest

import cases


def interp_floats(n: int, p: int, t: int) -> int:
    """The launcher's shared-memory size for interpolating faces (kernels_evolve.cu)."""
    best = 0
    for d in range(3):
        ext = [p if a == d else (t if a < d else n) for a in range(3)]
        E = [e // 2 + 5 for e in ext]
        best = max(best, E[0] * E[1] * E[2] + E[2] * E[1] * ext[0] + E[2] * ext[1] * ext[0])
    return best


def test_face_index_division_is_exact():
    k = np.arange(38 * 38 * 3 + 1, dtype=np.uint64)
    for e in range(1, 39):
        m = ((1 << 21) + e - 1) // e
        assert np.array_equal((k * np.uint64(m)) >> np.uint64(21), k // np.uint64(e)), e


def _boxes(st, n, p):
    """Per face with a coarser source and per pass: the needed shared-memory floats, and whether the
    base cells are monotone, with the kernel's single-precision geometry."""
    f32 = np.float32
    t = n + 2 * p
    used = st["used_slots"]
    words = np.asarray(st["boundaries"][: used * 6], np.uint64)
    out = []
    for slot in range(used):
        if int(st["positions"][slot]) == 0xFFFFFFFF:
            continue
        for face in range(6):
            bd = int(words[slot * 6 + face])
            nd = bd & 0xFFFFFFFF
            target = (nd & 0xFFFFFF) | (0xFF000000 if nd & (1 << 23) else 0)
            target = target - (1 << 32) if target >= (1 << 31) else target
            cd = -1 if (nd >> 28) == 15 else nd >> 28
            dd = (nd >> 24) & 15
            if target == -1 or cd <= 0 or dd == 0:
                continue
            rel = cases_cf3_decode(bd >> 32)
            d, side = face % 3, face // 3
            root_src = target == 0
            rel_scale = f32(1.0) / f32(1 << dd)
            E, ext = [], []
            monotone = True
            for a in range(3):
                lo = (p + n if side == 0 else 0) if a == d else (0 if a < d else p)
                ea = p if a == d else (t if a < d else n)
                w = np.arange(lo, lo + ea, dtype=np.float32)
                rp = (w - f32(p) + f32(0.5)) / f32(n) - f32(0.5)
                rp = rp * rel_scale + f32(rel[a])
                ri = (rp + f32(0.5)) * f32(n) + f32(p) - f32(0.5)
                lo_c = 1 if (root_src or a < d) else p + 1
                hi_c = t - 3 if (root_src or a < d) else t - p - 3
                b = np.clip(np.floor(ri).astype(np.int64), lo_c, hi_c)
                monotone &= bool(np.all(np.diff(b) >= 0))
                E.append(int(b.max() - b.min() + 4))
                ext.append(ea)
            out.append((E[0] * E[1] * E[2] + E[2] * E[1] * ext[0] + E[2] * ext[1] * ext[0], monotone))
    return out


def cases_cf3_decode(word: int):
    """The relative position of a boundary record (a compressed_float3 word): value_i = (1 - 2 s_i)
    m_i 2^(E - 22)."""
    e = (word >> 27) & 31
    vals = []
    for mpos, spos in ((0, 8), (9, 17), (18, 26)):
        m = (word >> mpos) & 255
        s = (word >> spos) & 1
        vals.append((-1.0 if s else 1.0) * m * 2.0 ** (e - 22))
    return vals


TREES = {
    "random0": lambda o: cases.tree_random(o, 4, 0.3, 0),
    "random3": lambda o: cases.tree_random(o, 6, 0.3, 3),
    "random25": lambda o: cases.tree_random(o, 5, 0.3, 25),
    "bssn": cases.tree_bssn,
    "uneven": cases.tree_uneven,
}


@pytest.mark.parametrize("tree", sorted(TREES))
def test_interpolating_faces_fit_the_launch(am, tree):
    o = am.Octree(3000)
    TREES[tree](o)
    st = o.state()
    o.close()
    checked = 0
    for n in (8, 16, 32):
        p = 3
        cap = interp_floats(n, p, n + 2 * p)
        for need, monotone in _boxes(st, n, p):
            assert monotone, f"{tree} at {n}^3: base cells not monotone"
            assert need <= cap, f"{tree} at {n}^3: a face needs {need} floats, the launch gives {cap}"
            checked += 1
    assert checked > 0


def test_random_tree_batches_equal_single_adds(am):
    class OneByOne:   # an octree without add_nodes: tree_random adds node by node
        def __init__(self, o):
            self.o = o

        def add_node(self, parent, offset):
            self.o.add_node(parent, offset)

        def state(self):
            return self.o.state()

    for depth, seed in ((4, 0), (6, 3), (5, 25)):
        a, b = am.Octree(3000), am.Octree(3000)
        cases.tree_random(a, depth, 0.3, seed)
        cases.tree_random(OneByOne(b), depth, 0.3, seed)
        sa, sb = a.state(), b.state()
        assert sa["used_slots"] == sb["used_slots"]
        for k in ("positions", "children", "boundaries"):
            assert np.array_equal(sa[k], sb[k]), (depth, seed, k)
        a.close()
        b.close()
