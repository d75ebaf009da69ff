"""Deterministic test cases shared by the fixture generators and the tests.

Inputs are regenerated from integer seeds with numpy's PCG64 generator, which gives
identical streams on x86_64 and aarch64, so a fixture only has to store seeds and the
outputs (or their sha256 digests).

Trees are built through an octree object exposing add_node(parent, offset) -- either the
reference's own AMR<T> (oracle/reflib.RefOctree) or this project's octree -- in the
orders the reference's driver uses (AdaptiveMesh/kernel.cu:49-50 and :69-83).
"""
from __future__ import annotations

import hashlib

import numpy as np

# ---------------------------------------------------------------- trees

def tree_wave(o):
    """Root plus its eight children (AdaptiveMesh/kernel.cu:49-50)."""
    for c in range(8):
        o.add_node(0, c)


def tree_bssn(o, first_free=None):
    """Nested refinement towards the centre to depth 6, 49 nodes (kernel.cu:69-83)."""
    children = []
    for c in range(8):
        children.append(o.state()["first_free"] if first_free is None else first_free())
        o.add_node(0, c)
    for _d in range(1, 6):
        for c in range(8):
            new_idx = o.state()["first_free"] if first_free is None else first_free()
            o.add_node(children[c], (~c) & 7)
            children[c] = new_idx


def tree_uneven(o):
    """An unevenly refined tree: depths 0..3 with partial octants."""
    for c in range(8):
        o.add_node(0, c)                     # slots 1..8, depth 1
    for c in (0, 3, 5, 6):
        o.add_node(1, c)                     # slots 9..12 under slot 1
    o.add_node(8, 2)                         # slot 13 under slot 8
    o.add_node(9, 7)                         # slot 14, depth 3 under slot 9
    o.add_node(9, 1)                         # slot 15, depth 3


def tree_uniform(o, depth: int):
    """Uniform refinement to `depth` (all octants), breadth first."""
    level = [0]
    for _d in range(depth):
        nxt = []
        for p in level:
            for c in range(8):
                idx = o.state()["first_free"]
                o.add_node(p, c)
                nxt.append(idx)
        level = nxt


def tree_random(o, depth: int, p_refine: float = 0.3, seed: int = 0):
    """Seeded Bernoulli refinement: the root is refined, then every domain at depth 1 .. depth-1 is
    refined (all eight octants) with probability p_refine, level by level."""
    rng = np.random.default_rng(seed)
    level = [0]
    for d in range(depth):
        chosen = [p for p in level if d == 0 or rng.random() < p_refine]
        if hasattr(o, "add_nodes"):   # one batch per level: the same slots as the calls one by one
            o.add_nodes([p for p in chosen for _ in range(8)], [c for _ in chosen for c in range(8)])
        else:
            for p in chosen:
                for c in range(8):
                    o.add_node(p, c)
        ch = o.state()["children"]
        level = [int(ch[p * 8 + c]) for p in chosen for c in range(8)]


def tree_root(o):
    """The root alone: one domain at depth 0, no ghost fill."""


def tree_deep(o):
    """Nested refinement towards the centre down to the depth limit, 8 (AMR.h:9): 65 nodes.  Then
    one add below a depth-8 node, which the octree ignores (AMR.h:211)."""
    children = []
    for c in range(8):
        children.append(o.state()["first_free"])
        o.add_node(0, c)
    for _d in range(1, 8):
        for c in range(8):
            new_idx = o.state()["first_free"]
            o.add_node(children[c], (~c) & 7)
            children[c] = new_idx
    o.add_node(children[0], 0)


def tree_full(o):
    """Root and eight children in a 9-slot octree: a further add is ignored (AMR.h:210) until a
    removal frees a slot, which the next add reuses."""
    for c in range(8):
        o.add_node(0, c)
    o.add_node(1, 0)
    o.remove_node(3)
    o.add_node(1, 0)
    o.add_node(2, 5)


TREES = {"wave": tree_wave, "bssn": tree_bssn, "uneven": tree_uneven}
# limits: the depth limit and a full slot array (slots: deep 80, full 9)
EDGE_TREES = {"root": tree_root, "deep": tree_deep, "full": tree_full}
EDGE_SLOTS = {"root": 64, "deep": 80, "full": 9}
ALL_TREES = {**TREES, **EDGE_TREES}


# ---------------------------------------------------------------- field inputs

def cell_coordinates(positions: np.ndarray, used: int, n: int, p: int, outer_size: float):
    """Absolute coordinates of every padded cell of the first `used` slots, following
    the seed kernel's mapping (AdaptiveMesh/kernel.cu:21-22).  Unused slots get NaN."""
    t = n + 2 * p
    idx = np.arange(t, dtype=np.float64)
    out = np.full((used, t, t, t, 3), np.nan)
    for s in range(used):
        pos = int(positions[s])
        if pos == 0xFFFFFFFF:
            continue
        depth = pos >> 27
        c = np.zeros(3)
        path = pos & ((1 << 27) - 1)
        for i in range(depth):
            for a, bit in enumerate((1, 2, 4)):
                c[a] += (0.25 if path & bit else -0.25) / (1 << i)
            path >>= 3
        c *= outer_size
        h = (outer_size / n) / (1 << depth)
        off = (idx + 0.5 - t * 0.5) * h
        out[s, ..., 0] = c[0] + off[None, None, :]
        out[s, ..., 1] = c[1] + off[None, :, None]
        out[s, ..., 2] = c[2] + off[:, None, None]
    return out


def smooth_field(xyz: np.ndarray, outer_size: float, k: int, seed: int, noise: float = 1e-3) -> np.ndarray:
    """A smooth scalar field over the domain plus a little seeded noise, as float32.
    Unused slots (NaN coordinates) become 0."""
    rng = np.random.default_rng(seed)
    L = outer_size
    ph = rng.uniform(0, 2 * np.pi, 3)
    x, y, z = xyz[..., 0], xyz[..., 1], xyz[..., 2]
    f = (0.5 * np.sin(2 * np.pi * (k + 1) * x / L + ph[0]) * np.cos(2 * np.pi * y / L + ph[1])
         + 0.3 * np.cos(2 * np.pi * (k + 2) * z / L + ph[2]) + 0.2 * np.exp(-(x * x + y * y + z * z) / (0.05 * L * L)))
    f = f + noise * rng.standard_normal(f.shape)
    f = np.where(np.isnan(f), 0.0, f)
    return f.astype(np.float32).reshape(-1)


def metric_fields(xyz: np.ndarray, outer_size: float, seed: int) -> list[np.ndarray]:
    """Six conformal-metric components (xx, xy, xz, yy, yz, zz), positive definite."""
    out = []
    for k, (diag, scale) in enumerate([(1, 0.1), (0, 0.05), (0, 0.05), (1, 0.1), (0, 0.05), (1, 0.1)]):
        f = smooth_field(xyz, outer_size, k, seed + 17 * k)
        out.append((diag + scale * f).astype(np.float32))
    # unused slots: identity metric keeps the inverse finite there too
    used_mask = ~np.isnan(xyz[..., 0]).reshape(-1)
    for k in (0, 3, 5):
        out[k] = np.where(used_mask, out[k], np.float32(1.0)).astype(np.float32)
    return out


# ---------------------------------------------------------------- codec inputs

def codec_inputs(n: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """Triples spanning the codec's regimes plus per-element generator seeds.

    Covers zeros, signed zeros, subnormals, exponent saturation (|x| >= 2^17), flush of
    small components, mixed magnitudes, NaN/Inf and random bit patterns."""
    rng = np.random.default_rng(seed)
    parts = []
    m = n // 8
    f32 = lambda a: a.astype(np.float32)  # noqa: E731
    with np.errstate(invalid="ignore", over="ignore"):
        parts.append(f32(rng.standard_normal((m, 3))))                                   # O(1)
        parts.append(f32(rng.standard_normal((m, 3)) * 10.0 ** rng.uniform(-12, 12, (m, 1))))  # common scale
        parts.append(f32(rng.standard_normal((m, 3)) * 10.0 ** rng.uniform(-8, 8, (m, 3))))    # mixed magnitudes
        parts.append(f32(rng.uniform(-300, 300, (m, 3))))
        bits = rng.integers(0, 2 ** 32, (m, 3), dtype=np.uint64).astype(np.uint32)
        parts.append(bits.view(np.float32))                                   # random patterns (incl. NaN/Inf)
        special = np.array([[0, 0, 0], [-0.0, 0, 0], [1e-40, -1e-41, 0], [2 ** 17, 1, -1], [2 ** 20, -3, 5],
                            [np.inf, 1, 0], [np.nan, 1, 2], [-np.inf, 0, 1], [1e-38, 1e-38, -1e-38],
                            [3.4e38, -3.4e38, 1], [2 ** -22, 2 ** -23, 2 ** -24], [1, -0.5, 0.25], [3, 1e-9, -7]])
        parts.append(f32(np.tile(special, (m // len(special) + 1, 1))[:m]))
        parts.append(f32(rng.standard_normal((m, 3)) * 2.0 ** rng.integers(-30, 30, (m, 1))))
        rest = n - 7 * m
        parts.append(f32(rng.standard_normal((rest, 3)) * 1e-3))
    xyz = np.concatenate(parts)
    seeds = rng.integers(-2 ** 31, 2 ** 31, n, dtype=np.int64).astype(np.int32)
    return np.ascontiguousarray(xyz.reshape(-1)), seeds


def digest(a) -> str:
    """sha256 of an array's raw bytes (numpy or torch)."""
    if not isinstance(a, np.ndarray):
        a = a.detach().cpu().numpy()
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def codec_words(n: int, seed: int) -> np.ndarray:
    """Random compressed_float3 words (every bit pattern is a valid word)."""
    return np.random.default_rng(seed).integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)


def substeps_for(md: int) -> list[int]:
    """Substeps exercised per tree: the first two, the middle-plus-one and the last of a timestep
    (timer_helper values, AMR.h:178), so every depth is active in at least one of them."""
    s = {0, 1, (1 << md) - 1}
    if md >= 2:
        s.add((1 << (md - 1)) + 1)
    return sorted(x for x in s if x < (1 << md))


def ghost_write_mask(boundaries: np.ndarray, used: int, n: int, p: int, md: int, s: int) -> np.ndarray:
    """Cells the ghost fill writes at substep s: the face ghost layers of every face with a
    neighbour whose depth is active (AMR.h:710-735), as a flat mask over the padded fields."""
    t = n + 2 * p
    m = np.zeros((used, t, t, t), bool)          # [slot, z, y, x]
    lo, hi, inn = slice(0, p), slice(p + n, t), slice(p, p + n)
    faces = [(inn, inn, hi), (inn, hi, inn), (hi, inn, inn), (inn, inn, lo), (inn, lo, inn), (lo, inn, inn)]
    for slot in range(used):
        for f in range(6):
            b = int(boundaries[slot * 6 + f])
            nd = b & 0xFFFFFFFF
            target = (nd & 0xFFFFFF) - ((1 << 24) if nd & (1 << 23) else 0)
            cd = -1 if (nd >> 28) == 15 else nd >> 28
            if target == -1 or cd <= 0 or (s & ((1 << (md - cd)) - 1)) != 0:
                continue
            zs, ys, xs = faces[f]
            m[slot, zs, ys, xs] = True
    return m.reshape(-1)
