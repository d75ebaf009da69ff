"""Sharding by domain on CPU ranks: partition, exchange plan and the exchange itself.

A rank holds valid data only for the domains it owns (here everything else is NaN).  After it
receives the boxes of its exchange plan, its ghost fill (the oracle's, which reads the pre-fill
state as the GPU fill does) must give, on every ghost cell of its own domains, exactly the values of
a fill over the whole, unsharded state: any cell the plan missed would bring a NaN in.  The
multi-process test runs the exchange over torch.distributed with the gloo backend."""
from __future__ import annotations

import ctypes
import os
import socket

import numpy as np
import pytest

import cases
from conftest import GOLDEN

OUTER = 100.0
CONFIGS = [(16, 3), (28, 2), (32, 3), (8, 2)]


def _tree(name: str):
    hg = np.load(os.path.join(GOLDEN, "host_golden.npz"))
    sc = hg[f"tree/{name}/scalars"]
    return hg[f"tree/{name}/positions"], hg[f"tree/{name}/boundaries"], int(sc[3]), int(sc[1])


def _fields(pos, used, n, p):
    xyz = cases.cell_coordinates(pos, used, n, p, OUTER)
    return cases.smooth_field(xyz, OUTER, 1, 11), cases.smooth_field(xyz, OUTER, 1, 12)


def _pack_host(field: np.ndarray, boxes: np.ndarray, t: int) -> np.ndarray:
    """Host copy of amr_pack_boxes: each box, x fastest, back to back."""
    cube = field.reshape(-1, t, t, t)
    parts = [cube[b[0], b[4]:b[4] + b[7], b[3]:b[3] + b[6], b[2]:b[2] + b[5]].reshape(-1) for b in boxes]
    return np.concatenate(parts) if parts else np.zeros(0, np.float32)


def _unpack_host(field: np.ndarray, boxes: np.ndarray, t: int, buf: np.ndarray) -> None:
    cube = field.reshape(-1, t, t, t)
    o = 0
    for b in boxes:
        k = int(b[5]) * int(b[6]) * int(b[7])
        cube[b[0], b[4]:b[4] + b[7], b[3]:b[3] + b[6], b[2]:b[2] + b[5]] = buf[o:o + k].reshape(b[7], b[6], b[5])
        o += k


def _owned_mask(owner: np.ndarray, r: int, t: int) -> np.ndarray:
    return np.repeat(owner == r, t ** 3)


@pytest.mark.parametrize("tree", ["bssn", "uneven", "uniform2"])
@pytest.mark.parametrize("ranks", [1, 2, 3, 5])
def test_partition_is_balanced_and_contiguous(am, tree, ranks):
    from adaptivemesh_gb300 import sharding
    pos, _bd, used, _md = _tree(tree)
    owner = sharding.partition_morton(pos, used, ranks)
    live = pos[:used] != 0xFFFFFFFF
    assert np.all((owner >= 0) == live)
    counts = np.bincount(owner[live], minlength=ranks)
    assert counts.max() - counts.min() <= 1
    # contiguous in preorder: walking the tree depth first, the owner never decreases
    children = {}
    for s in range(1, used):
        if live[s]:
            d = int(pos[s]) >> 27
            parent_path = int(pos[s]) & ((1 << (3 * (d - 1))) - 1)
            children.setdefault((d - 1, parent_path), []).append(((int(pos[s]) >> (3 * (d - 1))) & 7, s))
    order = []

    def walk(slot, depth, path):
        order.append(slot)
        for _off, c in sorted(children.get((depth, path), [])):
            walk(c, depth + 1, int(pos[c]) & ((1 << (3 * (depth + 1))) - 1))
    walk(0, 0, 0)
    assert sorted(order) == list(np.nonzero(live)[0])
    assert np.all(np.diff(owner[order]) >= 0)


@pytest.mark.parametrize("n,p", CONFIGS)
@pytest.mark.parametrize("tree", ["bssn", "uneven", "uniform2"])
@pytest.mark.parametrize("ranks", [2, 3])
def test_plan_brings_every_cell_the_fill_reads(am, orc, n, p, tree, ranks):
    from adaptivemesh_gb300 import sharding
    pos, bd, used, md = _tree(tree)
    t = n + 2 * p
    cfg = am.Config(n, p, OUTER)
    oc = orc.cfg(n, p, OUTER)
    f_old, f_new = _fields(pos, used, n, p)
    owner = sharding.partition_morton(pos, used, ranks)
    received = 0
    for s in range(1 << md):
        full_old, full_new = f_old.copy(), f_new.copy()
        orc.lib().orc_copy_boundaries(ctypes.byref(oc), orc.P(full_old), orc.P(full_new), orc.P(bd), used, s, md, 0)
        written = cases.ghost_write_mask(bd, used, n, p, md, s)
        for r in range(ranks):
            boxes = sharding.exchange_plan(cfg, bd, owner, used, s, md, r)
            received += len(boxes)
            mine = _owned_mask(owner, r, t)
            lo, ln = np.where(mine, f_old, np.nan).astype(np.float32), np.where(mine, f_new, np.nan).astype(np.float32)
            for src, dst in ((f_old, lo), (f_new, ln)):
                _unpack_host(dst, boxes, t, _pack_host(src, boxes, t))
            orc.lib().orc_copy_boundaries(ctypes.byref(oc), orc.P(lo), orc.P(ln), orc.P(bd), used, s, md, 0)
            sel = mine & written
            assert np.array_equal(lo[sel].view(np.uint32), full_old[sel].view(np.uint32)), f"substep {s} rank {r} old"
            assert np.array_equal(ln[sel].view(np.uint32), full_new[sel].view(np.uint32)), f"substep {s} rank {r} new"
    assert received > 0


def _free_port() -> int:
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, n: int, p: int, tree: str):
    import torch
    import torch.distributed as dist
    import adaptivemesh_gb300 as am
    from adaptivemesh_gb300 import sharding
    from oracle import oracle as orc
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        pos, bd, used, md = _tree(tree)
        ch = np.load(os.path.join(GOLDEN, "host_golden.npz"))[f"tree/{tree}/children"]
        t = n + 2 * p
        cfg, oc = am.Config(n, p, OUTER), orc.cfg(n, p, OUTER)
        f_old, f_new = _fields(pos, used, n, p)
        owner = sharding.partition_morton(pos, used, world)
        mine = _owned_mask(owner, rank, t)
        pack = lambda f, b: torch.from_numpy(_pack_host(f, b, t))                 # noqa: E731
        unpack = lambda f, b, buf: _unpack_host(f, b, t, buf.numpy())            # noqa: E731
        for s in range(1 << md):
            # this rank's state: its own domains only; a substep's restriction, then its ghost fill
            lo = np.where(mine, f_old, np.nan).astype(np.float32)
            ln = np.where(mine, f_new, np.nan).astype(np.float32)
            plans = [sharding.restriction_plan(cfg, pos, ch, owner, used, s, md, q) for q in range(world)]
            sharding.exchange(dist, rank, world, plans, [ln], pack=pack, unpack=unpack)
            orc.lib().orc_copy_new_to_old(ctypes.byref(oc), orc.P(lo), orc.P(ln), orc.P(pos), orc.P(ch), used, s, md)
            plans = [sharding.exchange_plan(cfg, bd, owner, used, s, md, q) for q in range(world)]
            sharding.exchange(dist, rank, world, plans, [lo, ln], pack=pack, unpack=unpack)
            orc.lib().orc_copy_boundaries(ctypes.byref(oc), orc.P(lo), orc.P(ln), orc.P(bd), used, s, md, 0)
            full_old, full_new = f_old.copy(), f_new.copy()
            orc.lib().orc_copy_new_to_old(ctypes.byref(oc), orc.P(full_old), orc.P(full_new), orc.P(pos), orc.P(ch),
                                          used, s, md)
            orc.lib().orc_copy_boundaries(ctypes.byref(oc), orc.P(full_old), orc.P(full_new), orc.P(bd), used, s, md, 0)
            depth = np.array([int(x) >> 27 if x != 0xFFFFFFFF else -1 for x in pos[:used]])
            active = np.repeat(np.array([d >= 0 and (s & ((1 << (md - d)) - 1)) == 0 for d in depth]), t ** 3)
            sel = mine & (cases.ghost_write_mask(bd, used, n, p, md, s) | active)
            assert np.array_equal(lo[sel].view(np.uint32), full_old[sel].view(np.uint32)), f"rank {rank} substep {s}"
            assert np.array_equal(ln[sel].view(np.uint32), full_new[sel].view(np.uint32)), f"rank {rank} substep {s}"
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,n,p,tree", [(2, 16, 3, "bssn"), (3, 28, 2, "uneven")])
def test_exchange_over_gloo(orc, world, n, p, tree):
    """Each substep's two exchanges (children before the restriction, source boxes before the
    ghost fill) over torch.distributed with gloo: every rank's own domains end as in the unsharded
    substep."""
    import torch.multiprocessing as mp
    mp.spawn(_rank_main, args=(world, _free_port(), n, p, tree), nprocs=world, join=True)


@pytest.mark.parametrize("n,p", [(16, 3), (28, 2)])
@pytest.mark.parametrize("tree", ["bssn", "uneven", "uniform2"])
@pytest.mark.parametrize("ranks", [2, 3, 5])
def test_restriction_plan_brings_every_child(am, orc, n, p, tree, ranks):
    """With only its own domains valid (the rest NaN), a rank that receives its restriction plan's
    boxes restricts every active domain it owns exactly as the unsharded restriction does."""
    from adaptivemesh_gb300 import sharding
    hg = np.load(os.path.join(GOLDEN, "host_golden.npz"))
    pos, _bd, used, md = _tree(tree)
    ch = hg[f"tree/{tree}/children"]
    t = n + 2 * p
    cfg, oc = am.Config(n, p, OUTER), orc.cfg(n, p, OUTER)
    f_old, f_new = _fields(pos, used, n, p)
    owner = sharding.partition_morton(pos, used, ranks)
    depth = np.array([int(x) >> 27 if x != 0xFFFFFFFF else -1 for x in pos[:used]])
    received = 0
    for s in range(1 << md):
        full_old = f_old.copy()
        orc.lib().orc_copy_new_to_old(ctypes.byref(oc), orc.P(full_old), orc.P(f_new), orc.P(pos), orc.P(ch), used, s, md)
        for r in range(ranks):
            boxes = sharding.restriction_plan(cfg, pos, ch, owner, used, s, md, r)
            received += len(boxes)
            assert all(owner[b[0]] == b[1] != r for b in boxes)
            mine = _owned_mask(owner, r, t)
            lo = np.where(mine, f_old, np.nan).astype(np.float32)
            ln = np.where(mine, f_new, np.nan).astype(np.float32)
            _unpack_host(ln, boxes, t, _pack_host(f_new, boxes, t))
            orc.lib().orc_copy_new_to_old(ctypes.byref(oc), orc.P(lo), orc.P(ln), orc.P(pos), orc.P(ch), used, s, md)
            active = np.array([d >= 0 and (s & ((1 << (md - d)) - 1)) == 0 for d in depth])
            sel = np.repeat((owner == r) & active, t ** 3)
            assert np.array_equal(lo[sel].view(np.uint32), full_old[sel].view(np.uint32)), f"substep {s} rank {r}"
    if ranks > 1 and tree != "uniform2":
        assert received > 0


def test_plan_refuses_records_deeper_than_the_tree(am):
    """A boundary record whose depth exceeds max_depth (a bad upload or checkpoint) would make the
    plan shift by a negative count: refused with AMR_ERR_INVALID."""
    from adaptivemesh_gb300 import sharding
    pos, bd, used, md = _tree("bssn")
    owner = sharding.partition_morton(pos, used, 2)
    bd = bd.copy()
    slot = next(s for s in range(used) if int(bd[s * 6]) & 0xFFFFFF not in (0xFFFFFF,) and owner[s] == 1)
    word = int(bd[slot * 6])
    bd[slot * 6] = (word & ~(0xF << 28)) | ((md + 1) << 28)
    with pytest.raises(am.AmrError) as info:
        sharding.exchange_plan(am.Config(16, 3, OUTER), bd, owner, used, 0, md, 1)
    assert info.value.status == am.ERR_INVALID
