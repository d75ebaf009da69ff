"""Sharding the per-timestep path by domain across ranks.

Domains are independent given their ghost cells, so ranks own contiguous Morton ranges of the
octree's slots (amr_partition_morton) and compute only those.  Two exchanges per substep: before
the restriction, each rank receives the new field's interior of the children, owned elsewhere, of
its active domains (amr_restriction_exchange_plan); before the ghost fill, it receives from the
owners the source boxes its faces interpolate from (amr_ghost_exchange_plan; the boxes the fill
kernel itself reads), for the old and the new field of every component, then fills its own
domains' ghosts locally.  The reference runs on one
GPU (AdaptiveMesh/AMR.h:880-933 fills all faces in one launch); this module is the host side of
the multi-rank form.  Transport is torch.distributed point-to-point (NCCL on GPUs, gloo on CPUs);
packing and unpacking are passed in, so device buffers use amr_pack_boxes / amr_unpack_boxes and
host arrays any equivalent copy.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import ERR_CAPACITY, Config, check, load

BOX_WORDS = 8   # {source slot, source rank, lo x, lo y, lo z, extent x, extent y, extent z}


def partition_morton(positions: np.ndarray, used: int, ranks: int) -> np.ndarray:
    """owner[slot] for the first `used` slots: balanced contiguous preorder ranges, -1 if free."""
    lib = load()
    pos = np.ascontiguousarray(positions[:used], dtype=np.uint32)
    owner = np.empty(used, np.int32)
    check(lib.amr_partition_morton(pos.ctypes.data, used, ranks, owner.ctypes.data))
    return owner


def exchange_plan(cfg: Config, boundaries: np.ndarray, owner: np.ndarray, used: int, substep: int, max_depth: int,
                  rank: int) -> np.ndarray:
    """The boxes `rank` receives before the ghost fill of `substep`, as an (n, 8) uint32 array."""
    lib = load()
    bd = np.ascontiguousarray(boundaries[: used * 6], dtype=np.uint64)
    own = np.ascontiguousarray(owner[:used], dtype=np.int32)
    n = ctypes.c_uint32(0)
    st = lib.amr_ghost_exchange_plan(ctypes.byref(cfg), bd.ctypes.data, own.ctypes.data, used, substep, max_depth,
                                     rank, None, 0, ctypes.byref(n))
    if st != ERR_CAPACITY:   # a zero-capacity call reports the count needed
        check(st)
    boxes = np.zeros((n.value, BOX_WORDS), np.uint32)
    if n.value:
        check(lib.amr_ghost_exchange_plan(ctypes.byref(cfg), bd.ctypes.data, own.ctypes.data, used, substep,
                                          max_depth, rank, boxes.ctypes.data, n.value, ctypes.byref(n)))
    return boxes


def restriction_plan(cfg: Config, positions: np.ndarray, children: np.ndarray, owner: np.ndarray, used: int,
                     substep: int, max_depth: int, rank: int) -> np.ndarray:
    """The boxes (children's interiors of the new field) `rank` receives before the restriction of
    `substep`, as an (n, 8) uint32 array (amr_restriction_exchange_plan)."""
    lib = load()
    pos = np.ascontiguousarray(positions[:used], dtype=np.uint32)
    ch = np.ascontiguousarray(children[: used * 8], dtype=np.int32)
    own = np.ascontiguousarray(owner[:used], dtype=np.int32)
    n = ctypes.c_uint32(0)
    args = (ctypes.byref(cfg), pos.ctypes.data, ch.ctypes.data, own.ctypes.data, used, substep, max_depth, rank)
    st = lib.amr_restriction_exchange_plan(*args, None, 0, ctypes.byref(n))
    if st != ERR_CAPACITY:
        check(st)
    boxes = np.zeros((n.value, BOX_WORDS), np.uint32)
    if n.value:
        check(lib.amr_restriction_exchange_plan(*args, boxes.ctypes.data, n.value, ctypes.byref(n)))
    return boxes


def box_offsets(boxes: np.ndarray) -> np.ndarray:
    """Float offset of each box in a packed buffer (boxes back to back), plus the total at the end."""
    sizes = boxes[:, 5].astype(np.uint64) * boxes[:, 6] * boxes[:, 7] if len(boxes) else np.zeros(0, np.uint64)
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)


def pack_boxes(cfg: Config, field, used: int, boxes_dev, offsets_dev, n_boxes: int, out, stream=None) -> None:
    """Device gather of the boxes of one padded field into `out` (amr_pack_boxes)."""
    check(load().amr_pack_boxes(ctypes.byref(cfg), field.data_ptr(), used, boxes_dev.data_ptr(),
                                offsets_dev.data_ptr(), n_boxes, out.data_ptr(), stream))


def unpack_boxes(cfg: Config, field, used: int, boxes_dev, offsets_dev, n_boxes: int, buf, stream=None) -> None:
    """Device scatter of a packed buffer into the boxes of one padded field (amr_unpack_boxes)."""
    check(load().amr_unpack_boxes(ctypes.byref(cfg), field.data_ptr(), used, boxes_dev.data_ptr(),
                                  offsets_dev.data_ptr(), n_boxes, buf.data_ptr(), stream))


def exchange(dist, rank: int, world: int, plans: list[np.ndarray], fields: list, pack, unpack) -> None:
    """One ghost exchange.  plans[q] = exchange_plan(..., rank=q) for every rank q (each rank computes
    all of them from the same octree).  For every other rank q this rank sends, per field, the boxes
    of plans[q] whose source it owns, and receives those of plans[rank] owned by q.
    pack(field, boxes) -> tensor and unpack(field, boxes, tensor) do the copies."""
    requests, receives, outgoing = [], [], []
    for q in range(world):
        if q == rank:
            continue
        send = plans[q][plans[q][:, 1] == rank] if len(plans[q]) else plans[q]
        recv = plans[rank][plans[rank][:, 1] == q] if len(plans[rank]) else plans[rank]
        for f in fields:
            if len(send):
                outgoing.append(pack(f, send))   # kept alive until the sends complete
                requests.append(dist.isend(outgoing[-1], dst=q))
            if len(recv):
                buf = pack(f, recv)   # a buffer of the right size and kind; overwritten by the receive
                requests.append(dist.irecv(buf, src=q))
                receives.append((f, recv, buf))
    for r in requests:
        r.wait()
    for f, recv, buf in receives:
        unpack(f, recv, buf)
