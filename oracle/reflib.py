"""ctypes access to the reference-build library (oracle/_ref/libamr_ref_<cfg>.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
reference leg.  The library wraps the reference's own code; see oracle/ref_harness.cu.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_ref

_c = ctypes
VP = _c.c_void_p
U32 = _c.c_uint32
I32 = _c.c_int32

_SIGS = {
    "refh_constants": (None, [VP, VP]),
    "refh_prng_ints": (None, [I32, _c.c_int, VP]),
    "refh_prng_floats": (None, [I32, _c.c_int, VP]),
    "refh_prng_ranged": (None, [I32, _c.c_int, I32, I32, VP]),
    "refh_cf3_encode_stream": (I32, [VP, _c.c_int, I32, VP]),
    "refh_cf3_encode_seeded": (None, [VP, VP, _c.c_int, VP]),
    "refh_cf3_encode_det": (None, [VP, _c.c_int, VP]),
    "refh_cf3_decode": (None, [VP, _c.c_int, VP]),
    "refh_sum_coordinates": (U32, [U32, U32, _c.c_int]),
    "refh_diff_coordinates": (U32, [U32, U32, _c.c_int]),
    "refh_reverse_bits": (U32, [U32]),
    "refh_abs_position": (None, [U32, VP]),
    "refh_boundary": (_c.c_uint64, [U32, U32, I32]),
    "refh_boundary_decode": (None, [_c.c_uint64, VP, VP, VP, VP, VP]),
    "refh_octree_create": (VP, [U32]),
    "refh_octree_destroy": (None, [VP]),
    "refh_octree_add_node": (None, [VP, I32, I32]),
    "refh_octree_remove_node": (None, [VP, I32]),
    "refh_octree_increment_timer": (None, [VP]),
    "refh_octree_find_node_idx": (U32, [VP, U32, U32]),
    "refh_octree_state": (None, [VP, VP, VP, VP, VP, VP, VP]),
    "refh_sym_inverse": (None, [VP, _c.c_int, VP]),
    "refd_cf3_encode_seeded": (_c.c_int, [VP, VP, _c.c_int, VP]),
    "refd_cf3_encode_det": (_c.c_int, [VP, _c.c_int, VP]),
    "refd_cf3_decode": (_c.c_int, [VP, _c.c_int, VP]),
    "refd_prng_floats": (_c.c_int, [VP, _c.c_int, _c.c_int, VP]),
    "refd_sym_inverse": (_c.c_int, [VP, _c.c_int, VP]),
    "refd_probe": (_c.c_int, [_c.c_int, VP, _c.c_int, VP]),
    "refd_differentiate": (_c.c_int, [VP, VP, VP, VP, U32, U32, U32, I32]),
    "refd_mixed_partials": (_c.c_int, [VP, VP, VP, U32, U32, U32, I32]),
    "refd_deriv_trace": (_c.c_int, [VP, VP, VP, VP, VP, U32, U32, U32]),
    "refd_christoffel": (_c.c_int, [VP, VP, I32, VP, VP, U32, U32, U32]),
    "refd_copy_boundaries": (_c.c_int, [VP, VP, VP, U32, U32, U32, _c.c_int]),
    "refd_copy_new_to_old": (_c.c_int, [VP, VP, VP, VP, U32, U32, U32]),
    "refd_copy_to_child": (_c.c_int, [VP, U32, I32, I32]),
    "refd_wave_step": (_c.c_int, [_c.c_int, VP, VP, VP, VP, VP, U32, U32, U32]),
    "refd_criterion": (_c.c_int, [VP, VP, VP, VP, U32, U32, U32]),
    "refd_rasterise": (_c.c_int, [VP, VP, VP, U32, U32, _c.c_float]),
    "refd_scan": (_c.c_int, [_c.c_int, _c.c_int, VP, U32]),
    "refd_extreme": (_c.c_int, [_c.c_int, _c.c_int, _c.c_int, VP, U32, VP]),
    "refd_bssn_create": (VP, [U32]),
    "refd_bssn_destroy": (None, [VP]),
    "refd_bssn_add_node": (None, [VP, I32, I32]),
    "refd_bssn_remove_node": (None, [VP, I32]),
    "refd_bssn_field": (VP, [VP, _c.c_int, _c.c_int]),
    "refd_bssn_cf3": (VP, [VP, _c.c_int, _c.c_int]),
    "refd_bssn_timestep": (_c.c_int, [VP]),
    "refd_bssn_copy_bounds": (_c.c_int, [VP]),
    "refd_bssn_rng_seed": (I32, [VP]),
    "refd_bssn_octree_state": (None, [VP, VP, VP, VP, VP, VP, VP]),
    "refd_wave_create": (VP, [U32]),
    "refd_wave_destroy": (None, [VP]),
    "refd_wave_add_node": (None, [VP, I32, I32]),
    "refd_wave_field": (VP, [VP, _c.c_int]),
    "refd_wave_cf3": (VP, [VP, _c.c_int]),
    "refd_wave_criterion_host": (VP, [VP]),
    "refd_wave_timestep": (_c.c_int, [VP]),
    "refd_wave_copy_bounds": (_c.c_int, [VP]),
    "refd_wave_rng_seed": (I32, [VP]),
    "refd_wave_octree_state": (None, [VP, VP, VP, VP, VP, VP, VP]),
}

_LIBS: dict[str, ctypes.CDLL] = {}


def available(cfg: str = "n28p2") -> bool:
    return os.path.exists(build_ref.lib_path(cfg))


def load(cfg: str = "n28p2") -> ctypes.CDLL:
    """Load (building first if needed and possible) the reference-build library for a configuration."""
    if cfg in _LIBS:
        return _LIBS[cfg]
    path = build_ref.lib_path(cfg)
    if os.path.isdir(os.path.join(build_ref.OUT, "src", cfg)):
        build_ref.build([cfg])  # incremental: rebuilds only when the harness or headers changed
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[cfg] = lib
    return lib


def ptr(a) -> int:
    """Address of a numpy array or torch tensor."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def constants(lib) -> dict:
    u = np.zeros(4, np.uint32)
    f = np.zeros(3, np.float32)
    lib.refh_constants(ptr(u), ptr(f))
    return {"size_domain": int(u[0]), "padding_domain": int(u[1]), "total": int(u[2]), "depth_limit": int(u[3]),
            "outer_size": float(f[0]), "outer_dx": float(f[1]), "outer_dt": float(f[2])}


class RefOctree:
    """The reference's host octree AMR<blank_AMR_data> (AdaptiveMesh/AMR.h:118-294)."""

    def __init__(self, lib, slots: int):
        self.lib, self.slots = lib, slots
        self.h = lib.refh_octree_create(slots)

    def add_node(self, parent: int, offset: int):
        self.lib.refh_octree_add_node(self.h, parent, offset)

    def remove_node(self, idx: int):
        self.lib.refh_octree_remove_node(self.h, idx)

    def increment_timer(self):
        self.lib.refh_octree_increment_timer(self.h)

    def find_node_idx(self, packed: int, max_depth: int = 0xFFFFFFFF) -> int:
        return self.lib.refh_octree_find_node_idx(self.h, packed, max_depth)

    def state(self) -> dict:
        return octree_state(self.lib.refh_octree_state, self.h, self.slots)

    def close(self):
        if self.h:
            self.lib.refh_octree_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def octree_state(fn, h, slots: int) -> dict:
    pos = np.zeros(slots, np.uint32)
    par = np.zeros(slots, np.int32)
    ch = np.zeros(slots * 8, np.int32)
    bd = np.zeros(slots * 6, np.uint64)
    life = np.zeros(slots, np.uint32)
    sc = np.zeros(5, np.uint32)
    fn(h, ptr(pos), ptr(par), ptr(ch), ptr(bd), ptr(life), ptr(sc))
    return {"positions": pos, "parent": par, "children": ch, "boundaries": bd, "lifetime": life,
            "timer": int(sc[0]), "max_depth": int(sc[1]), "first_free": int(sc[2]), "used_slots": int(sc[3]),
            "max_slots": int(sc[4])}
