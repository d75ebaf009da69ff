"""Python handles of the C++ octree and plugin simulations (include/amr_gb300.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import MODE_GRAPH, SIM_BSSN, Config, VP, U32, U64, check, load


def _state(fn, h, slots: int) -> dict:
    pos = np.zeros(slots, np.uint32)
    par = np.zeros(slots, np.int32)
    ch = np.zeros(slots * 8, np.int32)
    bd = np.zeros(slots * 6, np.uint64)
    life = np.zeros(slots, np.uint32)
    sc = np.zeros(5, np.uint32)
    check(fn(h, pos.ctypes.data, par.ctypes.data, ch.ctypes.data, bd.ctypes.data, life.ctypes.data, sc.ctypes.data),
          "octree_state")
    return {"positions": pos, "parent": par, "children": ch, "boundaries": bd, "lifetime": life,
            "timer": int(sc[0]), "max_depth": int(sc[1]), "first_free": int(sc[2]), "used_slots": int(sc[3]),
            "max_slots": int(sc[4])}


class Octree:
    """The reference's AMR<T> host octree (AdaptiveMesh/AMR.h:118-294) without device data."""

    def __init__(self, slots: int):
        self.slots = slots
        h = VP()
        check(load().amr_octree_create(slots, ctypes.byref(h)), "amr_octree_create")
        self.h = h

    def add_node(self, parent: int, offset: int) -> None:
        check(load().amr_octree_add_node(self.h, parent, offset), "amr_octree_add_node")

    def remove_node(self, node: int) -> None:
        check(load().amr_octree_remove_node(self.h, node), "amr_octree_remove_node")

    def set_periodic(self, periodic: bool = True) -> None:
        """Periodic root: faces leaving the root take the domain on the opposite side."""
        check(load().amr_octree_set_periodic(self.h, 1 if periodic else 0), "amr_octree_set_periodic")

    def add_nodes(self, parents, offsets) -> None:
        """add_node for each (parent, offset) in order, as one batch (amr_octree_add_nodes)."""
        p, o = np.ascontiguousarray(parents, np.int32), np.ascontiguousarray(offsets, np.int32)
        check(load().amr_octree_add_nodes(self.h, p.ctypes.data, o.ctypes.data, p.size), "amr_octree_add_nodes")

    def remove_nodes(self, nodes) -> None:
        """remove_node for each node in order, as one batch (amr_octree_remove_nodes)."""
        n = np.ascontiguousarray(nodes, np.int32)
        check(load().amr_octree_remove_nodes(self.h, n.ctypes.data, n.size), "amr_octree_remove_nodes")

    def increment_timer(self) -> None:
        check(load().amr_octree_increment_timer(self.h), "amr_octree_increment_timer")

    def find_node_idx(self, packed: int, max_depth: int = 0xFFFFFFFF) -> int:
        return int(load().amr_octree_find_node_idx(self.h, packed, max_depth))

    def state(self) -> dict:
        return _state(load().amr_octree_state, self.h, self.slots)

    def close(self) -> None:
        if self.h:
            load().amr_octree_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Sim:
    """A reference plugin (BSSN_AMR_data or wave_AMR_data) driven through the C ABI."""

    # buffer ids of amr_sim_buffer
    OLD, NEW, RICCI, DMET, CHR = 0, 1, 2, 3, 4
    WAVE_DERIVS, WAVE_HESS, WAVE_CRIT = 3, 4, 5

    def __init__(self, cfg: Config, kind: int = SIM_BSSN, slots: int = 128, mode: int = MODE_GRAPH):
        self.cfg, self.kind, self.slots = cfg, kind, slots
        h = VP()
        check(load().amr_sim_create(ctypes.byref(cfg), kind, slots, mode, ctypes.byref(h)), "amr_sim_create")
        self.h = h

    def set_mode(self, mode: int) -> None:
        check(load().amr_sim_set_mode(self.h, mode), "amr_sim_set_mode")

    def add_node(self, parent: int, offset: int) -> None:
        check(load().amr_sim_add_node(self.h, parent, offset), "amr_sim_add_node")

    def remove_node(self, node: int) -> None:
        check(load().amr_sim_remove_node(self.h, node), "amr_sim_remove_node")

    def phase(self, phase: int) -> None:
        """One phase of the plugin's timestep loop (amr_sim_phase; PHASE_* constants)."""
        check(load().amr_sim_phase(self.h, phase), "amr_sim_phase")

    def set_octree(self, state: dict) -> None:
        """Replace the octree with arrays in the layout of state() (amr_sim_set_octree)."""
        arrays = [np.ascontiguousarray(state[k], t) for k, t in
                  (("positions", np.uint32), ("parent", np.int32), ("children", np.int32),
                   ("boundaries", np.uint64), ("lifetime", np.uint32))]
        sc = np.array([state["timer"], state["max_depth"], state["first_free"], state["used_slots"],
                       state["max_slots"]], np.uint32)
        check(load().amr_sim_set_octree(self.h, *[a.ctypes.data for a in arrays], sc.ctypes.data),
              "amr_sim_set_octree")

    def add_nodes(self, parents, offsets) -> None:
        """add_node for each (parent, offset) in order, as one batch: the new nodes are prolongated
        at the end, one launch per depth level (amr_sim_add_nodes)."""
        p, o = np.ascontiguousarray(parents, np.int32), np.ascontiguousarray(offsets, np.int32)
        check(load().amr_sim_add_nodes(self.h, p.ctypes.data, o.ctypes.data, p.size), "amr_sim_add_nodes")

    def remove_nodes(self, nodes) -> None:
        """remove_node for each node in order, as one batch (amr_sim_remove_nodes)."""
        n = np.ascontiguousarray(nodes, np.int32)
        check(load().amr_sim_remove_nodes(self.h, n.ctypes.data, n.size), "amr_sim_remove_nodes")

    def state(self) -> dict:
        return _state(load().amr_sim_octree_state, self.h, self.slots)

    def buffer(self, which: int, comp: int = 0) -> tuple[int, int]:
        """(device address, element count) of a simulation buffer."""
        p, n = VP(), U64()
        check(load().amr_sim_buffer(self.h, which, comp, ctypes.byref(p), ctypes.byref(n)), "amr_sim_buffer")
        return int(p.value or 0), int(n.value)

    def tensor(self, which: int, comp: int = 0, dtype=None):
        """A torch view of a simulation buffer (float32 or int32 for compressed words)."""
        import torch
        addr, n = self.buffer(which, comp)
        if dtype is None:
            floaty = which in (self.OLD, self.NEW) or (self.kind == SIM_BSSN and which == self.RICCI) or \
                (self.kind != SIM_BSSN and which == self.WAVE_CRIT)
            dtype = torch.float32 if floaty else torch.int32
        typestr = {torch.float32: "<f4", torch.int32: "<i4"}[dtype]

        class _Mem:
            __cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (addr, False), "version": 3}
        return torch.as_tensor(_Mem(), device="cuda")

    def copy_to_device(self, which: int, comp: int, host, count: int | None = None) -> None:
        """Asynchronous host -> buffer copy on the simulation's stream (host: pinned tensor/array)."""
        n = host.numel() if count is None and hasattr(host, "numel") else (count if count is not None else host.size)
        addr = host.data_ptr() if hasattr(host, "data_ptr") else host.ctypes.data
        check(load().amr_sim_copy_to_device(self.h, which, comp, addr, n), "amr_sim_copy_to_device")

    def copy_to_host(self, which: int, comp: int, host, count: int | None = None) -> None:
        """Asynchronous buffer -> host copy on the simulation's stream."""
        n = host.numel() if count is None and hasattr(host, "numel") else (count if count is not None else host.size)
        addr = host.data_ptr() if hasattr(host, "data_ptr") else host.ctypes.data
        check(load().amr_sim_copy_to_host(self.h, which, comp, addr, n), "amr_sim_copy_to_host")

    def copy_to_host_side(self, which: int, comp: int, host, count: int | None = None) -> None:
        """The same copy on the simulation's side stream (amr_sim_copy_to_host_side): overlaps later
        uploads of other buffers; later work touching this buffer waits for it."""
        n = host.numel() if count is None and hasattr(host, "numel") else (count if count is not None else host.size)
        addr = host.data_ptr() if hasattr(host, "data_ptr") else host.ctypes.data
        check(load().amr_sim_copy_to_host_side(self.h, which, comp, addr, n), "amr_sim_copy_to_host_side")

    def stage_to_device(self, which: int, comp: int, host, count: int | None = None) -> None:
        """Upload through the buffer's staging copy (amr_sim_stage_to_device): the host transfer
        overlaps work already enqueued; the buffer receives it after that work."""
        n = host.numel() if count is None and hasattr(host, "numel") else (count if count is not None else host.size)
        addr = host.data_ptr() if hasattr(host, "data_ptr") else host.ctypes.data
        check(load().amr_sim_stage_to_device(self.h, which, comp, addr, n), "amr_sim_stage_to_device")

    def snapshot_to_host(self, which: int, comp: int, host, count: int | None = None) -> None:
        """Download through a device snapshot (amr_sim_snapshot_to_host): the host transfer
        overlaps later work, which may overwrite the buffer at once."""
        n = host.numel() if count is None and hasattr(host, "numel") else (count if count is not None else host.size)
        addr = host.data_ptr() if hasattr(host, "data_ptr") else host.ctypes.data
        check(load().amr_sim_snapshot_to_host(self.h, which, comp, addr, n), "amr_sim_snapshot_to_host")

    @staticmethod
    def _many(items):
        n = len(items)
        which = np.array([it[0] for it in items], np.int32)
        comp = np.array([it[1] for it in items], np.int32)
        addr = (ctypes.c_void_p * max(n, 1))(*[it[2].data_ptr() if hasattr(it[2], "data_ptr") else it[2].ctypes.data
                                                for it in items])
        count = np.array([it[3] if len(it) > 3 else (it[2].numel() if hasattr(it[2], "numel") else it[2].size)
                          for it in items], np.uint64)
        return n, which, comp, addr, count

    def stage_many(self, items) -> None:
        """stage_to_device for several distinct buffers, [(which, comp, host[, count])], with one
        copy launch for all (amr_sim_stage_many)."""
        n, which, comp, addr, count = self._many(items)
        check(load().amr_sim_stage_many(self.h, n, which.ctypes.data, comp.ctypes.data, ctypes.addressof(addr),
                                        count.ctypes.data), "amr_sim_stage_many")

    def snapshot_many(self, items) -> None:
        """snapshot_to_host for several distinct buffers, [(which, comp, host[, count])], with one
        copy launch for all (amr_sim_snapshot_many)."""
        n, which, comp, addr, count = self._many(items)
        check(load().amr_sim_snapshot_many(self.h, n, which.ctypes.data, comp.ctypes.data, ctypes.addressof(addr),
                                           count.ctypes.data), "amr_sim_snapshot_many")

    def event_record(self, slot: int) -> None:
        check(load().amr_sim_event_record(self.h, slot), "amr_sim_event_record")

    def event_elapsed(self, first: int, second: int) -> float:
        ms = ctypes.c_float()
        check(load().amr_sim_event_elapsed(self.h, first, second, ctypes.byref(ms)), "amr_sim_event_elapsed")
        return float(ms.value)

    def save_checkpoint(self, directory: str) -> None:
        """Checkpoint into an existing directory (amr_sim_save)."""
        check(load().amr_sim_save(self.h, directory.encode()), "amr_sim_save")

    def load_checkpoint(self, directory: str) -> None:
        """Resume from a checkpoint of a simulation of the same kind and size (amr_sim_load)."""
        check(load().amr_sim_load(self.h, directory.encode()), "amr_sim_load")

    def timestep(self) -> None:
        check(load().amr_sim_timestep(self.h), "amr_sim_timestep")

    def copy_bounds(self) -> None:
        check(load().amr_sim_copy_bounds(self.h), "amr_sim_copy_bounds")

    @property
    def rng(self) -> int:
        s = ctypes.c_int32()
        check(load().amr_sim_rng(self.h, ctypes.byref(s)), "amr_sim_rng")
        return int(s.value)

    @rng.setter
    def rng(self, seed: int) -> None:
        check(load().amr_sim_set_rng(self.h, seed), "amr_sim_set_rng")

    @property
    def stream(self) -> int:
        s = VP()
        check(load().amr_sim_stream(self.h, ctypes.byref(s)), "amr_sim_stream")
        return int(s.value or 0)

    def set_stream(self, stream: int) -> None:
        """Run the simulation's work on a caller's stream (a cudaStream_t as an int; 0: its own)."""
        check(load().amr_sim_set_stream(self.h, stream or None), "amr_sim_set_stream")

    def synchronize(self) -> None:
        check(load().amr_sim_synchronize(self.h), "amr_sim_synchronize")

    @property
    def kernel_launches(self) -> int:
        return int(load().amr_sim_kernel_launches(self.h))

    def set_stencil_ctas(self, ctas: int) -> None:
        """CTAs of the fused BSSN derivative pass (0: the library's choice)."""
        check(load().amr_sim_set_stencil_ctas(self.h, ctas), "amr_sim_set_stencil_ctas")

    def autotune(self, reps: int = 3) -> dict:
        """Tune the fused BSSN pass's grid for the current octree (amr_sim_autotune); returns
        {active domains: CTAs}."""
        n = ctypes.c_uint32(0)
        check(load().amr_sim_autotune(self.h, reps, ctypes.byref(n)), "amr_sim_autotune")
        return self.tuned_shapes()

    def tuned_shapes(self) -> dict:
        cap = 64
        dom = (ctypes.c_uint32 * cap)()
        ctas = (ctypes.c_uint32 * cap)()
        cnt = ctypes.c_uint32(0)
        check(load().amr_sim_tuned_shapes(self.h, cap, dom, ctas, ctypes.byref(cnt)), "amr_sim_tuned_shapes")
        return {int(dom[i]): int(ctas[i]) for i in range(cnt.value)}

    # ---- evolution simulations (SIM_BSSN_EVOLVE, SIM_WAVE_RK4)
    OLD_STATE, NEW_STATE, STAGE, ACC, CONSTRAINTS, DERIVS = 0, 1, 2, 3, 4, 5

    def set_evolution(self, evolution) -> None:
        """Physics and gauge (amr_sim_set_evolution; an Evolution structure)."""
        check(load().amr_sim_set_evolution(self.h, ctypes.byref(evolution)), "amr_sim_set_evolution")

    def initial_data(self, data) -> None:
        """Analytic initial data on every live slot (amr_sim_initial_data; an InitialData structure)."""
        check(load().amr_sim_initial_data(self.h, ctypes.byref(data)), "amr_sim_initial_data")

    def constraint_norms(self, excision: float = 0.0) -> dict:
        """FP64 norms of the Hamiltonian and momentum constraints over the composite grid, leaving out
        cells within `excision` of a puncture."""
        out = (ctypes.c_double * 5)()
        check(load().amr_sim_constraint_norms(self.h, excision, out), "amr_sim_constraint_norms")
        return {"H_l2": out[0], "H_max": out[1], "M_l2": out[2], "M_max": out[3], "cells": int(out[4])}

    def tile_features(self):
        """(features [n][3][512], plain indicators [n]) as device tensors, and the leaf slots."""
        import torch
        import numpy as np
        n = U32()
        load().amr_sim_tile_features(self.h, None, None, None, 0, ctypes.byref(n))
        feats = torch.empty((max(n.value, 1), 3, 512), dtype=torch.float32, device="cuda")
        ind = torch.empty(max(n.value, 1), dtype=torch.float32, device="cuda")
        slots = np.zeros(max(n.value, 1), np.uint32)
        check(load().amr_sim_tile_features(self.h, feats.data_ptr(), ind.data_ptr(), slots.ctypes.data, n.value,
                                           ctypes.byref(n)), "amr_sim_tile_features")
        return feats[: n.value], ind[: n.value], slots[: n.value]

    def regrid(self, params, estimator=None) -> dict:
        """Refine / coarsen between timesteps (amr_sim_regrid): by the estimator judged by the plain
        criterion, or by the plain criterion alone."""
        stats = (U32 * 4)()
        check(load().amr_sim_regrid(self.h, estimator.h if estimator is not None else None, ctypes.byref(params),
                                    stats), "amr_sim_regrid")
        return {"refined": stats[0], "coarsened": stats[1], "overridden": stats[2], "leaves": stats[3]}

    def set_fault_injection(self, spin_limit: int = 0, withhold_plane: int = 0) -> None:
        """Failure-path test hook of the fused pass (amr_sim_set_fault_injection); (0, 0) is off."""
        check(load().amr_sim_set_fault_injection(self.h, spin_limit, withhold_plane), "amr_sim_set_fault_injection")

    def enable_kernel_timing(self, enable: bool = True) -> None:
        check(load().amr_sim_enable_kernel_timing(self.h, 1 if enable else 0), "amr_sim_enable_kernel_timing")

    def kernel_timing(self) -> tuple[float, int]:
        ms, n = ctypes.c_double(), U64()
        check(load().amr_sim_kernel_timing(self.h, ctypes.byref(ms), ctypes.byref(n)), "amr_sim_kernel_timing")
        return float(ms.value), int(n.value)

    def close(self) -> None:
        if self.h:
            load().amr_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
