"""Time the reference's own CUDA plugin (BSSN_AMR_data::timestep, BSSN.h:104-171) on this GPU.

Test infrastructure beside the reference-build library: it drives the reference's unmodified headers,
compiled for sm_103a into oracle/_ref/libamr_ref_<cfg>.so by oracle/build_ref.py, through the
harness entry points refd_bssn_*.  The workload is the benchmark's: a uniform octree of the given
depth (3: 512 leaf + 73 parent domains), domains of 16^3 cells with padding 3 (or the reference's
native 28^3 with padding 2), the six conformal-metric components seeded as in the tests.  Each
timestep is the reference's whole loop (copy_back, modify_nodes, predictor, copy_bounds,
corrector, increment_timer until the counter wraps), with the reference's own launches, streams
and synchronisations; it is timed by the wall clock between device synchronisations.  The
reference's ghost fill races on such trees, so its values are not checked here, only its speed.

usage: python oracle/time_reference_gpu.py [--size 16 --padding 3] [--depth 3] [--steps 20] [--warmup 3]
       python oracle/time_reference_gpu.py --plugin wave [--steps 20] [--warmup 3]   (SimpleWave, 28^3)
prints one JSON line: {"metric": "BSSN zone-cycles/s", "value": ..., "ms_per_step": ..., ...}
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

import cases  # noqa: E402
from oracle import reflib  # noqa: E402


def measure(n: int, p: int, depth: int, steps: int, warmup: int) -> dict:
    """zone-cycles/s of the reference's BSSN plugin on the uniform octree of `depth` (see above)."""
    import torch
    lib = reflib.load(f"n{n}p{p}")
    k = reflib.constants(lib)
    assert (k["size_domain"], k["padding_domain"]) == (n, p), k
    slots = sum(8 ** d for d in range(depth + 1))
    h = lib.refd_bssn_create(slots)

    class _Tree:
        def add_node(self, pa, off):
            lib.refd_bssn_add_node(h, pa, off)

        def state(self):
            return reflib.octree_state(lib.refd_bssn_octree_state, h, slots)
    tree = _Tree()
    cases.tree_uniform(tree, depth)
    st = tree.state()
    used, t = st["used_slots"], n + 2 * p
    xyz = cases.cell_coordinates(st["positions"], used, n, p, 100.0)
    metric = cases.metric_fields(xyz, 100.0, 500)
    del xyz

    class _Dev:
        def __init__(self, addr, count):
            self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<f4", "data": (addr, False),
                                             "version": 3}
    for which in (0, 1):
        for c in range(6):
            dst = torch.as_tensor(_Dev(lib.refd_bssn_field(h, which, c), used * t ** 3), device="cuda")
            dst.copy_(torch.from_numpy(metric[c]).cuda())
    torch.cuda.synchronize()
    for _ in range(warmup):
        assert lib.refd_bssn_timestep(h) == 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        assert lib.refd_bssn_timestep(h) == 0
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    leaves = 8 ** depth
    zones = leaves * n ** 3
    lib.refd_bssn_destroy(h)
    return {"metric": "BSSN zone-cycles/s", "value": zones * steps / sec, "unit": "zone-cycles/s",
            "ms_per_step": sec * 1e3 / steps, "steps": steps, "warmup": warmup,
            "impl": "reference CUDA plugin (BSSN_AMR_data::timestep), sm_103a",
            "workload": f"uniform depth-{depth} octree: {leaves} leaf + {used - leaves} parent domains of {n}^3, "
                        f"padding {p}"}


def wave_initial_field(n: int, p: int):
    """The SimpleWave runs' initial field on the root domain: a smooth seeded blob (the tests')."""
    import numpy as np
    xyz = cases.cell_coordinates(np.array([0], np.uint32), 1, n, p, 100.0)
    return cases.smooth_field(xyz, 100.0, 0, 77, noise=0.0) * np.float32(0.5)


def measure_wave(steps: int, warmup: int) -> dict:
    """zone-cycles/s of the reference's SimpleWave plugin (wave_AMR_data::timestep with its
    regridding, SimpleWave.h:189-262) at its native 28^3, padding 2: root + 8 children and the
    initial field of wave_initial_field, the tree then evolving as the plugin refines.  Each
    timestep is timed alone, between device synchronisations; its leaf zones are counted from the
    octree after it."""
    import numpy as np
    import torch
    n, p, slots = 28, 2, 128
    t = n + 2 * p
    lib = reflib.load("n28p2")
    h = lib.refd_wave_create(slots)
    f0 = wave_initial_field(n, p)

    class _Dev:
        def __init__(self, addr, count):
            self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<f4", "data": (addr, False),
                                             "version": 3}
    for which in (0, 1):
        torch.as_tensor(_Dev(lib.refd_wave_field(h, which), t ** 3), device="cuda").copy_(torch.from_numpy(f0).cuda())
    torch.cuda.synchronize()
    for c in range(8):
        lib.refd_wave_add_node(h, 0, c)
    assert lib.refd_wave_copy_bounds(h) == 0
    sec, zones = 0.0, 0
    for i in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        assert lib.refd_wave_timestep(h) == 0
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if i >= warmup:
            st = reflib.octree_state(lib.refd_wave_octree_state, h, slots)
            used = st["used_slots"]
            ch = st["children"][: used * 8].reshape(used, 8)
            leaves = int(sum(1 for s in range(used) if st["positions"][s] != 0xFFFFFFFF and (ch[s] == -1).all()))
            sec += dt
            zones += leaves * n ** 3
    lib.refd_wave_destroy(h)
    return {"metric": "SimpleWave zone-cycles/s", "value": zones / sec, "unit": "zone-cycles/s",
            "ms_per_step": sec * 1e3 / steps, "steps": steps, "warmup": warmup,
            "impl": "reference CUDA plugin (wave_AMR_data::timestep), sm_103a",
            "workload": "SimpleWave with regridding from root + 8 children, 28^3 domains, padding 2"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--plugin", default="bssn", choices=["bssn", "wave"])
    ap.add_argument("--size", type=int, default=16)
    ap.add_argument("--padding", type=int, default=3)
    ap.add_argument("--depth", type=int, default=3)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    args = ap.parse_args()
    if args.plugin == "wave":
        print(json.dumps(measure_wave(args.steps, args.warmup)))
    else:
        print(json.dumps(measure(args.size, args.padding, args.depth, args.steps, args.warmup)))


if __name__ == "__main__":
    main()
