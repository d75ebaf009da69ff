"""Benchmark: BSSN timesteps (reference semantics) on the uniform depth-3 octree, 16^3 domains.

Workload (the BSSN linear-gauge-wave configuration's octree): uniform refinement to depth 3
= 512 leaf domains + 73 covered parents = 585 slots, size_domain 16, padding 3 (6th-order FD,
as the reference couples FD order to the padding), root edge 100.  One step = one
BSSN_AMR_data::timestep(): 8 substeps of copy_back (restriction), predictor (metric gradients,
Hessians, g^kl d_k d_l g_ij, Christoffel symbols), copy_bounds (ghost fill), corrector.
Metric: zone-cycles/s = 512 * 16^3 leaf zones x steps / seconds (covered parents are overhead).

  value  device-resident state, graph replay of each timestep (inputs larger than L2: the
         state is 299 MB, so no L2 flush is needed between steps)
  e2e    the same metric through the C ABI with host buffers: every step uploads its input (the
         new metric; the old one is rewritten from it by the step's first phase) from pinned host
         memory and downloads new metric, gradients, Christoffel symbols and traces to pinned host
         memory, inside the timed region.  The transfers go through device staging copies
         (amr_sim_stage_to_device / amr_sim_snapshot_to_host): the next step's input is uploaded
         and this step's output downloaded while the next step computes.

  parity        the last end-to-end step recomputed on the host cores by the oracle from the same
                input and generator state: "ok" when every downloaded word equals it (the traces
                within 1e-4 of their scale: the device divides with the hardware reciprocal)
  cpu_baseline  the same stencils in FP64 without quantisation on all host cores (one whole
                timestep over every domain); cpu_fp32_port is the oracle's FP32 restatement

`--impl reference` times the reference path on the CPU: the reference has no CPU solver, so
this is the oracle's restatement of BSSN_AMR_data::timestep (bit-identical to the reference's
device build, OpenMP over planes), whole timesteps over every domain of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

N, P, OUTER, DEPTH = 16, 3, 100.0, 3
METRIC = "BSSN zone-cycles/s"
UNIT = "zone-cycles/s"
def workload(depth: int = DEPTH) -> str:
    return (f"BSSN fragment timestep (reference semantics), uniform depth-{depth} octree: {8 ** depth} leaf + "
            f"{sum(8 ** d for d in range(depth))} parent domains of {N}^3, padding {P}")


WORKLOAD = workload()


def progress(msg: str) -> None:
    print(f"[bench] {msg}", file=sys.stderr, flush=True)


def build_tree(o, depth: int = DEPTH):
    import cases
    cases.tree_uniform(o, depth)


def leaf_zones(st, n: int | None = None) -> int:
    used = st["used_slots"]
    ch = st["children"][: used * 8].reshape(used, 8)
    leaves = sum(1 for i in range(used) if st["positions"][i] != 0xFFFFFFFF and (ch[i] == -1).all())
    return leaves * (n or N) ** 3


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.samples, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "source": "fallback"}


def fused_kernel_bytes_per_domain() -> int:
    """Algorithmic HBM bytes of the fused BSSN stencil per domain: the six metric components'
    interior plus face ghosts read once (g = (N^3 + 6 p N^2) / N^3), and 18 inner-layout outputs
    written (6 compressed gradients, 6 traces, 6 compressed Christoffel symbols)."""
    return 6 * 4 * (N ** 3 + 6 * P * N ** 2) + 18 * 4 * N ** 3


def fused_restriction_bytes_per_leaf() -> int:
    """Added to a leaf domain in the predictor pass, which also performs its restriction: the six
    old fields' padded cubes written (the padded planes it reads anyway come from new)."""
    return 6 * 4 * (N + 2 * P) ** 3


def golden_tree(depth: int) -> dict:
    """The uniform octree's arrays as the reference's own host code (AMR<T>, AMR.h:118-294) builds
    them, from the committed fixture (tests/golden/gen_host_golden.py), so that the CPU legs need
    neither this library nor the reference-build library to lay out their work."""
    import numpy as np
    hg = np.load(os.path.join(ROOT, "tests", "golden", "host_golden.npz"))
    key = f"tree/uniform{depth}"
    if f"{key}/positions" not in hg.files:
        raise ValueError(f"no fixture of the uniform depth-{depth} tree")
    sc = hg[f"{key}/scalars"]
    return {"positions": hg[f"{key}/positions"], "children": hg[f"{key}/children"],
            "boundaries": hg[f"{key}/boundaries"], "used_slots": int(sc[3]), "max_depth": int(sc[1])}


class CpuTimestep:
    """One whole BSSN_AMR_data::timestep (8 substeps, every slot: 512 leaves and 73 parents) on the
    host cores through the oracle (OpenMP over planes): `fp32` is the restatement that is
    bit-identical to the reference's device build, `fp64` the same stencils in double precision
    without quantisation (oracle/fp64_path.c)."""

    def __init__(self, depth: int, threads: int | None = None):
        import numpy as np
        from oracle import oracle as orc
        import cases
        self.np, self.orc, self.L = np, orc, orc.lib()
        if threads:
            self.L.orc_set_num_threads(threads)
        self.cores = int(self.L.orc_num_threads())
        self.st = st = golden_tree(depth)
        self.used = used = st["used_slots"]
        self.zones = 8 ** depth * N ** 3
        xyz = cases.cell_coordinates(st["positions"], used, N, P, OUTER)
        self.metric = cases.metric_fields(xyz, OUTER, 500)
        self.c = orc.cfg(N, P, OUTER)

    def fp32(self, new6=None, seed: int = 12894712) -> tuple[float, dict]:
        np, orc, st = self.np, self.orc, self.st
        inner = self.used * N ** 3
        src = new6 if new6 is not None else self.metric
        arrays = {"old": [m.copy() for m in src], "new": [m.copy() for m in src],
                  "dmet": [np.zeros(inner, np.uint32) for _ in range(6)],
                  "chr": [np.zeros(inner, np.uint32) for _ in range(6)],
                  "ricci": [np.zeros(inner, np.float32) for _ in range(6)]}
        pp = {k: orc.ptrs(v) for k, v in arrays.items()}
        timer, rng = ctypes.c_uint32(0), ctypes.c_int32(seed)
        t0 = time.perf_counter()
        self.L.orc_bssn_timestep(ctypes.byref(self.c), pp["old"], pp["new"], pp["dmet"], pp["chr"], pp["ricci"],
                                 orc.P(st["positions"]), orc.P(st["children"]), orc.P(st["boundaries"]), self.used,
                                 st["max_depth"], ctypes.byref(timer), ctypes.byref(rng), 0, self.used)
        return time.perf_counter() - t0, arrays

    def fp64(self) -> float:
        np, orc, st = self.np, self.orc, self.st
        inner = self.used * N ** 3
        arrays = [[m.astype(np.float64) for m in self.metric], [m.astype(np.float64) for m in self.metric],
                  [np.zeros(inner * 3) for _ in range(6)], [np.zeros(inner * 3) for _ in range(6)],
                  [np.zeros(inner) for _ in range(6)]]
        pp = [orc.ptrs(a) for a in arrays]
        timer = ctypes.c_uint32(0)
        t0 = time.perf_counter()
        self.L.orc_bssn_timestep_f64(ctypes.byref(self.c), *pp, orc.P(st["positions"]), orc.P(st["children"]),
                                     orc.P(st["boundaries"]), self.used, st["max_depth"], ctypes.byref(timer))
        return time.perf_counter() - t0


def config_dict(depth: int, world: int) -> dict:
    """The workload description both arms print (identical keys and values at the same N)."""
    return {"workload": workload(depth), "leaf_domains": 8 ** depth * world, "zones_per_domain": N ** 3,
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "state 299 MB > L2 129 MB, no flush" if (depth, N, P) == (3, 16, 3) else "no flush"}


def reference_arm(args) -> None:
    """The reference's path on the host cores: the oracle's restatement of BSSN_AMR_data::timestep,
    bit-identical to the reference's device build (the reference has no CPU solver of its own),
    whole timesteps over every domain on all host threads.  Steps that would not finish within
    about three minutes are not run, and `steps` reports the steps timed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    port = CpuTimestep(args.depth)
    t_first, _ = port.fp32()                      # also the first warm-up step
    budget = 180.0
    warm = max(0, min(args.warmup - 1, int(budget * 0.2 / t_first)))
    for _ in range(warm):
        port.fp32()
    steps = max(1, min(args.steps, int((budget - (warm + 1) * t_first) / t_first)))
    times = [port.fp32()[0] for _ in range(steps)]
    total = sum(times)
    v = port.zones * steps / total
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": warm + 1, "ms_per_step": total / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(args.depth, args.gpus), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": port.cores, "kind": "port",
                             "sample": f"{steps} whole timesteps (8 substeps each) over all {port.used} domains "
                                       f"({port.zones // N ** 3} leaves), FP32 restatement"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if steps < args.steps:
        line["steps_requested"] = args.steps
    # For comparison only (not this arm's value): the reference's own CUDA plugin on this GPU, its
    # headers compiled for sm_103a into the reference-build library, on the same workload
    try:
        import torch
        if torch.cuda.is_available():
            from oracle import time_reference_gpu
            line["reference_gpu"] = time_reference_gpu.measure(N, P, args.depth, steps=10, warmup=2)
    except Exception as e:  # no reference-build library for this size, or no reference headers staged
        line["reference_gpu"] = {"unavailable": f"{type(e).__name__}: {e}"[:200]}
    print(json.dumps(line))


def wave_line(args) -> None:
    """SimpleWave (wave_AMR_data::timestep with its regridding) at 28^3, padding 2, from root + 8
    children and a smooth seeded blob: each timestep timed alone between device synchronisations
    (the plugin reads its criterion back to the host every substep), its leaf zones counted after
    it.  The reference plugin's figure on the same run comes from its own headers built for this
    GPU (the timing script beside the reference-build library)."""
    import numpy as np
    import torch
    import adaptivemesh_gb300 as am
    import cases
    n, p = 28, 2
    t = n + 2 * p
    sim = am.Sim(am.Config(n, p, OUTER), am.SIM_WAVE, slots=128, mode=am.MODE_BATCHED)
    xyz = cases.cell_coordinates(np.array([0], np.uint32), 1, n, p, OUTER)
    f0 = cases.smooth_field(xyz, OUTER, 0, 77, noise=0.0) * np.float32(0.5)
    for which in (am.Sim.OLD, am.Sim.NEW):
        sim.tensor(which)[: t ** 3].copy_(torch.from_numpy(f0).cuda())
    torch.cuda.synchronize()
    for c in range(8):
        sim.add_node(0, c)
    sim.copy_bounds()
    sec, zones = 0.0, 0
    for i in range(args.warmup + args.steps):
        sim.synchronize()
        t0 = time.perf_counter()
        sim.timestep()
        sim.synchronize()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            sec += dt
            zones += leaf_zones(sim.state(), n)
    sim.close()
    print(json.dumps({"metric": "SimpleWave zone-cycles/s", "value": zones / sec, "unit": UNIT, "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps,
                      "higher_is_better": True, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": "SimpleWave with regridding from root + 8 children, 28^3 domains, "
                                             "padding 2", "mode": "batched"}}))


def zone_cycles_per_root_step(st, n: int) -> int:
    """Leaf zones advanced per root step: a leaf at depth d takes 2^d steps (2:1 subcycling)."""
    used, pos, ch = st["used_slots"], st["positions"], st["children"]
    total = 0
    for s in range(used):
        p = int(pos[s])
        if p != 0xFFFFFFFF and all(c == -1 for c in ch[8 * s:8 * s + 8]):
            total += n ** 3 << (p >> 27)
    return total


class CpuEvolution:
    """The FP64 oracle of the BSSN evolution (oracle/bssn_evolve.c, OpenMP over domains) on the
    gauge-wave octree: one finest substep timed on all host cores."""

    def __init__(self, depth: int, n: int = 16):
        import numpy as np
        from oracle import oracle as orc
        self.np, self.orc, self.L = np, orc, orc.lib()
        st = golden_tree(depth)
        used = st["used_slots"]
        bd = np.zeros(used * 6, np.uint64)
        self.L.orc_periodic_boundaries(orc.P(st["positions"]), orc.P(st["children"]), used, orc.P(bd))
        st["boundaries"] = bd
        self.st, self.used, self.n = st, used, n
        e = orc.Evo()
        e.n, e.p, e.outer_size, e.physics, e.slicing, e.shift = n, 3, 1.0, 0, 0, 0
        e.eta, e.ko_sigma, e.cfl, e.chi_floor = 2.0, 0.1, 0.25, 1e-6
        e.id_kind, e.amplitude, e.wavelength = 1, 0.01, 1.0
        self.e = e
        t = n + 6
        padded, inner = used * t ** 3, used * n ** 3
        self.old = [np.zeros(padded) for _ in range(24)]
        self.L.orc_evo_initial_data(ctypes.byref(e), orc.P(orc.ptrs(self.old)), orc.P(st["positions"]), used)
        self.new = [f.copy() for f in self.old]
        self.stage = [f.copy() for f in self.old]
        self.acc = [np.zeros(inner) for _ in range(24)]
        self.cores = int(self.L.orc_num_threads())
        self.zones = sum(1 for s in range(used) if all(c == -1 for c in st["children"][8 * s:8 * s + 8])) * n ** 3

    def substep(self) -> float:
        orc, st = self.orc, self.st
        timer = ctypes.c_uint32(0)
        t0 = time.perf_counter()
        self.L.orc_evo_timestep(ctypes.byref(self.e), orc.P(orc.ptrs(self.old)), orc.P(orc.ptrs(self.new)),
                                orc.P(orc.ptrs(self.stage)), orc.P(orc.ptrs(self.acc)), orc.P(st["positions"]),
                                orc.P(st["children"]), orc.P(st["boundaries"]), self.used, st["max_depth"],
                                ctypes.byref(timer))
        return time.perf_counter() - t0


def evolution_report(cpu: bool = True, estimator_path: str | None = None, case: str = "all",
                     batched_mode: str = "graph", plain: bool = True, gw_depth: int = 3, gw_steps: int = 24) -> dict:
    """The full BSSN evolution's throughput (zone-cycles/s: leaf zones x steps at their own level)
    at fixed constraint error, batched (CUDA-graph replay of whole root steps) against the plain
    per-domain launches, which compute the same state bit for bit:

      gauge_wave  the linear gauge wave, A = 1e-2, L = 1, periodic box, uniform depth 3 (512 domains
                  of 16^3 = 128^3 zones), 1+log slicing, zero shift: 25 root steps (200 finest steps)
                  batched, the first untimed; 2 root steps plain, the first untimed; H and M L2 after
                  the 200 steps (FP64 reductions).  FP64 CPU baseline: one substep of the oracle.
      binary      binary Brill-Lindquist punctures (m = 0.5 at x = +-3, seeded jitter 0.01), 16^3
                  domains, root edge 32, refined around the punctures to depth 4; regridded every
                  8 root steps (before steps 0 and 8) up to depth 5 by the learned estimator judged
                  by the plain criterion ('learned') or by the plain criterion alone ('plain'),
                  both aiming at the same error tolerance (the plain indicator calibrated to an
                  error estimate on the estimator's training samples); 16 root steps batched,
                  regrids and graph recaptures included in the time; the plain per-domain launches
                  timed over one root step on the plain-criterion tree.  H and M L2 outside r = 1
                  of each puncture after the run.
      single_puncture  one puncture nested to depth 6 (2 121 domains of 16^3), batched against the
                  plain per-domain launches (single_puncture_report)
      sweep       random octrees of 16^3 and 32^3 domains with 1-4 punctures (sweep_report)"""
    import adaptivemesh_gb300 as am
    from adaptivemesh_gb300 import estimator as E
    import cases
    out = {}
    bmode = {"graph": am.MODE_GRAPH, "batched": am.MODE_BATCHED}[batched_mode]
    if case in ("all", "gauge_wave"):
        out["gauge_wave"] = gauge_wave_report(am, cases, bmode, cpu, plain, gw_depth, gw_steps)
    if case in ("all", "single"):
        out["single_puncture"] = single_puncture_report(am, E, bmode, plain)
    if case in ("all", "binary"):
        out["binary"] = binary_report(am, E, estimator_path, bmode, plain)
    if case in ("all", "sweep"):
        out["sweep"] = sweep_report(am, cases, bmode)
    if case == "pareto":
        out["pareto"] = pareto_report(am, E, estimator_path, bmode)
    return out


def gauge_wave_report(am, cases, bmode: int, cpu: bool, plain: bool, depth: int = 3, steps_batched: int = 24) -> dict:
    gw = {}
    arms = [("batched", bmode, steps_batched)] + ([("plain", am.MODE_PLAIN, 1)] if plain else [])
    for name, mode, steps in arms:
        progress(f"evolution: gauge wave, {name}")
        sim = am.Sim(am.Config(16, 3, 1.0), am.SIM_BSSN_EVOLVE, slots=sum(8 ** d for d in range(depth + 1)), mode=mode)
        cases.tree_uniform(sim, depth)
        sim.set_evolution(am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=0, ko_sigma=0.1, cfl=0.25, periodic=1))
        sim.initial_data(am.InitialData(kind=am.ID_GAUGE_WAVE, amplitude=1e-2, wavelength=1.0))
        tuned = sim.autotune(3) if mode != am.MODE_PLAIN else None   # the derivative pass's slab depth
        sim.timestep()                       # warm-up (graph capture)
        sim.synchronize()
        l0 = sim.kernel_launches
        sim.event_record(0)
        for _ in range(steps):
            sim.timestep()
        sim.event_record(1)
        sim.synchronize()
        ms = sim.event_elapsed(0, 1)
        zc = zone_cycles_per_root_step(sim.state(), 16) * steps
        gw[name] = {"value": zc / (ms / 1e3), "ms_per_root_step": ms / steps, "root_steps": steps,
                    "gpu_launches_per_root_step": (sim.kernel_launches - l0) / steps}
        if tuned:
            gw[name]["derivative_slab_planes"] = next(iter(tuned.values()))
        if name == "batched":
            gw[name].update({k: v for k, v in sim.constraint_norms().items() if k != "cells"})
            gw[name]["finest_steps"] = (1 << depth) * (steps + 1)
            gbs = evolution_bytes_per_root_step(sim.state(), 16) / (ms / steps / 1e3) / 1e9
            pk = peaks()
            gw[name]["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
                                    "frac": gbs / pk["hbm_gbs"], "peak_source": pk["source"],
                                    "bytes": "algorithmic bytes of the whole root step (bench.evolution_bytes_per_root_step)"}
        sim.close()
    if plain:
        gw["speedup"] = gw["batched"]["value"] / gw["plain"]["value"]
    if cpu:
        try:
            progress("evolution: FP64 CPU baseline")
            ce = CpuEvolution(depth)
            sec = ce.substep()
            gw["cpu_fp64"] = {"value": ce.zones / sec, "unit": UNIT, "cores": ce.cores, "kind": "port",
                              "sample": f"one finest substep of the FP64 oracle over all {ce.used} domains, "
                                        f"{sec:.2f} s"}
        except Exception as e:   # no fixture or oracle library
            gw["cpu_fp64"] = {"unavailable": f"{type(e).__name__}: {e}"[:200]}
    return gw


def evolution_bytes_per_root_step(st, n: int, p: int = 3) -> float:
    """Algorithmic HBM bytes of one root step of the BSSN evolution: every evolved domain active at a
    substep (covered parents included) does, per RK stage, a derivative pass (24 fields read once,
    93 derivative planes written: 117 planes of n^3 floats) and an update (93 derivative planes and
    the 24 fields read, plus the step-start values in stages 2-3 and the accumulator in stages 2-4;
    the 24 fields written, plus the accumulator in stages 1-3: 165 + 213 + 213 + 165 planes over
    the four stages), four ghost fills (every ghost cell of the 24 fields read once and written
    once) and one restriction (the padded state of the 24 fields copied)."""
    t = n + 2 * p
    used, pos, md = st["used_slots"], st["positions"], st["max_depth"]
    per_domain = (4 * 117 + 165 + 213 + 213 + 165) * n ** 3 * 4 + 4 * (t ** 3 - n ** 3) * 24 * 8 + t ** 3 * 24 * 8
    active = 0
    for k in range(used):
        q = int(pos[k])
        if q != 0xFFFFFFFF:
            active += 1 << (q >> 27)   # a depth-d domain is active at 2^d of the 2^max_depth substeps
    return float(active * per_domain)


def leaf_zone_cycles_of_substep(st, n: int, s: int) -> int:
    """Leaf zones that advance at substep s (a depth-d leaf advances when s is a multiple of
    2^(max_depth - d))."""
    used, pos, ch, md = st["used_slots"], st["positions"], st["children"], st["max_depth"]
    total = 0
    for k in range(used):
        p = int(pos[k])
        if p != 0xFFFFFFFF and all(c == -1 for c in ch[8 * k:8 * k + 8]) and s % (1 << (md - (p >> 27))) == 0:
            total += n ** 3
    return total


def single_puncture_report(am, E, bmode: int, plain: bool) -> dict:
    """A single Brill-Lindquist puncture (m = 1, seeded offset |d| < 0.05) on [-64, 64]^3, refined
    around it to depth 6 with shells of neighbours (2 121 domains of 16^3, 1 856 leaves), 1+log
    slicing and the Gamma-driver (eta = 2).  Batched: the derivative pass's slab depth autotuned,
    one root step (64 finest substeps) replayed from a CUDA graph after a warm-up root step.  Both
    forms also run the first two substeps phase by phase (every domain active, then the finest
    level alone), the plain per-domain launches against the batched ones, which compute the same
    state bit for bit; a whole plain root step would take about a minute."""
    import numpy as np
    rng = np.random.default_rng(2024)
    d = rng.normal(size=3)
    d = d / np.linalg.norm(d) * rng.uniform(0.0, 0.05)
    punct = [(1.0, tuple(float(v) for v in d))]
    rep = {"puncture": punct[0][1]}
    phases = (am.PHASE_COPY_BACK, am.PHASE_MODIFY_NODES, am.PHASE_PREDICTOR, am.PHASE_COPY_BOUNDS,
              am.PHASE_CORRECTOR, am.PHASE_INCREMENT_TIMER)
    arms = [("batched", bmode)] + ([("plain", am.MODE_PLAIN)] if plain else [])
    for name, mode in arms:
        progress(f"evolution: single puncture, {name}")
        sim = am.Sim(am.Config(16, 3, 128.0), am.SIM_BSSN_EVOLVE, slots=2200, mode=mode)
        E.refine_around(sim, [punct[0][1]], 6, 128.0, margin=3.25)
        sim.set_evolution(am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=1, eta=2.0, ko_sigma=0.1, cfl=0.25))
        sim.initial_data(am.InitialData(kind=am.ID_BRILL_LINDQUIST, punctures=punct))
        st = sim.state()
        arm = {}
        if mode != am.MODE_PLAIN:
            arm["derivative_slab_planes"] = next(iter(sim.autotune(3).values()))
            sim.timestep()                   # warm-up (graph capture)
            sim.synchronize()
            sim.event_record(0)
            sim.timestep()
            sim.event_record(1)
            sim.synchronize()
            ms = sim.event_elapsed(0, 1)
            arm.update({"value": zone_cycles_per_root_step(st, 16) / (ms / 1e3), "ms_per_root_step": ms})
            arm.update({k: v for k, v in sim.constraint_norms(1.0).items() if k != "cells"})
        sim.synchronize()
        sim.event_record(0)
        for _ in range(2):                   # substeps 0 and 1, phase by phase
            for ph in phases:
                sim.phase(ph)
        sim.event_record(1)
        sim.synchronize()
        ms2 = sim.event_elapsed(0, 1)
        zc2 = leaf_zone_cycles_of_substep(st, 16, 0) + leaf_zone_cycles_of_substep(st, 16, 1)
        arm["first_two_substeps"] = {"value": zc2 / (ms2 / 1e3), "ms": ms2}
        rep[name] = arm
        rep["domains"] = st["used_slots"]
        rep["leaves"] = sum(1 for k in range(st["used_slots"]) if st["positions"][k] != 0xFFFFFFFF and
                            all(c == -1 for c in st["children"][8 * k:8 * k + 8]))
        sim.close()
    if plain:
        rep["speedup_first_two_substeps"] = rep["batched"]["first_two_substeps"]["value"] / rep["plain"]["first_two_substeps"]["value"]
    return rep


def sweep_report(am, cases, bmode: int) -> list:
    """The throughput sweep's octrees: seeded Bernoulli(0.3) refinement per level (cases.tree_random)
    to depth 6 with 16^3 domains (1 569 domains) and to depth 5 with 32^3 domains (1 265), root edge
    64, holding 1-4 Brill-Lindquist punctures of seeded masses in [0.2, 1] and positions in
    [-8, 8]^3, 1+log slicing and the Gamma-driver: slab depth autotuned, one root step of batched
    launches (each a few seconds long, so launch overhead is negligible and no graph is captured)."""
    import numpy as np
    out = []
    bmode = am.MODE_BATCHED
    for n, depth, seed, slots in ((16, 6, 3, 1569), (32, 5, 25, 1265)):
        progress(f"evolution: sweep, {n}^3 domains")
        rng = np.random.default_rng(100 + seed)
        punct = [(float(rng.uniform(0.2, 1.0)), tuple(float(v) for v in rng.uniform(-8.0, 8.0, 3)))
                 for _ in range(1 + seed % 4)]
        sim = am.Sim(am.Config(n, 3, 64.0), am.SIM_BSSN_EVOLVE, slots=slots, mode=bmode)
        cases.tree_random(sim, depth, 0.3, seed)
        sim.set_evolution(am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=1, eta=2.0, ko_sigma=0.1, cfl=0.25))
        sim.initial_data(am.InitialData(kind=am.ID_BRILL_LINDQUIST, punctures=punct))
        st = sim.state()
        zs = next(iter(sim.autotune(2).values()))
        sim.synchronize()
        sim.event_record(0)
        sim.timestep()
        sim.event_record(1)
        sim.synchronize()
        ms = sim.event_elapsed(0, 1)
        leaves = sum(1 for k in range(st["used_slots"]) if st["positions"][k] != 0xFFFFFFFF and
                     all(c == -1 for c in st["children"][8 * k:8 * k + 8]))
        row = {"size_domain": n, "max_depth": st["max_depth"], "domains": st["used_slots"], "leaves": leaves,
               "punctures": len(punct), "derivative_slab_planes": zs,
               "value": zone_cycles_per_root_step(st, n) / (ms / 1e3), "ms_per_root_step": ms}
        row.update({k: v for k, v in sim.constraint_norms(1.0).items() if k != "cells"})
        out.append(row)
        sim.close()
    return out


def binary_run(am, E, punct, params, net, bmode: int, steps: int = 16) -> tuple[dict, object]:
    """One binary-puncture run: regrid every 8 root steps (before steps 0 and 8) by `net` judged by
    the plain criterion, or by the plain criterion alone (net None); the simulation is returned open."""
    sim = E.build_sim(16, 32.0, punct, 4, mode=bmode)
    sim.timestep()                                   # warm-up
    sim.synchronize()
    zc, regrids = 0, []
    t0 = time.perf_counter()
    for step in range(steps):
        if step % 8 == 0:
            regrids.append(sim.regrid(params, net))
            if bmode != am.MODE_PLAIN:
                sim.autotune(2)   # the derivative pass's slab depth for the new tree
        zc += zone_cycles_per_root_step(sim.state(), 16)
        sim.timestep()
    sim.synchronize()
    sec = time.perf_counter() - t0
    norms = sim.constraint_norms(1.0)
    return ({"value": zc / sec, "ms_per_root_step": sec * 1e3 / steps, "root_steps": steps,
             "leaves": regrids[-1]["leaves"], "regrids": regrids,
             **{k: v for k, v in norms.items() if k != "cells"}}, sim)


def regrid_params(am, tol: float, a: float, b: float):
    """Thresholds aiming at log10 error `tol`: the network's directly, the plain indicator's through
    the calibration log10(error) ~ a + b log10(indicator); coarsening 1.5 decades below."""
    return am.Regrid(refine_threshold=float(10 ** ((tol - a) / b)), coarsen_threshold=float(10 ** ((tol - 1.5 - a) / b)),
                     learned_refine=tol, learned_coarsen=tol - 1.5, judge_factor=4.0, max_depth=5, min_depth=2)


def pareto_report(am, E, estimator_path, bmode: int) -> dict:
    """Leaves and constraint norms of both criteria over a range of error tolerances."""
    est, (a, b), meta = E.load_trained(estimator_path or os.path.join(ROOT, "adaptivemesh_gb300", "data",
                                                                      "estimator_binary16.npz"))
    punct = E.binary_punctures(1001)
    out = []
    q50, q80, q90 = meta["target_quantiles"]
    for tol in (q50, 0.5 * (q50 + q80), q80, q90):   # the training targets' percentiles
        row = {"log10_tolerance": tol}
        for name, net in (("learned", est), ("plain_criterion", None)):
            progress(f"pareto: tolerance {tol:.2f}, {name}")
            r, sim = binary_run(am, E, punct, regrid_params(am, tol, a, b), net, bmode)
            sim.close()
            row[name] = {k: r[k] for k in ("leaves", "H_l2", "M_l2", "value")}
        out.append(row)
    est.close()
    return {"rows": out}


def binary_report(am, E, estimator_path, bmode: int, plain: bool) -> dict:
    path = estimator_path or os.path.join(ROOT, "adaptivemesh_gb300", "data", "estimator_binary16.npz")
    if os.path.exists(path):
        est, (a, b), meta = E.load_trained(path)
        origin = "trained weights " + os.path.relpath(path, ROOT)
    else:
        progress("evolution: training the estimator (no trained weights found)")
        est, (a, b), meta = E.train_default(n_seeds=10, held_out=2, epochs=40)
        origin = "trained in this run on 8 seeded configurations"
    tol = meta["target_quantiles"][1]            # log10 error tolerance: the training targets' 80th percentile
    params = regrid_params(am, tol, a, b)
    punct = E.binary_punctures(1001)
    bi = {"estimator": origin, "log10_error_tolerance": tol, "calibration": [a, b],
          "estimator_val_mse": {"network": meta["val_mse_network"],
                                "calibrated_indicator": meta["val_mse_calibrated_indicator"]}}
    for name, net in (("learned", est), ("plain_criterion", None)):
        progress(f"evolution: binary punctures, {name}")
        bi[name], sim = binary_run(am, E, punct, params, net, bmode)
        if net is None and plain:   # the plain per-domain launches on this tree: one root step
            progress("evolution: binary punctures, plain per-domain launches")
            st = sim.state()
            sim.set_mode(am.MODE_PLAIN)
            sim.synchronize()
            z1 = zone_cycles_per_root_step(st, 16)
            sim.event_record(0)
            sim.timestep()
            sim.event_record(1)
            sim.synchronize()
            ms = sim.event_elapsed(0, 1)
            bi["plain_launches"] = {"value": z1 / (ms / 1e3), "ms_per_root_step": ms, "root_steps": 1,
                                    "leaves": bi[name]["leaves"]}
        sim.close()
    est.close()
    if plain:
        bi["speedup_learned_batched_vs_plain_launches"] = bi["learned"]["value"] / bi["plain_launches"]["value"]
    return bi


def evolution_line(args) -> None:
    """--plugin evolution: the evolution's report as its own line."""
    rep = evolution_report(cpu=not args.no_cpu_baseline, estimator_path=args.estimator, case=args.evo_case,
                           batched_mode="batched" if args.mode == "batched" else "graph", plain=not args.no_plain,
                           gw_depth=args.evo_depth, gw_steps=args.evo_steps)
    bi = rep.get("binary")
    print(json.dumps({"metric": "BSSN zone-cycles/s at fixed constraint error, batched+learned vs plain",
                      "value": bi["learned"]["value"] if bi else None, "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
                      "dtype": "f32", "data": "synthetic",
                      "config": {"workload": "full BSSN evolution, binary Brill-Lindquist punctures with learned "
                                             "regridding (and the gauge wave on 128^3)"},
                      "evolution": rep}))


def main() -> None:
    global N, P
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="graph", choices=["plain", "batched", "graph"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--depth", type=int, default=DEPTH, help="uniform octree depth (3 = the benchmark workload)")
    ap.add_argument("--size", type=int, default=N, help="size_domain (16 = the benchmark workload; 8, 16, 28, 32)")
    ap.add_argument("--padding", type=int, default=P, help="padding_domain (3 = the benchmark workload)")
    ap.add_argument("--plugin", default="bssn", choices=["bssn", "wave", "evolution"],
                    help="wave: time the SimpleWave plugin instead (an extra line, not the benchmark); "
                         "evolution: the full BSSN evolution's report alone")
    ap.add_argument("--no-evolution", action="store_true", help="leave out the evolution's report")
    ap.add_argument("--no-autotune", action="store_true", help="time the library's launch-shape rule, untuned")
    ap.add_argument("--estimator", default=None, help="trained estimator weights (.npz) for the evolution's report")
    ap.add_argument("--evo-case", default="all", choices=["all", "gauge_wave", "single", "binary", "sweep", "pareto"],
                    help="--plugin evolution: the configurations to run")
    ap.add_argument("--no-plain", action="store_true", help="--plugin evolution: leave out the plain launches")
    ap.add_argument("--evo-depth", type=int, default=3, help="--plugin evolution: the gauge wave's uniform octree depth")
    ap.add_argument("--evo-steps", type=int, default=24, help="--plugin evolution: the gauge wave's timed root steps")
    args = ap.parse_args()
    N, P = args.size, args.padding
    if args.plugin == "wave":
        wave_line(args)
        return
    if args.plugin == "evolution":
        evolution_line(args)
        return
    if args.impl == "reference":
        reference_arm(args)
        return

    import numpy as np
    import torch
    import adaptivemesh_gb300 as am
    import cases

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    mode = {"plain": am.MODE_PLAIN, "batched": am.MODE_BATCHED, "graph": am.MODE_GRAPH}[args.mode]
    cfg = am.Config(N, P, OUTER)
    sim = am.Sim(cfg, am.SIM_BSSN, slots=sum(8 ** d for d in range(args.depth + 1)), mode=mode)
    build_tree(sim, args.depth)
    sim.synchronize()
    st = sim.state()
    used, md = st["used_slots"], st["max_depth"]
    zones = leaf_zones(st)
    xyz = cases.cell_coordinates(st["positions"], used, N, P, OUTER)
    metric = cases.metric_fields(xyz, OUTER, 500)
    T3 = cfg.total ** 3
    padded, inner = used * T3, used * N ** 3
    # host buffers (page-locked) of the state and of the step's outputs; every copy goes through
    # the C ABI on the simulation's stream
    # A timestep's inputs are the six `new` fields: its first phase (restriction at substep 0, when
    # every depth is active) rewrites every cell of every live domain's `old` field from them
    # (tests/test_gpu_plugins.py checks that poisoning `old` changes nothing).
    ins = [(am.Sim.NEW, k) for k in range(6)]
    outs = [(am.Sim.NEW, k, padded) for k in range(6)] + \
           [(w, k, inner) for w in (am.Sim.DMET, am.Sim.CHR, am.Sim.RICCI) for k in range(6)]
    h_in = [torch.from_numpy(metric[k]).pin_memory() for _, k in ins]
    h_out = [torch.empty(n, dtype=torch.float32, pin_memory=True) for _, _, n in outs]
    h2d = sum(t.numel() * 4 for t in h_in)
    d2h = sum(t.numel() * 4 for t in h_out)

    def upload():
        # host -> staging at once (overlapping the work enqueued so far), staging -> buffers on the
        # simulation's stream after that work, one copy launch for all
        sim.stage_many([(w, k, h) for (w, k), h in zip(ins, h_in)])

    def download():
        # buffers -> staging on the simulation's stream (one launch), staging -> host overlapping
        # later work
        sim.snapshot_many([(w, k, h) for (w, k, n), h in zip(outs, h_out)])

    upload()
    sim.synchronize()

    def barrier():
        sim.synchronize()
        if dist is not None:
            dist.barrier()

    tune = None
    if not args.no_autotune and mode != am.MODE_PLAIN:
        # the same timesteps on the library's launch-shape rule first, then the fused pass's grid
        # tuned for this octree (amr_sim_autotune), which the timed region below uses
        progress("autotune")
        for _ in range(args.warmup):
            sim.timestep()
        barrier()
        sim.event_record(0)
        for _ in range(args.steps):
            sim.timestep()
        sim.event_record(1)
        barrier()
        ms_rule = sim.event_elapsed(0, 1)
        shapes = sim.autotune(3)
        tune = {"ctas_by_active_domains": {str(k): v for k, v in sorted(shapes.items())},
                "ms_per_step_library_rule": ms_rule / args.steps}

    progress("value: device-resident timesteps")
    # ---- device-resident timesteps (value); clocks are sampled from the warm-up on, through the
    # end-to-end region below
    clocks = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        sim.timestep()
    barrier()
    launches0 = sim.kernel_launches
    sim.event_record(0)
    for _ in range(args.steps):
        sim.timestep()
    sim.event_record(1)
    barrier()
    ms = sim.event_elapsed(0, 1)
    gpu_launches = sim.kernel_launches - launches0
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = zones * args.steps * world / (ms / 1e3)

    progress("e2e")
    # ---- end to end through the C ABI with host buffers (e2e)

    last_seed = [0]

    def e2e_steps(k):
        upload()                  # the first step's input
        for i in range(k):
            last_seed[0] = sim.rng   # the host generator as this step starts (checked below)
            sim.timestep()
            download()            # this step's output ...
            if i + 1 < k:
                upload()          # ... and the next step's input, both moving while it computes

    e2e_steps(args.warmup)
    barrier()
    sim.event_record(2)
    e2e_steps(args.steps)
    sim.event_record(3)           # follows the last step's downloads
    barrier()
    ms_e2e = sim.event_elapsed(2, 3)
    clocks.__exit__(None, None, None)
    e2e_value = zones * args.steps * world / (ms_e2e / 1e3)

    progress("kernel timing")
    # ---- dominant kernel (fused BSSN stencil) timed with CUDA events around each launch
    sim.set_mode(am.MODE_BATCHED)
    sim.enable_kernel_timing(True)
    for _ in range(args.warmup):
        sim.timestep()
    sim.kernel_timing()   # discard warm-up
    for _ in range(args.steps):
        sim.timestep()
    k_ms, k_n = sim.kernel_timing()
    sim.enable_kernel_timing(False)
    # domains processed per timestep by the fused kernel: active domains of each substep, twice
    # (predictor and corrector); the predictor's leaves also write their restriction
    depths = [int(p) >> 27 for p in st["positions"][:used]]
    leaf = [all(c == -1 for c in st["children"][8 * i:8 * i + 8]) for i in range(used)]
    active = [[i for i, d in enumerate(depths) if (s & ((1 << (md - d)) - 1)) == 0] for s in range(1 << md)]
    per_step = sum(2 * len(a) for a in active)
    leaves_per_step = sum(sum(1 for i in a if leaf[i]) for a in active)
    bytes_per_launch = (fused_kernel_bytes_per_domain() * per_step +
                        fused_restriction_bytes_per_leaf() * leaves_per_step) / (2 << md)
    achieved = bytes_per_launch / (k_ms / k_n / 1e3) / 1e9 if k_n else None
    pk = peaks()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"] if achieved else None, "traffic": None,
                "kernel": f"k_stencil_bssn<{N},{P}> (fused BSSN derivatives)", "peak_source": pk["source"],
                "avg_launch_ms": k_ms / k_n if k_n else None, "launches_timed": k_n}
    try:   # DRAM bytes per domain from an ncu capture of the same kernel and workload, scaled per launch
        if (N, P) != (16, 3):
            raise OSError("the capture is of the 16/3 workload")
        with open(os.path.join(ROOT, "profiles", "k_stencil_bssn_16p3.traffic.json")) as f:
            tr = json.load(f)
        roofline["traffic"] = (tr["corrector_dram_bytes_per_domain"] * per_step / 2 +
                               tr["predictor_dram_bytes_per_domain"] * per_step / 2) / (2 << md)
        # The kernel is issue-bound: its instruction rate against the SMs' issue peak (4 warp
        # instructions per SM and cycle at the SM clock sampled under load)
        inst = (tr["corrector_warp_instructions_per_domain"] * per_step / 2 +
                tr["predictor_warp_instructions_per_domain"] * per_step / 2) / (2 << md)
        sm_mhz = clocks.summary()["sm_mhz"] or 2070.0
        issue_peak = torch.cuda.get_device_properties(local).multi_processor_count * 4 * sm_mhz * 1e6
        if k_n:
            rate = inst / (k_ms / k_n / 1e3)
            roofline["issue"] = {"achieved": rate, "peak": issue_peak, "unit": "warp-instructions/s",
                                 "frac": rate / issue_peak, "instructions_per_launch": inst}
    except (OSError, KeyError, ValueError):
        pass

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_dict(args.depth, world),
            "mode": args.mode,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": ms_e2e / args.steps},
            "gpu_launches": int(gpu_launches), "roofline": roofline, "clocks": clocks.summary()}
    if tune:
        tune["ms_per_step_tuned"] = ms / args.steps
        line["autotune"] = tune
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        progress("cpu baseline and parity of the last timed step")
        try:
            cpu = CpuTimestep(args.depth)
            # the last end-to-end step's input (the uploaded metric) and generator, on the host
            # cores: its outputs must equal what that step downloaded
            t32, ref = cpu.fp32([h.numpy() for h in h_in], last_seed[0])
            bad = []
            for i, (w, k, _n) in enumerate(outs):
                got = h_out[i].numpy()
                want = {am.Sim.NEW: ref["new"], am.Sim.DMET: ref["dmet"], am.Sim.CHR: ref["chr"],
                        am.Sim.RICCI: ref["ricci"]}[w][k]
                if w == am.Sim.RICCI:   # hardware reciprocal on the device, exact division here
                    if not np.all(np.abs(got - want) <= 1e-4 * (float(np.abs(want).max()) + 1e-30)):
                        bad.append(f"trace {k}")
                elif np.count_nonzero(got.view(np.uint32) != want.view(np.uint32)):
                    bad.append(f"buffer {w}/{k}")
            line["parity"] = "ok" if not bad else "mismatch: " + ", ".join(bad)
            t64 = cpu.fp64()
            line["cpu_baseline"] = {"value": cpu.zones / t64, "unit": UNIT, "cores": cpu.cores, "kind": "port",
                                    "sample": f"one whole timestep (8 substeps, all {cpu.used} domains) of the same "
                                              f"stencils in FP64 without quantisation, {t64:.2f} s"}
            line["cpu_fp32_port"] = {"value": cpu.zones / t32, "unit": UNIT, "cores": cpu.cores,
                                     "sample": f"the last timed step recomputed by the FP32 restatement, {t32:.2f} s"}
        except ValueError as e:   # no fixture of this tree depth
            line["parity"] = f"unchecked: {e}"
    # release every torch object that refers to the simulation's memory or stream first
    torch.cuda.synchronize()
    del h_in, h_out
    import gc
    gc.collect()
    torch.cuda.synchronize()
    sim.close()
    if rank == 0 and world == 1 and not args.no_evolution:
        # the full BSSN evolution's throughput at fixed constraint error, batched+learned against the
        # plain per-domain launches (not part of the timed region above)
        try:
            line["evolution"] = evolution_report(cpu=not args.no_cpu_baseline, estimator_path=args.estimator)
        except Exception as e:
            line["evolution"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
