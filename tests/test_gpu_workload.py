"""Parity of the benchmark's own workload, launch-shape independence and the failure path.

* The uniform depth-3 octree of the benchmark (512 leaves + 73 parents = 585 slots of 16^3,
  padding 3) through amr_sim_timestep in the graph and batched modes, two timesteps, against the
  oracle's BSSN_AMR_data::timestep over every slot (BSSN.h:160-170), and against the reference's
  own plugin (this tree has only same-level faces, where its ghost fill does not race).
* Uniform depth-2 trees at 32^3 / p3 and at the reference's own 28^3 / p2 against the oracle.
* The fused pass gives the same bits whatever its grid: one plane per CTA, four, the persistent
  cap (every CTA takes an equal contiguous range of planes).
* A data wait that runs out (a plane request withheld on purpose by the host-set test hook)
  makes amr_sim_synchronize report AMR_ERR_TIMEOUT once; the next timestep runs clean.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _slots(depth: int) -> int:
    return sum(8 ** d for d in range(depth + 1))


def _uniform_sim(am, cfg, depth, mode, seed=500):
    import torch
    sim = am.Sim(cfg, am.SIM_BSSN, slots=_slots(depth), mode=mode)
    cases.tree_uniform(sim, depth)
    sim.synchronize()
    st = sim.state()
    used, t = st["used_slots"], cfg.total
    xyz = cases.cell_coordinates(st["positions"], used, cfg.size_domain, cfg.padding_domain, cfg.outer_size)
    metric = cases.metric_fields(xyz, cfg.outer_size, seed)
    upload(am, sim, metric, used * t ** 3)
    return sim, st, metric


def upload(am, sim, metric, count):
    import torch
    for which in (am.Sim.OLD, am.Sim.NEW):
        for k in range(6):
            sim.tensor(which, k)[:count].copy_(torch.from_numpy(metric[k]).cuda())
    torch.cuda.synchronize()


def dump(am, sim, used, cfg) -> dict:
    out = {}
    for which, name, cells in ((am.Sim.OLD, "old", cfg.padded_cells), (am.Sim.NEW, "new", cfg.padded_cells),
                               (am.Sim.RICCI, "ricci", cfg.inner_cells), (am.Sim.DMET, "dmet", cfg.inner_cells),
                               (am.Sim.CHR, "chr", cfg.inner_cells)):
        for k in range(6):
            a = sim.tensor(which, k)[: used * cells].cpu().numpy()
            out[f"{name}{k}"] = a.view(np.uint32) if a.dtype == np.int32 else a
    out["rng"] = sim.rng
    return out


def same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    bad = np.count_nonzero(a.view(np.uint32) != b.view(np.uint32))
    assert bad == 0, f"{what}: {bad} of {a.size} words differ"


def oracle_timesteps(orc, cfg, st, metric, seed0, steps):
    n, used = cfg.size_domain, st["used_slots"]
    c = orc.cfg(n, cfg.padding_domain, cfg.outer_size)
    old6 = [m.copy() for m in metric]
    new6 = [m.copy() for m in metric]
    dm = [np.zeros(used * n ** 3, np.uint32) for _ in range(6)]
    ch = [np.zeros(used * n ** 3, np.uint32) for _ in range(6)]
    ri = [np.zeros(used * n ** 3, np.float32) for _ in range(6)]
    timer, rng = ctypes.c_uint32(0), ctypes.c_int32(seed0)
    for _ in range(steps):
        orc.lib().orc_bssn_timestep(ctypes.byref(c), orc.P(orc.ptrs(old6)), orc.P(orc.ptrs(new6)),
                                    orc.P(orc.ptrs(dm)), orc.P(orc.ptrs(ch)), orc.P(orc.ptrs(ri)),
                                    orc.P(st["positions"]), orc.P(st["children"]), orc.P(st["boundaries"]), used,
                                    st["max_depth"], ctypes.byref(timer), ctypes.byref(rng), 0, used)
    return {"old": old6, "new": new6, "dmet": dm, "chr": ch, "ricci": ri, "rng": rng.value}


def assert_matches_oracle(mine, ref, what):
    assert mine["rng"] == ref["rng"], f"{what}: host generator"
    for k in range(6):
        for name in ("old", "new", "dmet", "chr"):
            same(mine[f"{name}{k}"], ref[name][k], f"{what}: {name}{k} vs oracle")
        # the device divides by the determinant with the hardware reciprocal, the oracle exactly
        scale = float(np.abs(ref["ricci"][k]).max()) + 1e-30
        err = float(np.abs(mine[f"ricci{k}"] - ref["ricci"][k]).max())
        assert err <= 1e-4 * scale, f"{what}: ricci{k} off by {err} (scale {scale})"


@pytest.mark.parametrize("mode", ["graph", "batched"])
def test_benchmark_tree_matches_oracle(am, cuda, orc, mode):
    """The benchmark's 585-slot tree, two timesteps, every slot compared with the oracle."""
    cfg = am.Config(16, 3, 100.0)
    sim, st, metric = _uniform_sim(am, cfg, 3, {"graph": am.MODE_GRAPH, "batched": am.MODE_BATCHED}[mode])
    assert st["used_slots"] == 585
    seed0 = sim.rng
    sim.timestep()
    sim.timestep()
    sim.synchronize()
    mine = dump(am, sim, st["used_slots"], cfg)
    sim.close()
    assert_matches_oracle(mine, oracle_timesteps(orc, cfg, st, metric, seed0, 2), f"585-slot tree, {mode}")


def test_benchmark_tree_matches_reference_plugin(am, cuda, ref16):
    """One timestep of the 585-slot tree against the reference's BSSN_AMR_data on the same GPU."""
    import torch
    from oracle import reflib
    cfg = am.Config(16, 3, 100.0)
    sim, st, metric = _uniform_sim(am, cfg, 3, am.MODE_GRAPH)
    used, t, n = st["used_slots"], cfg.total, cfg.size_domain
    h = ref16.refd_bssn_create(585)

    class _T:
        def add_node(self, pa, off):
            ref16.refd_bssn_add_node(h, pa, off)

        def state(self):
            return reflib.octree_state(ref16.refd_bssn_octree_state, h, 585)
    cases.tree_uniform(_T(), 3)
    rst = _T().state()
    for k in ("positions", "children", "boundaries"):
        m = {"children": 8, "boundaries": 6}.get(k, 1)
        assert np.array_equal(st[k][: used * m], rst[k][: used * m]), k

    def wrap(addr, count, typestr):
        class _M:
            __cuda_array_interface__ = {"shape": (count,), "typestr": typestr, "data": (addr, False), "version": 3}
        return torch.as_tensor(_M(), device="cuda")
    for which in (0, 1):
        for k in range(6):
            wrap(ref16.refd_bssn_field(h, which, k), used * t ** 3, "<f4").copy_(torch.from_numpy(metric[k]).cuda())
    torch.cuda.synchronize()
    assert ref16.refd_bssn_timestep(h) == 0
    sim.timestep()
    sim.synchronize()
    mine = dump(am, sim, used, cfg)
    for which, name, cells in ((0, "old", t ** 3), (1, "new", t ** 3), (2, "ricci", n ** 3)):
        for k in range(6):
            same(mine[f"{name}{k}"], wrap(ref16.refd_bssn_field(h, which, k), used * cells, "<f4").cpu().numpy(),
                 f"{name}{k} vs reference plugin")
    for which, name in ((0, "dmet"), (1, "chr")):
        for k in range(6):
            same(mine[f"{name}{k}"], wrap(ref16.refd_bssn_cf3(h, which, k), used * n ** 3, "<i4").cpu().numpy(),
                 f"{name}{k} vs reference plugin")
    assert mine["rng"] == int(ref16.refd_bssn_rng_seed(h))
    ref16.refd_bssn_destroy(h)
    sim.close()


@pytest.mark.parametrize("n,p", [(32, 3), (28, 2)])
def test_uniform_depth2_matches_oracle(am, cuda, orc, n, p):
    cfg = am.Config(n, p, 100.0)
    sim, st, metric = _uniform_sim(am, cfg, 2, am.MODE_GRAPH)
    seed0 = sim.rng
    sim.timestep()
    sim.timestep()
    sim.synchronize()
    mine = dump(am, sim, st["used_slots"], cfg)
    sim.close()
    assert_matches_oracle(mine, oracle_timesteps(orc, cfg, st, metric, seed0, 2), f"uniform depth 2 at {n}/{p}")


@pytest.mark.parametrize("n,p", [(16, 3), (28, 2), (32, 3)])
def test_fused_pass_independent_of_grid(am, cuda, n, p):
    """The same two timesteps with the fused pass on one plane per CTA, four planes per CTA, one
    CTA per SM and the library's choice: bit-identical state and outputs."""
    import torch
    cfg = am.Config(n, p, 100.0)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    results = {}
    for label in ("auto", "1 plane", "4 planes", "1 per SM"):
        sim, st, _ = _uniform_sim(am, cfg, 1, am.MODE_BATCHED)
        used = st["used_slots"]
        planes = 9 * n   # every domain active at substep 0; fewer afterwards
        ctas = {"auto": 0, "1 plane": planes, "4 planes": (planes + 3) // 4, "1 per SM": sms}[label]
        sim.set_stencil_ctas(ctas)
        sim.timestep()
        sim.timestep()
        sim.synchronize()
        results[label] = dump(am, sim, used, cfg)
        sim.close()
    for label, got in results.items():
        for k, v in results["auto"].items():
            if k != "rng":
                same(got[k], v, f"{n}/{p} {label} vs auto: {k}")


@pytest.mark.parametrize("mode", ["graph", "batched"])
def test_autotune_leaves_state_and_results_unchanged(am, cuda, mode):
    """amr_sim_autotune on the benchmark's 585-slot tree between timesteps: every buffer of the
    simulation is bit-identical before and after it, it tunes every distinct active-domain count of
    the substeps (585, 584, 576 and 512 here), and the next two timesteps on the tuned grids equal
    those of an untuned simulation bit for bit."""
    cfg = am.Config(16, 3, 100.0)
    m = {"graph": am.MODE_GRAPH, "batched": am.MODE_BATCHED}[mode]
    results = []
    for tune in (False, True):
        sim, st, _ = _uniform_sim(am, cfg, 3, m)
        used = st["used_slots"]
        sim.timestep()
        sim.synchronize()
        if tune:
            before = dump(am, sim, used, cfg)
            shapes = sim.autotune(2)
            after = dump(am, sim, used, cfg)
            for k, v in before.items():
                if k != "rng":
                    same(after[k], v, f"autotune changed {k}")
            assert after["rng"] == before["rng"]
            assert sorted(shapes) == [512, 576, 584, 585], shapes
            assert all(c >= 1 for c in shapes.values())
            assert sim.tuned_shapes() == shapes
        sim.timestep()
        sim.timestep()
        sim.synchronize()
        results.append(dump(am, sim, used, cfg))
        sim.close()
    for k, v in results[0].items():
        if k != "rng":
            same(results[1][k], v, f"tuned vs library grid: {k}")
    assert results[1]["rng"] == results[0]["rng"]


def test_autotune_evolution_slab_depth(am, cuda):
    """amr_sim_autotune on the BSSN evolution (the gauge wave on uniform depth 2, 73 evolved
    domains of 16^3): it picks one of the derivative pass's compiled slab depths, leaves every
    state buffer bit-identical, and the next timestep on the tuned depth equals an untuned
    simulation's bit for bit (every cell's derivatives are the same arithmetic whatever the slab)."""
    import torch
    states = []
    for tune in (False, True):
        sim = am.Sim(am.Config(16, 3, 1.0), am.SIM_BSSN_EVOLVE, slots=73, mode=am.MODE_GRAPH)
        cases.tree_uniform(sim, 2)
        sim.set_evolution(am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=0, ko_sigma=0.1, cfl=0.25, periodic=1))
        sim.initial_data(am.InitialData(kind=am.ID_GAUGE_WAVE, amplitude=1e-2, wavelength=1.0))
        sim.timestep()
        sim.synchronize()
        used, t = sim.state()["used_slots"], sim.cfg.total
        if tune:
            before = [sim.tensor(w, f)[: used * t ** 3].clone() for w in (sim.OLD_STATE, sim.NEW_STATE) for f in range(24)]
            shapes = sim.autotune(2)
            after = [sim.tensor(w, f)[: used * t ** 3].clone() for w in (sim.OLD_STATE, sim.NEW_STATE) for f in range(24)]
            assert all(torch.equal(x, y) for x, y in zip(before, after)), "autotune changed the state"
            assert list(shapes) == [73] and shapes[73] in (1, 2, 4), shapes
        sim.timestep()
        sim.synchronize()
        states.append([sim.tensor(sim.NEW_STATE, f)[: used * t ** 3].cpu().numpy() for f in range(24)])
        sim.close()
    for f in range(24):
        same(states[1][f], states[0][f], f"tuned vs default slab depth: field {f}")


@pytest.mark.parametrize("mode", ["graph", "batched"])
def test_caller_stream(am, cuda, mode):
    """amr_sim_set_stream: the simulation enqueues on a caller's stream (a torch stream here), graph
    capture included; two timesteps on it equal two timesteps on the simulation's own stream bit
    for bit, and the caller's stream carries the work (a torch event recorded on it after the
    timesteps sees the results)."""
    import torch
    cfg = am.Config(16, 3, 100.0)
    m = {"graph": am.MODE_GRAPH, "batched": am.MODE_BATCHED}[mode]
    results = []
    for use_caller in (False, True):
        sim, st, _ = _uniform_sim(am, cfg, 2, m)
        s = torch.cuda.Stream()
        if use_caller:
            sim.set_stream(s.cuda_stream)
            assert sim.stream == s.cuda_stream
        sim.timestep()
        sim.timestep()
        if use_caller:
            done = torch.cuda.Event()
            done.record(s)
            done.synchronize()
            sim.set_stream(0)   # back to its own
        sim.synchronize()
        results.append(dump(am, sim, st["used_slots"], cfg))
        sim.close()
    for k, v in results[0].items():
        if k != "rng":
            same(results[1][k], v, f"caller's stream vs own: {k}")


def test_autotune_rejects_the_wave_plugin(am, cuda):
    sim = am.Sim(am.Config(28, 2, 100.0), am.SIM_WAVE, slots=9, mode=am.MODE_BATCHED)
    with pytest.raises(RuntimeError):
        sim.autotune(2)
    sim.close()


def test_bounded_wait_failure_is_reported_and_recovers(am, cuda):
    """The host tells each CTA's producer to skip its first plane request and shortens the data
    waits: the waits run out, the pass leaves (after every copy it issued has landed) and the
    device flag is raised; amr_sim_synchronize reports it once.  A clean timestep afterwards
    equals the same timestep of a simulation that never failed."""
    cfg = am.Config(16, 3, 100.0)
    sim, st, metric = _uniform_sim(am, cfg, 1, am.MODE_BATCHED)
    clean, _, _ = _uniform_sim(am, cfg, 1, am.MODE_BATCHED)
    used = st["used_slots"]
    rng0 = sim.rng
    sim.set_fault_injection(spin_limit=4096, withhold_plane=1)
    sim.timestep()
    with pytest.raises(am.AmrError) as info:
        sim.synchronize()
    assert info.value.status == am.ERR_TIMEOUT
    sim.synchronize()                       # reported once, then cleared
    assert am.load().amr_device_status(None) == am.OK
    sim.set_fault_injection(0, 0)
    upload(am, sim, metric, used * cfg.padded_cells)
    sim.rng = rng0
    sim.timestep()
    sim.synchronize()
    clean.timestep()
    clean.synchronize()
    a, b = dump(am, sim, used, cfg), dump(am, clean, used, cfg)
    for k in b:
        if k != "rng":
            same(a[k], b[k], f"after recovery: {k}")
    sim.close()
    clean.close()


def test_checkpoint_checks(am, cuda, tmp_path):
    """amr_sim_load refuses a checkpoint whose counter is outside 0 .. 2^max_depth - 1 or whose
    nodes lie deeper than its max depth, and a truncated field file leaves the simulation as it
    was (every file is read and checked before anything is uploaded)."""
    import shutil
    cfg = am.Config(16, 3, 100.0)
    sim, st, metric = _uniform_sim(am, cfg, 1, am.MODE_BATCHED)
    sim.timestep()
    sim.synchronize()
    good = tmp_path / "good"
    good.mkdir()
    sim.save_checkpoint(str(good))
    before = dump(am, sim, st["used_slots"], cfg)
    before_state = sim.state()

    def variant(name, edit):
        d = tmp_path / name
        shutil.copytree(good, d)
        edit(d)
        return str(d)

    def state_words(d, idx, value):
        w = np.fromfile(d / "state.bin", np.uint32)
        w[idx] = value
        w.tofile(d / "state.bin")

    def deep_node(d):
        pos = np.fromfile(d / "positions.bin", np.uint32)
        pos[3] = (5 << 27) | (pos[3] & ((1 << 27) - 1))   # depth 5 in a tree of max depth 1
        pos.tofile(d / "positions.bin")

    def truncate(d):
        f = d / "field_1_4.bin"
        f.write_bytes(f.read_bytes()[:-4])
    bad = [variant("timer", lambda d: state_words(d, 7, 2)), variant("depth", deep_node),
           variant("truncated", truncate)]
    # scribble on the simulation's state first: a refused load must leave the scribbled state as is
    for which in (am.Sim.NEW,):
        sim.tensor(which, 2).fill_(7.0)
    scribbled = dump(am, sim, st["used_slots"], cfg)
    for d in bad:
        with pytest.raises(am.AmrError) as info:
            sim.load_checkpoint(d)
        assert info.value.status == am.ERR_INVALID
        after = dump(am, sim, st["used_slots"], cfg)
        for k in scribbled:
            if k != "rng":
                same(after[k], scribbled[k], f"refused {d}: {k}")
        assert sim.state()["timer"] == before_state["timer"]
    sim.load_checkpoint(str(good))
    restored = dump(am, sim, st["used_slots"], cfg)
    for k in before:
        if k != "rng":
            same(restored[k], before[k], f"good checkpoint: {k}")
    sim.close()


def test_benchmark_tree_errors_against_fp64(am, cuda, orc):
    """Every floating-point output of one GPU timestep of the benchmark's tree against the FP64
    host oracle, with the tolerances stated in tests/test_fp64_errors.py."""
    from test_fp64_errors import fp32_slack, fp64_timestep, report
    cfg = am.Config(16, 3, 100.0)
    sim, st, metric = _uniform_sim(am, cfg, 3, am.MODE_GRAPH)
    sim.timestep()
    sim.synchronize()
    mine = dump(am, sim, st["used_slots"], cfg)
    sim.close()
    single = {"old": [mine[f"old{k}"] for k in range(6)], "new": [mine[f"new{k}"] for k in range(6)],
              "dmet": [mine[f"dmet{k}"] for k in range(6)], "chr": [mine[f"chr{k}"] for k in range(6)],
              "ricci": [mine[f"ricci{k}"] for k in range(6)]}
    print("\n585-slot tree at 16/3, one GPU timestep, relative errors against FP64:")
    report(orc, single, fp64_timestep(orc, 16, 3, st, metric), fp32_slack(metric, 16, 3, st))
