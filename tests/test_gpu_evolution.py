"""The GPU evolutions (AMR_SIM_BSSN_EVOLVE, AMR_SIM_WAVE_RK4) against the FP64 oracle
(oracle/bssn_evolve.c), and the configurations' physics measured on the GPU.

The reference has no evolution to compare with (its BSSN plugin stops at derivatives and
Christoffel symbols, BSSN.h:143-159): parity here is FP32 GPU against the FP64 restatement of the
same scheme, within the tolerances stated in each test, and the physics is checked by convergence.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import cases
from test_evolution_cpu import OracleEvolution, evo_params, tree_arrays

pytestmark = pytest.mark.gpu


def gpu_sim(am, n, outer, build, kind, evolution, data, mode, slots=None):
    cfg = am.Config(n, 3, outer)
    sim = am.Sim(cfg, kind, slots=slots or 600, mode=mode)
    build(sim)
    sim.set_evolution(evolution)
    sim.initial_data(data)
    sim.synchronize()
    return sim


def gpu_state(am, sim, nf):
    """The latest state as values (the BSSN evolution stores some fields less 1)."""
    used = sim.state()["used_slots"]
    t = sim.cfg.total
    off = am.BSSN_OFFSETS if nf == 24 else (0.0,) * nf
    return [sim.tensor(am.Sim.NEW_STATE, f)[: used * t ** 3].cpu().numpy().astype(np.float64) + off[f]
            for f in range(nf)]


def compare(gpu, ref, st, n, tol, what, mask=None):
    """Largest difference per field over the live slots' cells (and `mask`, if given), relative to
    the field's scale over the live cells."""
    used, t = st["used_slots"], n + 6
    live = np.repeat(st["positions"][:used] != 0xFFFFFFFF, t ** 3)
    sel = live if mask is None else live & mask
    worst = 0.0
    for f, (g, r) in enumerate(zip(gpu, ref)):
        scale = max(float(np.abs(r[live]).max()), 1e-3)
        err = float(np.abs(g[sel] - r[sel]).max()) / scale
        worst = max(worst, err)
        assert err <= tol, f"{what}: field {f} differs by {err:.3e} of its scale (tolerance {tol:.1e})"
    return worst


@pytest.mark.parametrize("mode", ["batched", "graph"])
def test_gauge_wave_matches_fp64(am, cuda, orc, mode):
    """Periodic gauge wave (A = 0.05), uniform depth 1 of 8^3 domains, 1+log slicing: two root steps
    on the GPU against the FP64 oracle; every field within 1e-4 of its scale (single-precision
    rounding of the metric, amplified by the second derivatives: about 2^-24 / (dx^2 / dt))."""
    build = lambda o: cases.tree_uniform(o, 1)   # noqa: E731
    ev_g = am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=0, ko_sigma=0.1, cfl=0.25, periodic=1)
    data = am.InitialData(kind=am.ID_GAUGE_WAVE, amplitude=0.05, wavelength=1.0)
    sim = gpu_sim(am, 8, 1.0, build, am.SIM_BSSN_EVOLVE, ev_g, data,
                  {"batched": am.MODE_BATCHED, "graph": am.MODE_GRAPH}[mode], slots=9)
    sim.timestep()
    sim.timestep()
    sim.synchronize()
    st = sim.state()
    gpu = gpu_state(am, sim, 24)
    e = evo_params(orc, 8, 1.0, slicing=0, shift=0, id_kind=1, amplitude=0.05, wavelength=1.0)
    ref = OracleEvolution(orc, e, st)
    ref.timestep(2)
    worst = compare(gpu, ref.new, st, 8, 1e-4, "gauge wave")
    print(f"\ngauge wave, GPU FP32 vs FP64 after 2 root steps: worst field error {worst:.2e} of scale")
    c_gpu, c_ref = sim.constraint_norms(), ref.constraints()
    print(f"H_l2 GPU {c_gpu['H_l2']:.4e} FP64 {c_ref['H_l2']:.4e}; M_l2 GPU {c_gpu['M_l2']:.4e} FP64 {c_ref['M_l2']:.4e}")
    assert c_gpu["cells"] == c_ref["cells"]
    assert abs(c_gpu["H_l2"] - c_ref["H_l2"]) <= 2e-2 * c_ref["H_l2"]
    assert abs(c_gpu["M_l2"] - c_ref["M_l2"]) <= 2e-2 * c_ref["M_l2"]
    sim.close()


def test_gauge_wave_32_matches_fp64(am, cuda, orc):
    """The same periodic gauge wave on 32^3 domains (uniform depth 1: 64^3 zones), one root step on
    the GPU (the derivative pass at its 32^3 slab depth) against the FP64 oracle: every field within
    1e-4 of its scale, as at 8^3."""
    build = lambda o: cases.tree_uniform(o, 1)   # noqa: E731
    ev_g = am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=0, ko_sigma=0.1, cfl=0.25, periodic=1)
    data = am.InitialData(kind=am.ID_GAUGE_WAVE, amplitude=0.05, wavelength=1.0)
    sim = gpu_sim(am, 32, 1.0, build, am.SIM_BSSN_EVOLVE, ev_g, data, am.MODE_GRAPH, slots=9)
    sim.timestep()
    sim.synchronize()
    st = sim.state()
    gpu = gpu_state(am, sim, 24)
    sim.close()
    e = evo_params(orc, 32, 1.0, slicing=0, shift=0, id_kind=1, amplitude=0.05, wavelength=1.0)
    ref = OracleEvolution(orc, e, st)
    ref.timestep(1)
    worst = compare(gpu, ref.new, st, 32, 1e-4, "gauge wave 32^3")
    print(f"\ngauge wave on 32^3 domains, GPU FP32 vs FP64 after one root step: worst field error {worst:.2e} of scale")


def test_puncture_matches_fp64(am, cuda, orc):
    """A Brill-Lindquist puncture (m = 1, offset) on the reference's nested tree (kernel.cu:69-83,
    depth 6, 8^3 domains) with 1+log slicing and the Gamma-driver shift: one root step (64 substeps
    at the finest depth) on the GPU against the FP64 oracle.  Outside r = M every field is within
    1e-3 of its scale; inside, where the conformal factor falls to ~1e-4 and is stored as its
    deviation from 1 (about four significant digits there) and the unresolved puncture amplifies
    every rounding, within 2e-2.  The constraint norms outside r = M agree to 2%."""
    punct = [(1.0, (0.013, -0.021, 0.007))]
    ev_g = am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=1, eta=2.0, ko_sigma=0.1, cfl=0.25)
    data = am.InitialData(kind=am.ID_BRILL_LINDQUIST, punctures=punct)
    sim = gpu_sim(am, 8, 16.0, cases.tree_bssn, am.SIM_BSSN_EVOLVE, ev_g, data, am.MODE_BATCHED, slots=64)
    sim.timestep()
    sim.synchronize()
    st = sim.state()
    gpu = gpu_state(am, sim, 24)
    e = evo_params(orc, 8, 16.0, slicing=0, shift=1, id_kind=2, punctures=punct)
    ref = OracleEvolution(orc, e, st)
    ref.timestep(1)
    xyz = cases.cell_coordinates(st["positions"], st["used_slots"], 8, 3, 16.0).reshape(-1, 3)
    outside = np.linalg.norm(xyz - np.asarray(punct[0][1]), axis=1) > 1.0
    worst_out = compare(gpu, ref.new, st, 8, 1e-3, "puncture (r > M)", outside)
    worst = compare(gpu, ref.new, st, 8, 2e-2, "puncture")
    c_gpu, c_ref = sim.constraint_norms(1.0), ref.constraints(1.0)
    print(f"\npuncture, GPU vs FP64 after one root step: worst field error {worst_out:.2e} (r > M), "
          f"{worst:.2e} (all); H_l2 (r > M) GPU "
          f"{c_gpu['H_l2']:.4e} FP64 {c_ref['H_l2']:.4e}; M_l2 GPU {c_gpu['M_l2']:.4e} FP64 {c_ref['M_l2']:.4e}")
    assert c_gpu["cells"] == c_ref["cells"]
    assert abs(c_gpu["H_l2"] - c_ref["H_l2"]) <= 2e-2 * c_ref["H_l2"]
    sim.close()


def test_random_octree_punctures_match_fp64(am, cuda, orc):
    """The throughput sweep's shape at test size: a seeded Bernoulli(0.3) octree (refined to depth 4,
    185 domains of 8^3 with neighbours up to two levels apart, root edge 16) holding two
    Brill-Lindquist punctures of seeded masses in [0.2, 1] and positions in [-4, 4]^3, 1+log slicing
    and the Gamma-driver.  One root step (16 finest substeps): the plain per-domain launches, the
    batched launches and the graph replay give the same state bit for bit, and the GPU state is
    within 1e-3 of each field's scale of the FP64 oracle outside r = M of each puncture (2e-2
    everywhere, as for the single puncture), with H L2 outside r = M within 2 %."""
    rng = np.random.default_rng(11)
    punct = [(float(rng.uniform(0.2, 1.0)), tuple(float(v) for v in rng.uniform(-4.0, 4.0, 3))) for _ in range(2)]
    build = lambda o: cases.tree_random(o, 4, 0.3, 0)   # noqa: E731
    ev_g = am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=1, eta=2.0, ko_sigma=0.1, cfl=0.25)
    data = am.InitialData(kind=am.ID_BRILL_LINDQUIST, punctures=punct)
    states = []
    for mode in (am.MODE_PLAIN, am.MODE_BATCHED, am.MODE_GRAPH):
        sim = gpu_sim(am, 8, 16.0, build, am.SIM_BSSN_EVOLVE, ev_g, data, mode, slots=200)
        sim.timestep()
        sim.synchronize()
        st = sim.state()
        states.append(gpu_state(am, sim, 24))
        if mode == am.MODE_GRAPH:
            c_gpu = sim.constraint_norms(1.0)
        sim.close()
    assert st["used_slots"] == 185 and st["max_depth"] == 4
    for other in states[1:]:
        for f in range(24):
            assert np.array_equal(states[0][f], other[f]), f"field {f} differs between modes"
    e = evo_params(orc, 8, 16.0, slicing=0, shift=1, id_kind=2, punctures=punct)
    ref = OracleEvolution(orc, e, st)
    ref.timestep(1)
    xyz = cases.cell_coordinates(st["positions"], st["used_slots"], 8, 3, 16.0).reshape(-1, 3)
    outside = np.ones(len(xyz), bool)
    for m, pos in punct:
        outside &= np.linalg.norm(xyz - np.asarray(pos), axis=1) > max(m, 1.0)
    worst_out = compare(states[0], ref.new, st, 8, 1e-3, "random octree (r > M)", outside)
    worst = compare(states[0], ref.new, st, 8, 2e-2, "random octree")
    c_ref = ref.constraints(1.0)
    print(f"\nrandom octree, two punctures, GPU vs FP64 after one root step: worst field error {worst_out:.2e} "
          f"(r > M), {worst:.2e} (all); H_l2 GPU {c_gpu['H_l2']:.4e} FP64 {c_ref['H_l2']:.4e}")
    assert c_gpu["cells"] == c_ref["cells"]
    assert abs(c_gpu["H_l2"] - c_ref["H_l2"]) <= 2e-2 * c_ref["H_l2"]


def test_wave_equation_config_matches_fp64(am, cuda, orc):
    """The scalar-wave configuration: root 16^3 with one octant refined (two levels), [-1, 1]^3,
    u = exp(-|x|^2 / 0.1^2), u_t = 0, RK4 at CFL 0.25 with 2:1 subcycling, 64 coarse steps.  The
    L2 error of u against the FP64 oracle over the composite grid stays below 1e-5 of max |u|."""
    build = lambda o: o.add_node(0, 0)   # noqa: E731
    ev_g = am.Evolution(ko_sigma=0.0, cfl=0.25)
    data = am.InitialData(kind=am.ID_GAUSSIAN_PULSE, width=0.1)
    sim = gpu_sim(am, 16, 2.0, build, am.SIM_WAVE_RK4, ev_g, data, am.MODE_GRAPH, slots=2)
    for _ in range(64):
        sim.timestep()
    sim.synchronize()
    st = sim.state()
    gpu = gpu_state(am, sim, 2)
    e = evo_params(orc, 16, 2.0, physics=1, id_kind=3, width=0.1, ko=0.0)
    ref = OracleEvolution(orc, e, st)
    ref.timestep(64)
    t = 22
    u_g = gpu[0].reshape(-1, t, t, t)[:, 3:19, 3:19, 3:19]
    u_r = ref.new[0].reshape(-1, t, t, t)[:, 3:19, 3:19, 3:19]
    covered = np.zeros_like(u_r, bool)
    covered[0, :8, :8, :8] = True     # the root's octant 0 is covered by the child
    d = (u_g - u_r)[~covered]
    l2 = float(np.sqrt(np.mean(d ** 2)))
    print(f"\nwave equation, 64 coarse steps: L2 error against FP64 {l2:.3e} (max |u| {np.abs(u_r).max():.3e})")
    assert l2 <= 1e-5 * float(np.abs(u_r).max())
    sim.close()


def test_gauge_wave_converges_on_gpu(am, cuda, orc):
    """Fourth-order convergence of the GPU evolution on the periodic gauge wave (A = 0.05, 16^3 and
    32^3 zones of 8^3 domains, four root steps), with the FP64 oracle's ratio beside it."""
    norms = {}
    for depth in (1, 2):
        ev_g = am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=0, ko_sigma=0.1, cfl=0.25, periodic=1)
        data = am.InitialData(kind=am.ID_GAUGE_WAVE, amplitude=0.05, wavelength=1.0)
        sim = gpu_sim(am, 8, 1.0, lambda o, d=depth: cases.tree_uniform(o, d), am.SIM_BSSN_EVOLVE, ev_g, data,
                      am.MODE_GRAPH, slots=sum(8 ** k for k in range(depth + 1)))
        for _ in range(4):
            sim.timestep()
        norms[depth] = sim.constraint_norms()
        sim.close()
    r_h = norms[1]["H_l2"] / norms[2]["H_l2"]
    r_m = norms[1]["M_l2"] / norms[2]["M_l2"]
    print(f"\ngauge wave on the GPU 16^3 -> 32^3: H_l2 {norms[1]['H_l2']:.3e} -> {norms[2]['H_l2']:.3e} (ratio {r_h:.1f}), "
          f"M_l2 {norms[1]['M_l2']:.3e} -> {norms[2]['M_l2']:.3e} (ratio {r_m:.1f})")
    assert r_h > 10.0 and r_m > 10.0


def test_gauge_wave_config_on_gpu(am, cuda):
    """The gauge-wave configuration as specified: 128^3 zones (uniform depth 3 of 16^3 domains,
    padding 3), A = 1e-2, L = 1, periodic, 1+log slicing, zero shift, 200 steps at the finest depth
    (25 root steps of eight substeps), beside the same run at 64^3.  At these resolutions the
    truncation error of the constraints (~1e-6) is below the single-precision rounding of the state
    (the constraints take second derivatives: rounding / dx^2), so the norms report that floor; they
    must stay below 2e-4 and finite over the run."""
    for depth in (2, 3):
        ev_g = am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=0, ko_sigma=0.1, cfl=0.25, periodic=1)
        data = am.InitialData(kind=am.ID_GAUGE_WAVE, amplitude=1e-2, wavelength=1.0)
        sim = gpu_sim(am, 16, 1.0, lambda o, d=depth: cases.tree_uniform(o, d), am.SIM_BSSN_EVOLVE, ev_g, data,
                      am.MODE_GRAPH, slots=sum(8 ** k for k in range(depth + 1)))
        for _ in range(25):
            sim.timestep()
        c = sim.constraint_norms()
        sim.close()
        print(f"\ngauge wave {16 << depth}^3, 200 finest steps: H_l2 {c['H_l2']:.3e} M_l2 {c['M_l2']:.3e} "
              f"H_max {c['H_max']:.3e} M_max {c['M_max']:.3e}")
        assert np.isfinite(c["H_l2"]) and c["H_l2"] < 2e-4 and c["M_l2"] < 2e-4


def test_modes_agree(am, cuda):
    """The plain per-domain launches, the batched launches and the graph replay give the same state
    bit for bit (a Brill-Lindquist puncture on the uneven tree, Gamma-driver shift, one root step)."""
    punct = [(1.0, (10.013, -10.021, 0.007))]
    states = []
    for mode in (am.MODE_PLAIN, am.MODE_BATCHED, am.MODE_GRAPH):
        ev_g = am.Evolution(slicing=am.SLICING_1PLUSLOG, shift=1, eta=2.0, ko_sigma=0.1, cfl=0.25)
        data = am.InitialData(kind=am.ID_BRILL_LINDQUIST, punctures=punct)
        sim = gpu_sim(am, 16, 100.0, cases.tree_uneven, am.SIM_BSSN_EVOLVE, ev_g, data, mode, slots=32)
        sim.timestep()
        sim.timestep()
        sim.synchronize()
        states.append(gpu_state(am, sim, 24))
        sim.close()
    for other in states[1:]:
        for f in range(24):
            assert np.array_equal(states[0][f], other[f]), f"field {f} differs between modes"


def test_new_domains_are_prolongated_to_fourth_order(am, cuda):
    """A domain added to an evolution takes its padded cells from its parent by tricubic
    interpolation: a cubic polynomial in the parent's padded cells (ghost layer included) is
    reproduced exactly, to single-precision rounding, in every cell of each child, ghosts included.
    The conformal factor and the lapse are interpolated through their fourth and square roots: chi =
    q^4 and alpha = q^2 with q linear are reproduced exactly."""
    import torch
    n, p = 8, 3
    t = n + 2 * p
    sim = am.Sim(am.Config(n, p, 1.0), am.SIM_BSSN_EVOLVE, slots=9, mode=am.MODE_BATCHED)
    sim.set_evolution(am.Evolution())
    sim.initial_data(am.InitialData(kind=am.ID_FLAT))
    sim.synchronize()
    ix = torch.arange(t, dtype=torch.float64, device="cuda")
    z, y, x = torch.meshgrid(ix, ix, ix, indexing="ij")

    def cubic(x, y, z, f):
        if f in (am.F_CHI, am.F_ALPHA):   # stored less 1; q = 0.2 + 0.03 x + 0.02 y + 0.01 z > 0
            q = 0.2 + 0.03 * x + 0.02 * y + 0.01 * z
            return (q ** 4 if f == am.F_CHI else q ** 2) - 1.0
        return 0.1 * f + 1e-3 * (x ** 3 - 2 * y ** 2 * z + 3 * x * y * z + z ** 3 / 4 - 5 * x + 7)

    for f in range(24):
        for buf in (sim.OLD_STATE, sim.NEW_STATE):
            sim.tensor(buf, f)[: t ** 3].copy_(cubic(x, y, z, f).reshape(-1).float())
    torch.cuda.synchronize()
    sim.add_nodes([0] * 8, list(range(8)))
    sim.synchronize()
    st = sim.state()
    worst = 0.0
    for o in range(8):
        child = int(st["children"][o])
        oc = [(o >> a) & 1 for a in range(3)]
        # child cell w sits at parent coordinate o * n / 2 + p + (w - p + 1/2) / 2 - 1/2
        px, py, pz = [oc[a] * (n // 2) + p + ((c - p + 0.5) / 2 - 0.5) for a, c in enumerate((x, y, z))]
        for f in (0, 5, 12, 17, 23):
            want = cubic(px, py, pz, f)
            for buf in (sim.OLD_STATE, sim.NEW_STATE):
                got = sim.tensor(buf, f)[child * t ** 3:(child + 1) * t ** 3].double().reshape(t, t, t)
                worst = max(worst, float((got - want).abs().max() / want.abs().max()))
    print(f"\ncubic prolongation: largest relative error {worst:.2e}")
    assert worst < 1e-5
    sim.close()
