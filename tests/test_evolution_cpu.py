"""The evolution's host logic and its FP64 oracle, on the CPU.

* Periodic boundary words of this library's octree equal the oracle's, computed independently from
  integer cell coordinates; faces that do not leave the root keep the reference's words.
* The FP64 oracle of the BSSN evolution converges at fourth order on the periodic gauge wave (the
  Hamiltonian and momentum constraints vanish for the continuum solution in any slicing), and holds
  the exact solution of the harmonic-slicing gauge wave.
* The FP64 oracle of the scalar wave u_tt = Δu (RK4) converges at fourth order on a uniform tree.
* A flat space evolves to itself; a Brill-Lindquist puncture keeps its constraints at the level of
  its initial data over a few steps (no blow-up).
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import cases


def tree_arrays(am, build, periodic=False, slots=600):
    o = am.Octree(slots)
    build(o)
    if periodic:
        o.set_periodic(True)
    st = o.state()
    o.close()
    return st


def evo_params(orc, n, outer, physics=0, slicing=0, shift=0, ko=0.1, cfl=0.25, **kw):
    e = orc.Evo()
    e.n, e.p, e.outer_size, e.physics, e.slicing, e.shift = n, 3, outer, physics, slicing, shift
    e.eta, e.ko_sigma, e.cfl, e.chi_floor = 2.0, ko, cfl, 1e-6
    e.id_kind = kw.get("id_kind", 0)
    e.amplitude, e.wavelength, e.width = kw.get("amplitude", 0.0), kw.get("wavelength", outer), kw.get("width", 0.1)
    punct = kw.get("punctures", ())
    e.n_punctures = len(punct)
    for i, (m, pos) in enumerate(punct):
        e.mass[i] = m
        for k in range(3):
            e.pos[i][k] = pos[k]
    return e


class OracleEvolution:
    """The FP64 oracle's state for one tree (padded double arrays per field)."""

    def __init__(self, orc, e, st):
        self.orc, self.e, self.st = orc, e, st
        self.used, self.md = st["used_slots"], st["max_depth"]
        self.nf = 24 if e.physics == 0 else 2
        t = e.n + 2 * e.p
        padded, inner = self.used * t ** 3, self.used * e.n ** 3
        self.old = [np.zeros(padded) for _ in range(self.nf)]
        self.new = [np.zeros(padded) for _ in range(self.nf)]
        self.stage = [np.zeros(padded) for _ in range(self.nf)]
        self.acc = [np.zeros(inner) for _ in range(self.nf)]
        L = orc.lib()
        L.orc_evo_initial_data(ctypes.byref(e), orc.P(orc.ptrs(self.old)), orc.P(st["positions"]), self.used)
        for f in range(self.nf):   # every state buffer starts from the data: the root's ghost layer
            self.new[f][:] = self.old[f]   # (the outer boundary) is never refilled
            self.stage[f][:] = self.old[f]
        self.timer = ctypes.c_uint32(0)

    def timestep(self, k=1):
        L, orc, st = self.orc.lib(), self.orc, self.st
        for _ in range(k):
            L.orc_evo_timestep(ctypes.byref(self.e), orc.P(orc.ptrs(self.old)), orc.P(orc.ptrs(self.new)),
                               orc.P(orc.ptrs(self.stage)), orc.P(orc.ptrs(self.acc)), orc.P(st["positions"]),
                               orc.P(st["children"]), orc.P(st["boundaries"]), self.used, self.md,
                               ctypes.byref(self.timer))

    def constraints(self, excision=0.0, cons4=None):
        out = (ctypes.c_double * 5)()
        self.orc.lib().orc_evo_constraints(ctypes.byref(self.e), self.orc.P(self.orc.ptrs(self.new)),
                                           self.orc.P(self.st["positions"]), self.orc.P(self.st["children"]),
                                           self.used, excision, self.orc.P(self.orc.ptrs(cons4)) if cons4 else None,
                                           out)
        return {"H_l2": out[0], "H_max": out[1], "M_l2": out[2], "M_max": out[3], "cells": int(out[4])}


@pytest.mark.parametrize("tree", ["uniform1", "uniform2", "uneven", "bssn", "wave"])
def test_periodic_boundaries_match_oracle(am, orc, tree):
    build = {"uniform1": lambda o: cases.tree_uniform(o, 1), "uniform2": lambda o: cases.tree_uniform(o, 2),
             **cases.TREES}[tree]
    plain = tree_arrays(am, build)
    per = tree_arrays(am, build, periodic=True)
    used = per["used_slots"]
    want = np.zeros(used * 6, np.uint64)
    orc.lib().orc_periodic_boundaries(orc.P(per["positions"]), orc.P(per["children"]), used, orc.P(want))
    got = per["boundaries"][: used * 6]
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} words differ"
    # faces that stay inside the root keep the reference's words (non-periodic octree)
    inside = (plain["boundaries"][: used * 6] & 0xFFFFFF) != 0
    assert np.array_equal(got[inside], plain["boundaries"][: used * 6][inside])


def gauge_wave_run(am, orc, n, depth, steps, slicing=0, amplitude=0.01):
    st = tree_arrays(am, lambda o: cases.tree_uniform(o, depth), periodic=True, slots=sum(8 ** d for d in range(depth + 1)))
    e = evo_params(orc, n, 1.0, slicing=slicing, id_kind=1, amplitude=amplitude, wavelength=1.0)
    ev = OracleEvolution(orc, e, st)
    ev.timestep(steps)
    return ev


def test_gauge_wave_converges_at_fourth_order(am, orc):
    """Same physical time (4 root steps, dt_root = cfl / N), 16^3 and 32^3 zones of the periodic
    box: the constraint norms fall by about 2^4."""
    coarse = gauge_wave_run(am, orc, 8, 1, 4, amplitude=0.05)
    fine = gauge_wave_run(am, orc, 8, 2, 4, amplitude=0.05)
    c, f = coarse.constraints(), fine.constraints()
    print(f"\ngauge wave H_l2 {c['H_l2']:.3e} -> {f['H_l2']:.3e} (ratio {c['H_l2'] / f['H_l2']:.1f}), "
          f"M_l2 {c['M_l2']:.3e} -> {f['M_l2']:.3e} (ratio {c['M_l2'] / f['M_l2']:.1f})")
    assert c["H_l2"] / f["H_l2"] > 10.0
    assert c["M_l2"] / f["M_l2"] > 10.0


def test_harmonic_gauge_wave_is_exact(am, orc):
    """With harmonic slicing the gauge wave is an exact solution: after the run the lapse is
    sqrt(1 - A sin(2 pi (x - t))) to the truncation error, which falls at fourth order."""
    errs = []
    for depth in (1, 2):
        ev = gauge_wave_run(am, orc, 8, depth, 4, slicing=1, amplitude=0.05)
        n, p, t = 8, 3, 14
        time = 4 * 0.25 / 8   # four root steps of dt = cfl * outer / N
        xyz = cases.cell_coordinates(ev.st["positions"], ev.used, n, p, 1.0)
        leaves = [i for i in range(ev.used) if all(c == -1 for c in ev.st["children"][8 * i:8 * i + 8])]
        sl = np.s_[p:p + n, p:p + n, p:p + n]
        err = 0.0
        for s in leaves:
            x = xyz[s][sl][..., 0]
            exact = np.sqrt(1 - 0.05 * np.sin(2 * np.pi * (x - time)))
            got = ev.new[17].reshape(ev.used, t, t, t)[s][sl]
            err = max(err, float(np.abs(got - exact).max()))
        errs.append(err)
    print(f"\nharmonic gauge wave lapse error {errs[0]:.3e} -> {errs[1]:.3e}")
    assert errs[1] < 1e-4 and errs[0] / errs[1] > 10.0


def test_wave_equation_converges(am, orc):
    """u_tt = Δu from a Gaussian pulse in a periodic box: the 16^3 and 32^3 solutions after the same
    time, each compared with a 64^3 solution sampled at the same points, converge at fourth order."""
    def run(depth):
        st = tree_arrays(am, lambda o: cases.tree_uniform(o, depth), periodic=True,
                         slots=sum(8 ** d for d in range(depth + 1)))
        e = evo_params(orc, 8, 2.0, physics=1, id_kind=3, width=0.4, ko=0.0)
        ev = OracleEvolution(orc, e, st)
        ev.timestep(4)
        return ev

    def sample(ev, depth):
        # the leaf cells' values on the uniform grid of 8 * 2^depth cells per edge
        n, p, t = 8, 3, 14
        m = 8 << depth
        grid = np.zeros((m, m, m))
        xyz = cases.cell_coordinates(ev.st["positions"], ev.used, n, p, 2.0)
        for s in range(ev.used):
            if any(c != -1 for c in ev.st["children"][8 * s:8 * s + 8]):
                continue
            c = xyz[s][p:p + n, p:p + n, p:p + n]
            i = np.rint((c + 1.0) * m / 2.0 - 0.5).astype(int)
            grid[i[..., 2], i[..., 1], i[..., 0]] = ev.new[0].reshape(ev.used, t, t, t)[s][p:p + n, p:p + n, p:p + n]
        return grid
    g1, g2, g3 = sample(run(1), 1), sample(run(2), 2), sample(run(3), 3)
    # restrict the finer grids to the coarse points by averaging 2x2x2 (cell centres coincide in the mean)
    def down(g):
        m = g.shape[0] // 2
        return g.reshape(m, 2, m, 2, m, 2).mean(axis=(1, 3, 5))
    e1 = np.sqrt(np.mean((g1 - down(down(g3))) ** 2))
    e2 = np.sqrt(np.mean((down(g2) - down(down(g3))) ** 2))
    print(f"\nwave equation error {e1:.3e} -> {e2:.3e} (ratio {e1 / e2:.1f})")
    assert e1 / e2 > 3.0


def test_flat_space_stays_flat(am, orc):
    st = tree_arrays(am, cases.tree_uneven)
    e = evo_params(orc, 8, 100.0, id_kind=0, shift=1)
    ev = OracleEvolution(orc, e, st)
    ev.timestep(1)
    c = ev.constraints()
    assert c["H_max"] == 0.0 and c["M_max"] == 0.0 and c["cells"] > 0
    for f in range(24):
        want = 1.0 if f in (0, 1, 4, 6, 17) else 0.0
        assert np.abs(ev.new[f] - want).max() < 1e-14 or not st["positions"].any()


def test_puncture_constraints_stay_bounded(am, orc):
    """A single Brill-Lindquist puncture on the reference's nested tree (kernel.cu:69-83) with the
    moving-puncture gauge: outside r = M (inside, the puncture is not resolved and its violation
    grows, as in any moving-puncture run) the composite-grid constraint norms settle after the first
    step instead of growing (no instability)."""
    st = tree_arrays(am, cases.tree_bssn)
    e = evo_params(orc, 8, 16.0, slicing=0, shift=1, id_kind=2, punctures=[(1.0, (0.013, -0.021, 0.007))], cfl=0.25)
    ev = OracleEvolution(orc, e, st)
    norms = [ev.constraints(1.0)]
    for _ in range(3):
        ev.timestep(1)
        norms.append(ev.constraints(1.0))
    print("\npuncture (r > M) H_l2 " + " -> ".join(f"{c['H_l2']:.2e}" for c in norms) +
          ", M_l2 " + " -> ".join(f"{c['M_l2']:.2e}" for c in norms))
    assert all(np.isfinite(c["H_l2"]) and np.isfinite(c["M_l2"]) for c in norms)
    assert norms[3]["H_l2"] < 2.0 * norms[1]["H_l2"]
    assert norms[3]["M_l2"] < 5.0 * norms[1]["M_l2"]
