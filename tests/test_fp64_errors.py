"""Error of every floating-point output of the BSSN timestep against an FP64 host oracle.

The single-precision path (the oracle's restatement here, bit-identical to this library's kernels
and to the reference's device build by the parity tests) is compared with the same timestep in
double precision without compressed_float3 quantisation (oracle/fp64_path.c).  Stated tolerances,
relative to the largest magnitude of each output (max) or to its L2 norm (L2):

  output                          max        L2      source of the error
  old / new metric (padded)       2e-6       1e-6    float rounding of restriction and ghost fill
  metric gradients (cf3)          2^-6       5e-3    shared-exponent quantisation: 8-bit mantissas,
                                                     stochastic rounding; per word |err| <= one
                                                     quantisation step 2^(E-15)/128, plus the
                                                     single-precision rounding of the stencil sum
                                                     (16 * 2^-24 * sum|weights| * max|field| / dx)
  Christoffel symbols (cf3)       2^-5       1e-2    quantised gradients, then quantised again
  g^kl d_k d_l g_ij (float)       2^-5       1e-2    quantised Hessians (diagonal and mixed)

`report()` prints the measured figures (pytest -s shows them).
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import cases

TOL = {"metric": (2e-6, 1e-6), "grad": (2.0 ** -6, 5e-3), "chr": (2.0 ** -5, 1e-2), "ricci": (2.0 ** -5, 1e-2)}


def fp64_timestep(orc, n, p, st, metric):
    used = st["used_slots"]
    c = orc.cfg(n, p, 100.0)
    inner = used * n ** 3
    o64 = [m.astype(np.float64) for m in metric]
    n64 = [m.astype(np.float64) for m in metric]
    g64 = [np.zeros(inner * 3) for _ in range(6)]
    c64 = [np.zeros(inner * 3) for _ in range(6)]
    r64 = [np.zeros(inner) for _ in range(6)]
    timer = ctypes.c_uint32(0)
    orc.lib().orc_bssn_timestep_f64(ctypes.byref(c), orc.P(orc.ptrs(o64)), orc.P(orc.ptrs(n64)), orc.P(orc.ptrs(g64)),
                                    orc.P(orc.ptrs(c64)), orc.P(orc.ptrs(r64)), orc.P(st["positions"]),
                                    orc.P(st["children"]), orc.P(st["boundaries"]), used, st["max_depth"],
                                    ctypes.byref(timer))
    return {"old": o64, "new": n64, "grad": g64, "chr": c64, "ricci": r64}


def fp32_timestep(orc, n, p, st, metric, seed=12894712):
    used = st["used_slots"]
    c = orc.cfg(n, p, 100.0)
    inner = used * n ** 3
    old6 = [m.copy() for m in metric]
    new6 = [m.copy() for m in metric]
    dm = [np.zeros(inner, np.uint32) for _ in range(6)]
    ch = [np.zeros(inner, np.uint32) for _ in range(6)]
    ri = [np.zeros(inner, np.float32) for _ in range(6)]
    timer, rng = ctypes.c_uint32(0), ctypes.c_int32(seed)
    orc.lib().orc_bssn_timestep(ctypes.byref(c), orc.P(orc.ptrs(old6)), orc.P(orc.ptrs(new6)), orc.P(orc.ptrs(dm)),
                                orc.P(orc.ptrs(ch)), orc.P(orc.ptrs(ri)), orc.P(st["positions"]), orc.P(st["children"]),
                                orc.P(st["boundaries"]), used, st["max_depth"], ctypes.byref(timer), ctypes.byref(rng),
                                0, used)
    return {"old": old6, "new": new6, "dmet": dm, "chr": ch, "ricci": ri}


def rel_errors(got: np.ndarray, ref: np.ndarray) -> tuple[float, float]:
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    e = np.abs(got - ref)
    return float(e.max() / (np.abs(ref).max() + 1e-300)), float(np.linalg.norm(e) / (np.linalg.norm(ref) + 1e-300))


def report(orc, single: dict, double: dict, fp32_slack: float = 0.0) -> dict:
    """Per output and component: (max, L2) relative errors; asserts the stated tolerances.
    single holds float arrays and compressed words ('dmet', 'chr' as uint32)."""
    out = {}
    for k in range(6):
        out[f"old{k}"] = rel_errors(single["old"][k], double["old"][k])
        out[f"new{k}"] = rel_errors(single["new"][k], double["new"][k])
        out[f"grad{k}"] = rel_errors(orc.cf3_decode(single["dmet"][k]), double["grad"][k])
        out[f"chr{k}"] = rel_errors(orc.cf3_decode(single["chr"][k]), double["chr"][k])
        out[f"ricci{k}"] = rel_errors(single["ricci"][k], double["ricci"][k])
    for name, (mx, l2) in out.items():
        kind = "metric" if name[:3] in ("old", "new") else name.rstrip("012345")
        tmax, tl2 = TOL[kind]
        print(f"  {name:8s} max {mx:.3e} (<= {tmax:.1e})  L2 {l2:.3e} (<= {tl2:.1e})")
        assert mx <= tmax and l2 <= tl2, f"{name}: max {mx:.3e} L2 {l2:.3e} beyond ({tmax}, {tl2})"
    # per word: the quantisation step bound of the metric gradients
    for k in range(6):
        w = np.asarray(single["dmet"][k], np.uint32)
        step = np.ldexp(1.0, (w >> 27).astype(np.int64) - 15) / 128.0
        dec = orc.cf3_decode(w).astype(np.float64).reshape(-1, 3)
        ref = double["grad"][k].reshape(-1, 3)
        bound = step[:, None] + 1e-5 * np.abs(ref).max(axis=1, keepdims=True) + fp32_slack
        over = np.count_nonzero(np.abs(dec - ref) > bound)
        assert over == 0, f"grad{k}: {over} components beyond one quantisation step"
    return out


def fp32_slack(metric, n, p, st) -> float:
    """Bound of the single-precision rounding of a gradient stencil: 16 ulps of the largest field
    value times the stencil's sum of |weights| (2 suffices for 2nd-6th order) at the finest depth."""
    md = st["max_depth"]
    inv_dx = (1 << md) * n / 100.0
    return 16 * 2.0 ** -24 * 2.0 * max(float(np.abs(m).max()) for m in metric) * inv_dx


@pytest.mark.parametrize("n,p,tree", [(16, 3, "uneven"), (28, 2, "wave")])
def test_timestep_errors_against_fp64(am, orc, n, p, tree):
    o = am.Octree(128)
    cases.ALL_TREES[tree](o)
    st = o.state()
    used = st["used_slots"]
    xyz = cases.cell_coordinates(st["positions"], used, n, p, 100.0)
    metric = cases.metric_fields(xyz, 100.0, 500)
    single = fp32_timestep(orc, n, p, st, metric)
    double = fp64_timestep(orc, n, p, st, metric)
    print(f"\n{tree} tree at {n}/{p}, one timestep, relative errors against FP64:")
    report(orc, single, double, fp32_slack(metric, n, p, st))
    o.close()
