"""Generate device-side golden fixtures from the reference's own CUDA kernels.

Runs on a GPU machine with the reference checker libraries built (oracle/build_ref.py).
For every case it runs the reference's kernels (through oracle/ref_harness.cu) on the
seeded inputs of tests/golden/cases.py and writes
  <out>/device_golden.json   -- sha256 digests of every output buffer (committed as
                                tests/golden/device_golden.json)
  <out>/<case>.npz           -- the full outputs, for small cases (a subset is committed)

usage: python tests/golden/gen_device_golden.py <out_dir> <n28p2|n16p3>
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import reflib  # noqa: E402
import cases  # noqa: E402

DEV = torch.device("cuda")


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def host(t: torch.Tensor) -> np.ndarray:
    return t.detach().cpu().numpy()


def ptr_array(ts):
    """A C table of device addresses; pass the object itself so it outlives the call."""
    import ctypes
    return (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])


def substeps_for(max_depth: int) -> list[int]:
    s = {0, 1, (1 << max_depth) - 1}
    if max_depth >= 2:
        s.add((1 << (max_depth - 1)) + 1)
    return sorted(x for x in s if x < (1 << max_depth))


def codec_case(lib, out: dict, full: dict):
    xyz, seeds = cases.codec_inputs(200_000, 1234)
    n = len(seeds)
    xd, sd = dev(xyz), dev(seeds)
    enc = torch.zeros(n, dtype=torch.int32, device=DEV)
    assert lib.refd_cf3_encode_seeded(xd.data_ptr(), sd.data_ptr(), n, enc.data_ptr()) == 0
    det = torch.zeros(n, dtype=torch.int32, device=DEV)
    assert lib.refd_cf3_encode_det(xd.data_ptr(), n, det.data_ptr()) == 0
    words = np.random.default_rng(99).integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    dec = torch.zeros(n * 3, dtype=torch.float32, device=DEV)
    assert lib.refd_cf3_decode(dev(words.view(np.int32)).data_ptr(), n, dec.data_ptr()) == 0
    pf = torch.zeros(n * 4, dtype=torch.float32, device=DEV)
    assert lib.refd_prng_floats(sd.data_ptr(), n, 4, pf.data_ptr()) == 0
    r = {"enc_stoch": host(enc).view(np.uint32), "enc_det": host(det).view(np.uint32),
         "dec": host(dec), "prng4": host(pf)}
    for k, v in r.items():
        out[f"codec/{k}"] = cases.digest(v)
    full["codec"] = r


def probe_case(lib, out: dict, full: dict):
    rng = np.random.default_rng(7)
    n = 100_000
    res = {}
    for kind, width in [(0, 9), (1, 12), (4, 3), (5, 6)]:
        x = rng.standard_normal((n, width)).astype(np.float32)
        if kind in (0, 5):
            x[:, [0, 3, 5]] += 1.0
        ow = {0: 3, 1: 1, 4: 1, 5: 1}[kind]
        o = torch.zeros(n * ow, dtype=torch.float32, device=DEV)
        assert lib.refd_probe(kind, dev(x).data_ptr(), n, o.data_ptr()) == 0
        res[f"in{kind}"] = x
        res[f"out{kind}"] = host(o)
        out[f"probe/{kind}"] = cases.digest(res[f"out{kind}"])
    d = np.arange(9, dtype=np.float32)
    o = torch.zeros(9, dtype=torch.float32, device=DEV)
    assert lib.refd_probe(3, dev(d).data_ptr(), 9, o.data_ptr()) == 0
    res["out3"] = host(o)
    out["probe/3"] = cases.digest(res["out3"])
    m = rng.standard_normal((n, 6)).astype(np.float32) * 0.1
    m[:, [0, 3, 5]] += 1.0
    o = torch.zeros(n * 6, dtype=torch.float32, device=DEV)
    assert lib.refd_sym_inverse(dev(m).data_ptr(), n, o.data_ptr()) == 0
    res["inv_in"] = m
    res["inv_out"] = host(o)
    out["probe/inverse"] = cases.digest(res["inv_out"])
    full["probes"] = res


def kernel_case(lib, cfgname: str, tree: str, out: dict, full: dict, keep_full: bool):
    c = reflib.constants(lib)
    N, P, T, OS = c["size_domain"], c["padding_domain"], c["total"], c["outer_size"]
    o = reflib.RefOctree(lib, 64)
    cases.TREES[tree](o)
    st = o.state()
    used, md = st["used_slots"], st["max_depth"]
    cells, inner = T ** 3, N ** 3
    xyz = cases.cell_coordinates(st["positions"], used, N, P, OS)
    pos_d = dev(st["positions"][:used].view(np.int32))
    ch_d = dev(st["children"][: used * 8])
    bd_d = dev(st["boundaries"][: used * 6].view(np.int64))
    f_old = cases.smooth_field(xyz, OS, 1, 11)
    f_new = cases.smooth_field(xyz, OS, 1, 12)
    metric = cases.metric_fields(xyz, OS, 300)
    key = f"{cfgname}/{tree}"
    res = {"positions": st["positions"][:used], "children": st["children"][: used * 8],
           "boundaries": st["boundaries"][: used * 6], "max_depth": np.int32(md), "used": np.int32(used)}
    z_cf3 = lambda: torch.zeros(used * inner, dtype=torch.int32, device=DEV)  # noqa: E731
    z_in = lambda: torch.zeros(used * inner, dtype=torch.float32, device=DEV)  # noqa: E731
    for s in substeps_for(md):
        seed = 1000 + 17 * s
        tag = f"{key}/s{s}"
        fd = dev(f_old)
        # fused gradient + diagonal Hessian, and gradient only
        dif, d2 = z_cf3(), z_cf3()
        assert lib.refd_differentiate(fd.data_ptr(), dif.data_ptr(), d2.data_ptr(), pos_d.data_ptr(), used, s, md, seed) == 0
        g1 = z_cf3()
        assert lib.refd_differentiate(fd.data_ptr(), g1.data_ptr(), None, pos_d.data_ptr(), used, s, md, seed + 1) == 0
        off = z_cf3()
        assert lib.refd_mixed_partials(fd.data_ptr(), off.data_ptr(), pos_d.data_ptr(), used, s, md, seed + 2) == 0
        # deriv trace with the metric
        mets = [dev(m) for m in metric]
        mp = ptr_array(mets)
        lap = z_in()
        assert lib.refd_deriv_trace(d2.data_ptr(), off.data_ptr(), mp, lap.data_ptr(), pos_d.data_ptr(), used, s, md) == 0
        # metric derivatives + Christoffel symbols
        mder = [z_cf3() for _ in range(6)]
        for k in range(6):
            assert lib.refd_differentiate(mets[k].data_ptr(), mder[k].data_ptr(), None, pos_d.data_ptr(), used, s, md, seed + 10 + k) == 0
        chr_ = [z_cf3() for _ in range(6)]
        assert lib.refd_christoffel(mp, ptr_array(mder), seed + 20, ptr_array(chr_),
                                    pos_d.data_ptr(), used, s, md) == 0
        # ghost fill: both modes
        go, gn = dev(f_old), dev(f_new)
        assert lib.refd_copy_boundaries(go.data_ptr(), gn.data_ptr(), bd_d.data_ptr(), used, s, md, 0) == 0
        go2, gn2 = dev(f_old), dev(f_new)
        assert lib.refd_copy_boundaries(go2.data_ptr(), gn2.data_ptr(), bd_d.data_ptr(), used, s, md, 1) == 0
        # restriction
        ro = dev(f_old)
        assert lib.refd_copy_new_to_old(ro.data_ptr(), dev(f_new).data_ptr(), pos_d.data_ptr(), ch_d.data_ptr(), used, s, md) == 0
        # SimpleWave predictor / corrector (derivatives from the fused kernel above)
        wn = dev(f_new)
        assert lib.refd_wave_step(0, fd.data_ptr(), dif.data_ptr(), d2.data_ptr(), wn.data_ptr(), pos_d.data_ptr(), used, s, md) == 0
        wc = dev(f_new)
        assert lib.refd_wave_step(1, fd.data_ptr(), dif.data_ptr(), d2.data_ptr(), wc.data_ptr(), pos_d.data_ptr(), used, s, md) == 0
        # refinement criterion
        cr = torch.zeros(used * N * N, dtype=torch.float32, device=DEV)
        rc = lib.refd_criterion(dif.data_ptr(), d2.data_ptr(), cr.data_ptr(), pos_d.data_ptr(), used, s, md)
        r = {"dif": dif, "d2": d2, "grad": g1, "off": off, "lap": lap, "ghost_old": go, "ghost_new": gn,
             "ghost_new_only": gn2, "ghost_old_only": go2, "restrict": ro, "pred": wn, "corr": wc}
        if rc == 0:
            r["crit"] = cr
        else:
            # the reference's launch shape for the criterion is empty at this domain size
            # (SimpleWave.h:146-147: grid y = (n/2) / threadsF = 0 when n = 16)
            out[f"{tag}/crit"] = f"launch_error:{rc}"
        for k in range(6):
            r[f"mder{k}"] = mder[k]
            r[f"chr{k}"] = chr_[k]
        for k, v in r.items():
            a = host(v)
            if a.dtype == np.int32:
                a = a.view(np.uint32)
            out[f"{tag}/{k}"] = cases.digest(a)
            if keep_full:
                res[f"s{s}/{k}"] = a
    # prolongation into every non-root node, in slot order (as node_ctor does on add_node)
    pb = dev(f_old)
    par = st["parent"]
    for child in range(1, used):
        if st["positions"][child] == 0xFFFFFFFF:
            continue
        offset = (int(st["positions"][child]) >> ((((int(st["positions"][child]) >> 27)) - 1) * 3)) & 7
        assert lib.refd_copy_to_child(pb.data_ptr(), offset, child, int(par[child])) == 0
    a = host(pb)
    out[f"{key}/prolong"] = cases.digest(a)
    if keep_full:
        res["prolong"] = a
        full[f"kern_{cfgname}_{tree}"] = res
    o.close()


def plugin_case(lib, cfgname: str, out: dict, full: dict, keep_full: bool):
    c = reflib.constants(lib)
    N, P, T, OS = c["size_domain"], c["padding_domain"], c["total"], c["outer_size"]
    cells = T ** 3
    # BSSN_AMR_data on the nested tree: set the metric, one timestep, read everything back
    for tree in ("wave", "bssn"):
        h = lib.refd_bssn_create(128)
        helper = _PluginTree(lib, h, "bssn", 128)
        cases.TREES[tree](helper)
        st = helper.state()
        used = st["used_slots"]
        xyz = cases.cell_coordinates(st["positions"], used, N, P, OS)
        metric = cases.metric_fields(xyz, OS, 500)
        for which in (0, 1):
            for k in range(6):
                p = lib.refd_bssn_field(h, which, k)
                t = torch.from_numpy(metric[k]).to(DEV)
                torch.cuda.synchronize()
                _memcpy_d2d(p, t.data_ptr(), t.numel() * 4)
        assert lib.refd_bssn_timestep(h) == 0
        key = f"{cfgname}/plugin_bssn_{tree}"
        res = {}
        for which, name in ((0, "old"), (1, "new"), (2, "ricci")):
            for k in range(6):
                n_el = used * (cells if which < 2 else N ** 3)
                a = _fetch(lib.refd_bssn_field(h, which, k), n_el, np.float32)
                out[f"{key}/{name}{k}"] = cases.digest(a)
                res[f"{name}{k}"] = a
        for which, name in ((0, "dmet"), (1, "chr")):
            for k in range(6):
                a = _fetch(lib.refd_bssn_cf3(h, which, k), used * N ** 3, np.uint32)
                out[f"{key}/{name}{k}"] = cases.digest(a)
                res[f"{name}{k}"] = a
        out[f"{key}/rng"] = int(lib.refd_bssn_rng_seed(h))
        if keep_full and tree == "wave":
            full[f"plugin_bssn_{cfgname}_{tree}"] = res
        lib.refd_bssn_destroy(h)
    # wave_AMR_data: seed the root, add eight children (prolongation), fill ghosts, three timesteps.
    # Its regrid step needs the criterion kernels, which only launch when threadsF divides n/2.
    if N % 4 != 0 or (N // 2) % min(16, max(d for d in range(1, 17) if N % d == 0)) != 0:
        out[f"{cfgname}/plugin_wave"] = "skipped: reference criterion launch is empty at this size"
        return
    h = lib.refd_wave_create(128)
    st0 = reflib.octree_state(lib.refd_wave_octree_state, h, 128)
    xyz = cases.cell_coordinates(st0["positions"], 1, N, P, OS)
    f0 = cases.smooth_field(xyz, OS, 0, 77, noise=0.0) * np.float32(0.5)
    for which in (0, 1):
        t = torch.from_numpy(f0).to(DEV)
        _memcpy_d2d(lib.refd_wave_field(h, which), t.data_ptr(), t.numel() * 4)
    torch.cuda.synchronize()
    for cidx in range(8):
        lib.refd_wave_add_node(h, 0, cidx)
    assert lib.refd_wave_copy_bounds(h) == 0
    key = f"{cfgname}/plugin_wave"
    res = {}
    for step in range(3):
        assert lib.refd_wave_timestep(h) == 0
        st = reflib.octree_state(lib.refd_wave_octree_state, h, 128)
        used = st["used_slots"]
        for nm in ("positions", "parent", "children", "boundaries", "lifetime"):
            out[f"{key}/t{step}/{nm}"] = cases.digest(st[nm])
            res[f"t{step}/{nm}"] = st[nm]
        out[f"{key}/t{step}/scalars"] = [st["timer"], st["max_depth"], st["first_free"], st["used_slots"]]
        for which, name in ((0, "old"), (1, "new")):
            a = _fetch(lib.refd_wave_field(h, which), used * cells, np.float32)
            out[f"{key}/t{step}/{name}"] = cases.digest(a)
            res[f"t{step}/{name}"] = a
        out[f"{key}/t{step}/rng"] = int(lib.refd_wave_rng_seed(h))
    if keep_full:
        full[f"plugin_wave_{cfgname}"] = res
    lib.refd_wave_destroy(h)


class _PluginTree:
    """Adapter so cases.TREES builders can drive a reference plugin's octree."""

    def __init__(self, lib, h, kind, slots):
        self.lib, self.h, self.kind, self.slots = lib, h, kind, slots

    def add_node(self, parent, offset):
        getattr(self.lib, f"refd_{self.kind}_add_node")(self.h, parent, offset)

    def state(self):
        return reflib.octree_state(getattr(self.lib, f"refd_{self.kind}_octree_state"), self.h, self.slots)


def _memcpy_d2d(dst: int, src: int, nbytes: int):
    dst_t = _wrap(dst, nbytes // 4, torch.float32)
    src_t = _wrap(src, nbytes // 4, torch.float32)
    dst_t.copy_(src_t)
    torch.cuda.synchronize()


def _wrap(addr: int, n: int, dtype) -> torch.Tensor:
    """A torch view of raw device memory (n elements of dtype at addr)."""
    class _Holder:
        pass
    h = _Holder()
    h.__cuda_array_interface__ = {"shape": (n,), "typestr": {torch.float32: "<f4", torch.int32: "<i4"}[dtype],
                                  "data": (addr, False), "version": 3}
    return torch.as_tensor(h, device=DEV)


def _fetch(addr: int, n: int, dtype) -> np.ndarray:
    t = _wrap(addr, n, torch.int32 if dtype == np.uint32 else torch.float32)
    a = t.cpu().numpy()
    return a.view(np.uint32) if dtype == np.uint32 else a


def main():
    out_dir, cfgname = sys.argv[1], sys.argv[2]
    os.makedirs(out_dir, exist_ok=True)
    digests: dict = {}
    full: dict = {}
    lib = reflib.load(cfgname)
    if cfgname == "n28p2":
        codec_case(lib, digests, full)
        probe_case(lib, digests, full)
    else:
        d = np.arange(9, dtype=np.float32)
        o = torch.zeros(9, dtype=torch.float32, device=DEV)
        assert lib.refd_probe(3, dev(d).data_ptr(), 9, o.data_ptr()) == 0
        full["dx1_n16p3"] = {"out3": host(o)}
    for tree in ("wave", "uneven", "bssn"):
        kernel_case(lib, cfgname, tree, digests, full, keep_full=(cfgname == "n16p3" and tree != "bssn")
                    or (cfgname == "n28p2" and tree == "wave"))
        torch.cuda.synchronize()
    plugin_case(lib, cfgname, digests, full, keep_full=(cfgname == "n16p3"))
    with open(os.path.join(out_dir, f"device_golden_{cfgname}.json"), "w") as f:
        json.dump(digests, f, indent=0, sort_keys=True)
    for name, res in full.items():
        np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **{k.replace("/", "__"): np.asarray(v) for k, v in res.items()})
    print("cases:", len(digests), "files:", sorted(full))


if __name__ == "__main__":
    main()
