"""Generate the device-side golden fixtures from the reference's own CUDA kernels.

Runs on a GPU machine where the reference-build libraries build (oracle/build_ref.py).  For
every case it runs the reference's kernels (through oracle/ref_harness.cu) on the seeded inputs
of tests/golden/cases.py, and the CPU oracle on the same inputs, and writes

  <out>/device_golden.json   sha256 of every reference output buffer, per case
  <out>/device_trees.npz     the reference octree's arrays for every tree the cases build
  <out>/device_patches.npz   for outputs the oracle must reproduce bit for bit: the cells where the
                             oracle's output differs from the reference's, with the reference's
                             values there (expected only for ghost cells the reference's fill
                             computes racily); for the trace g^kl H_kl and the criterion, where the
                             device uses hardware approximations of 1/x and sqrt, every 127th value
                             of the reference's output instead ("<key>/sample")

All three are committed under tests/golden/ and checked on the CPU by tests/test_device_golden.py.

usage: python tests/golden/gen_device_golden.py <out_dir>
"""
from __future__ import annotations

import ctypes
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as orc  # noqa: E402
from oracle import reflib  # noqa: E402
import cases  # noqa: E402

DEV = torch.device("cuda")
SUBSTEPS = cases.substeps_for
SAMPLE_STRIDE = 127


def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def host(t: torch.Tensor) -> np.ndarray:
    a = t.detach().cpu().numpy()
    return a.view(np.uint32) if a.dtype == np.int32 else a


def ptr_array(ts):
    """A C table of device addresses; pass the object itself so it outlives the call."""
    return (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])


class Recorder:
    def __init__(self):
        self.digests: dict = {}
        self.patches: dict = {}
        self.trees: dict = {}

    def tree(self, key: str, st: dict):
        used = st["used_slots"]
        self.trees[f"{key}/positions"] = st["positions"][:used].copy()
        self.trees[f"{key}/parent"] = st["parent"][:used].copy()
        self.trees[f"{key}/children"] = st["children"][: used * 8].copy()
        self.trees[f"{key}/boundaries"] = st["boundaries"][: used * 6].copy()
        self.trees[f"{key}/lifetime"] = st["lifetime"][:used].copy()
        self.trees[f"{key}/scalars"] = np.array([st["timer"], st["max_depth"], st["first_free"], used], np.uint32)

    def put(self, key: str, ref: np.ndarray, oracle_out: np.ndarray | None, approx: bool = False):
        self.digests[key] = cases.digest(ref)
        if approx:   # hardware 1/x or sqrt inside: keep a sample of the reference's values
            self.patches[key + "/sample"] = np.ascontiguousarray(ref[::SAMPLE_STRIDE])
            return
        if oracle_out is None:
            return
        bad = np.nonzero(np.asarray(oracle_out).view(np.uint32) != ref.view(np.uint32))[0]
        if bad.size:
            self.patches[key + "/idx"] = bad.astype(np.uint32)
            self.patches[key + "/val"] = ref[bad]


def codec_case(lib, rec: Recorder):
    xyz, seeds = cases.codec_inputs(200_000, 1234)
    n = len(seeds)
    enc = torch.zeros(n, dtype=torch.int32, device=DEV)
    xd, sd = dev(xyz), dev(seeds)      # named, so they stay allocated while the kernels run
    assert lib.refd_cf3_encode_seeded(xd.data_ptr(), sd.data_ptr(), n, enc.data_ptr()) == 0
    rec.put("codec/enc_stoch", host(enc), orc.cf3_encode_seeded(xyz, seeds, orc.DEVICE_FLAGS))
    det = torch.zeros(n, dtype=torch.int32, device=DEV)
    assert lib.refd_cf3_encode_det(xd.data_ptr(), n, det.data_ptr()) == 0
    rec.put("codec/enc_det", host(det), orc.cf3_encode_det(xyz, orc.DEVICE_FLAGS))
    words = cases.codec_words(200_000, 99)
    dec = torch.zeros(n * 3, dtype=torch.float32, device=DEV)
    wd = dev(words.view(np.int32))
    assert lib.refd_cf3_decode(wd.data_ptr(), n, dec.data_ptr()) == 0
    rec.put("codec/dec", host(dec), orc.cf3_decode(words))
    f = np.load(os.path.join(HERE, "codec_fused_probe_inputs.npz"))
    px, ps = f["xyz"].astype(np.float32), f["seeds"].astype(np.int32)
    pr = torch.zeros(len(ps), dtype=torch.int32, device=DEV)
    pxd, psd = dev(px), dev(ps)
    assert lib.refd_cf3_encode_seeded(pxd.data_ptr(), psd.data_ptr(), len(ps), pr.data_ptr()) == 0
    rec.put("codec/noise_rounding", host(pr), orc.cf3_encode_seeded(px, ps, orc.DEVICE_FLAGS))


def kernel_case(lib, cfgname: str, tree: str, rec: Recorder):
    c = reflib.constants(lib)
    N, P, OS = c["size_domain"], c["padding_domain"], c["outer_size"]
    o = reflib.RefOctree(lib, 64)
    cases.TREES[tree](o)
    st = o.state()
    used, md = st["used_slots"], st["max_depth"]
    inner = N ** 3
    xyz = cases.cell_coordinates(st["positions"], used, N, P, OS)
    pos, ch, bd = st["positions"], st["children"], st["boundaries"]
    pos_d, ch_d, bd_d = dev(pos[:used].view(np.int32)), dev(ch[: used * 8]), dev(bd[: used * 6].view(np.int64))
    f_old = cases.smooth_field(xyz, OS, 1, 11)
    f_new = cases.smooth_field(xyz, OS, 1, 12)
    metric = cases.metric_fields(xyz, OS, 300)
    oc = orc.cfg(N, P, OS)
    L = orc.lib()
    C = ctypes.byref(oc)
    key = f"{cfgname}/{tree}"
    rec.tree(key, st)
    zu = lambda: torch.zeros(used * inner, dtype=torch.int32, device=DEV)  # noqa: E731
    for s in SUBSTEPS(md):
        seed = 1000 + 17 * s
        tag = f"{key}/s{s}"
        fd = dev(f_old)
        dif, d2, g1, off = zu(), zu(), zu(), zu()
        assert lib.refd_differentiate(fd.data_ptr(), dif.data_ptr(), d2.data_ptr(), pos_d.data_ptr(), used, s, md, seed) == 0
        assert lib.refd_differentiate(fd.data_ptr(), g1.data_ptr(), None, pos_d.data_ptr(), used, s, md, seed + 1) == 0
        assert lib.refd_mixed_partials(fd.data_ptr(), off.data_ptr(), pos_d.data_ptr(), used, s, md, seed + 2) == 0
        o_dif, o_d2, o_g1, o_off = (np.zeros(used * inner, np.uint32) for _ in range(4))
        L.orc_differentiate(C, orc.P(f_old), orc.P(o_dif), orc.P(o_d2), orc.P(pos), used, s, md, seed)
        L.orc_differentiate(C, orc.P(f_old), orc.P(o_g1), None, orc.P(pos), used, s, md, seed + 1)
        L.orc_mixed_partials(C, orc.P(f_old), orc.P(o_off), orc.P(pos), used, s, md, seed + 2)
        for nm, r_, o_ in (("dif", dif, o_dif), ("d2", d2, o_d2), ("grad", g1, o_g1), ("off", off, o_off)):
            rec.put(f"{tag}/{nm}", host(r_), o_)
        mets = [dev(m) for m in metric]
        lap = torch.zeros(used * inner, dtype=torch.float32, device=DEV)
        assert lib.refd_deriv_trace(d2.data_ptr(), off.data_ptr(), ptr_array(mets), lap.data_ptr(), pos_d.data_ptr(), used, s, md) == 0
        h_d2, h_off = host(d2), host(off)
        o_lap = np.zeros(used * inner, np.float32)
        L.orc_deriv_trace(C, orc.P(h_d2), orc.P(h_off), orc.ptrs(metric), orc.P(o_lap), orc.P(pos), used, s, md)
        rec.put(f"{tag}/lap", host(lap), o_lap, approx=True)
        mder = [zu() for _ in range(6)]
        for k in range(6):
            assert lib.refd_differentiate(mets[k].data_ptr(), mder[k].data_ptr(), None, pos_d.data_ptr(), used, s, md, seed + 10 + k) == 0
        chr_ = [zu() for _ in range(6)]
        assert lib.refd_christoffel(ptr_array(mets), ptr_array(mder), seed + 20, ptr_array(chr_), pos_d.data_ptr(), used, s, md) == 0
        h_mder = [host(t) for t in mder]
        o_chr = [np.zeros(used * inner, np.uint32) for _ in range(6)]
        L.orc_christoffel(C, orc.ptrs(metric), orc.ptrs(h_mder), seed + 20, orc.ptrs(o_chr), orc.P(pos), used, s, md, 0)
        for k in range(6):
            o_m = np.zeros(used * inner, np.uint32)
            L.orc_differentiate(C, orc.P(metric[k]), orc.P(o_m), None, orc.P(pos), used, s, md, seed + 10 + k)
            rec.put(f"{tag}/mder{k}", h_mder[k], o_m)
            rec.put(f"{tag}/chr{k}", host(chr_[k]), o_chr[k])
        for only_new in (0, 1):
            go, gn = dev(f_old), dev(f_new)
            assert lib.refd_copy_boundaries(go.data_ptr(), gn.data_ptr(), bd_d.data_ptr(), used, s, md, only_new) == 0
            oo, on = f_old.copy(), f_new.copy()
            L.orc_copy_boundaries(C, orc.P(oo), orc.P(on), orc.P(bd), used, s, md, only_new)
            rec.put(f"{tag}/ghost{only_new}_old", host(go), oo)
            rec.put(f"{tag}/ghost{only_new}_new", host(gn), on)
        ro = dev(f_old)
        rn = dev(f_new)
        assert lib.refd_copy_new_to_old(ro.data_ptr(), rn.data_ptr(), pos_d.data_ptr(), ch_d.data_ptr(), used, s, md) == 0
        oo = f_old.copy()
        L.orc_copy_new_to_old(C, orc.P(oo), orc.P(f_new), orc.P(pos), orc.P(ch), used, s, md)
        rec.put(f"{tag}/restrict", host(ro), oo)
        h_dif = host(dif)
        for corr in (0, 1):
            w = dev(f_new)
            assert lib.refd_wave_step(corr, fd.data_ptr(), dif.data_ptr(), d2.data_ptr(), w.data_ptr(), pos_d.data_ptr(), used, s, md) == 0
            ow = f_new.copy()
            L.orc_wave_step(C, corr, orc.P(f_old), orc.P(h_dif), orc.P(h_d2), orc.P(ow), orc.P(pos), used, s, md)
            rec.put(f"{tag}/wave{corr}", host(w), ow)
        cr = torch.zeros(used * N * N, dtype=torch.float32, device=DEV)
        if lib.refd_criterion(dif.data_ptr(), d2.data_ptr(), cr.data_ptr(), pos_d.data_ptr(), used, s, md) == 0:
            r = host(cr)
            # NaN payloads (inactive columns) are not part of the comparison: canonicalise them
            rec.put(f"{tag}/crit", np.where(np.isnan(r), np.float32(np.nan), r), None, approx=True)
    pb = dev(f_old)
    ob = f_old.copy()
    for child in range(1, used):
        p_ = int(pos[child])
        off_ = (p_ >> (((p_ >> 27) - 1) * 3)) & 7
        assert lib.refd_copy_to_child(pb.data_ptr(), off_, child, int(st["parent"][child])) == 0
        L.orc_copy_to_child(C, orc.P(ob), off_, child, int(st["parent"][child]))
    rec.put(f"{key}/prolong", host(pb), ob)
    o.close()


def plugin_case(lib, cfgname: str, rec: Recorder):
    """BSSN_AMR_data::timestep on the root-plus-eight tree (no racy ghost reads at size 16)."""
    c = reflib.constants(lib)
    N, P, OS = c["size_domain"], c["padding_domain"], c["outer_size"]
    T = N + 2 * P
    h = lib.refd_bssn_create(128)
    for cidx in range(8):
        lib.refd_bssn_add_node(h, 0, cidx)
    st = reflib.octree_state(lib.refd_bssn_octree_state, h, 128)
    used = st["used_slots"]
    rec.tree(f"{cfgname}/plugin_bssn", st)
    xyz = cases.cell_coordinates(st["positions"], used, N, P, OS)
    metric = cases.metric_fields(xyz, OS, 500)
    for which in (0, 1):
        for k in range(6):
            dst = _wrap(lib.refd_bssn_field(h, which, k), used * T ** 3, torch.float32)
            dst.copy_(torch.from_numpy(metric[k]).cuda())
    torch.cuda.synchronize()
    seed0 = int(lib.refd_bssn_rng_seed(h))
    assert lib.refd_bssn_timestep(h) == 0
    old6 = [m.copy() for m in metric]
    new6 = [m.copy() for m in metric]
    dm = [np.zeros(used * N ** 3, np.uint32) for _ in range(6)]
    chr6 = [np.zeros(used * N ** 3, np.uint32) for _ in range(6)]
    ri = [np.zeros(used * N ** 3, np.float32) for _ in range(6)]
    timer, rng = ctypes.c_uint32(0), ctypes.c_int32(seed0)
    oc = orc.cfg(N, P, OS)
    orc.lib().orc_bssn_timestep(ctypes.byref(oc), orc.ptrs(old6), orc.ptrs(new6), orc.ptrs(dm), orc.ptrs(chr6),
                                orc.ptrs(ri), orc.P(st["positions"]), orc.P(st["children"]), orc.P(st["boundaries"]),
                                used, st["max_depth"], ctypes.byref(timer), ctypes.byref(rng), 0, used)
    key = f"{cfgname}/plugin_bssn"
    for k in range(6):
        rec.put(f"{key}/old{k}", _wrap(lib.refd_bssn_field(h, 0, k), used * T ** 3, torch.float32).cpu().numpy(), old6[k])
        rec.put(f"{key}/new{k}", _wrap(lib.refd_bssn_field(h, 1, k), used * T ** 3, torch.float32).cpu().numpy(), new6[k])
        rec.put(f"{key}/ricci{k}", _wrap(lib.refd_bssn_field(h, 2, k), used * N ** 3, torch.float32).cpu().numpy(), ri[k], approx=True)
        rec.put(f"{key}/dmet{k}", host(_wrap(lib.refd_bssn_cf3(h, 0, k), used * N ** 3, torch.int32)), dm[k])
        rec.put(f"{key}/chr{k}", host(_wrap(lib.refd_bssn_cf3(h, 1, k), used * N ** 3, torch.int32)), chr6[k])
    rec.digests[f"{key}/rng"] = int(lib.refd_bssn_rng_seed(h))
    assert rec.digests[f"{key}/rng"] == rng.value
    lib.refd_bssn_destroy(h)


def _wrap(addr: int, n: int, dtype) -> torch.Tensor:
    """A torch view of raw device memory (n elements of dtype at addr)."""
    class _Mem:
        __cuda_array_interface__ = {"shape": (n,), "typestr": {torch.float32: "<f4", torch.int32: "<i4"}[dtype],
                                    "data": (addr, False), "version": 3}
    return torch.as_tensor(_Mem(), device=DEV)


def main():
    out_dir = sys.argv[1]
    os.makedirs(out_dir, exist_ok=True)
    rec = Recorder()
    lib28, lib16 = reflib.load("n28p2"), reflib.load("n16p3")
    codec_case(lib28, rec)
    for cfgname, lib in (("n28p2", lib28), ("n16p3", lib16)):
        for tree in ("wave", "uneven", "bssn"):
            kernel_case(lib, cfgname, tree, rec)
            torch.cuda.synchronize()
    plugin_case(lib16, "n16p3", rec)
    with open(os.path.join(out_dir, "device_golden.json"), "w") as f:
        json.dump(rec.digests, f, indent=0, sort_keys=True)
    np.savez_compressed(os.path.join(out_dir, "device_patches.npz"), **rec.patches)
    np.savez_compressed(os.path.join(out_dir, "device_trees.npz"), **rec.trees)
    counts = {k[:-4]: int(v.size) for k, v in rec.patches.items() if k.endswith("/idx")}
    print("digests:", len(rec.digests), "patched outputs:", len(counts),
          "sampled outputs:", sum(k.endswith("/sample") for k in rec.patches))
    for k in sorted(counts):
        print(f"  {k}: {counts[k]}")


if __name__ == "__main__":
    main()
