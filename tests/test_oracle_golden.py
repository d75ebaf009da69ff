"""CPU parity against fixtures made from the reference's own host code (tests/golden/host_golden.npz,
written by tests/golden/gen_host_golden.py): the oracle's prng, codec, Morton arithmetic, boundary
words and inverse, and this library's host octree, which must reproduce AMR<T>'s arrays bit for bit
(AdaptiveMesh/AMR.h:118-294).  No GPU is used."""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

import cases
from conftest import GOLDEN
import gen_host_golden as hgen


@pytest.fixture(scope="module")
def hg():
    return np.load(os.path.join(GOLDEN, "host_golden.npz"))


def _u32(a):
    return np.asarray(a).view(np.uint32)


def test_prng_streams(orc, hg):
    L = orc.lib()
    for i, seed in enumerate(hg["prng/seeds"]):
        assert np.array_equal(orc.prng_ints(int(seed), 64), hg["prng/ints"][i]), f"generate_int, seed {seed}"
        s = ctypes.c_int32(int(seed))
        floats = np.array([L.orc_prng_float(ctypes.byref(s)) for _ in range(64)], np.float32)
        assert np.array_equal(_u32(floats), _u32(hg["prng/floats"][i])), f"generate_float, seed {seed}"
        for j, (lo, hi) in enumerate(hg["prng/ranges"]):
            s = ctypes.c_int32(int(seed))
            got = np.array([L.orc_prng_ranged(ctypes.byref(s), int(lo), int(hi)) for _ in range(32)], np.int32)
            assert np.array_equal(got, hg["prng/ranged"][i, j]), f"generate_int({lo},{hi}), seed {seed}"


def test_codec_host_build(orc, hg):
    """The oracle with the host build's float semantics (no flush, no contraction) reproduces the
    reference's host encoder and decoder on every regime of cases.codec_inputs."""
    xyz, seeds = cases.codec_inputs(12_000, 4321)
    assert np.array_equal(orc.cf3_encode_seeded(xyz, seeds, orc.HOST_FLAGS), hg["codec/seeded"])
    assert np.array_equal(orc.cf3_encode_det(xyz, orc.HOST_FLAGS), hg["codec/det"])
    out = np.zeros(len(seeds), np.uint32)
    final = orc.lib().orc_cf3_encode_stream(orc.P(xyz), len(seeds), 77, orc.P(out), orc.HOST_FLAGS)
    assert np.array_equal(out, hg["codec/stream"])
    assert final == int(hg["codec/stream_final_seed"][0])
    dec = orc.cf3_decode(cases.codec_words(len(seeds), 4322))
    assert np.array_equal(_u32(dec), _u32(hg["codec/decoded"]))


def test_morton_arithmetic(orc, hg):
    L = orc.lib()
    a, b = hg["morton/a"], hg["morton/b"]
    for ov in (0, 1):
        s = np.array([L.orc_sum_coordinates(int(x), int(y), ov) for x, y in zip(a, b)], np.uint32)
        d = np.array([L.orc_diff_coordinates(int(x), int(y), ov) for x, y in zip(a, b)], np.uint32)
        assert np.array_equal(s, hg[f"morton/sum{ov}"]), f"yield_sum_coordinates overflow={ov}"
        assert np.array_equal(d, hg[f"morton/diff{ov}"]), f"yield_diff_coordinates overflow={ov}"
    r = np.array([L.orc_reverse_bits(int(x)) for x in hg["morton/rev_in"]], np.uint32)
    assert np.array_equal(r, hg["morton/rev"])


@pytest.mark.parametrize("tree", ["bssn", "uneven"])
def test_boundary_words(orc, hg, tree):
    L = orc.lib()
    pos = hg[f"tree/{tree}/positions"]
    words = np.array([L.orc_boundary(int(pos[i]), int(pos[j]), int(j)) for i, j in hg[f"boundary/{tree}/pairs"]],
                     np.uint64)
    assert np.array_equal(words, hg[f"boundary/{tree}/words"])


def test_inverse_within_contraction_noise(orc, hg):
    """The oracle's inverse follows the device build's contraction; against the host build it
    agrees to within a few ulp of the largest entry (the bound is written here: 2e-6 relative)."""
    L = orc.lib()
    m, ref = hg["inverse/in"], hg["inverse/out"]
    out = np.zeros_like(m)
    for i in range(len(m)):
        L.orc_sym_inverse(m[i].ctypes.data, out[i].ctypes.data)
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(out - ref) <= 2e-6 * scale)


@pytest.mark.parametrize("tree", ["wave", "bssn", "uneven", "uniform2", "uniform3", "root", "deep", "full"])
def test_octree_matches_reference(am, hg, tree):
    """The octree arrays after building each tree equal the reference octree's, including the
    depth limit ('deep'), a full slot array ('full') and the benchmark's tree ('uniform3')."""
    uniform = {"uniform2": (2, 80), "uniform3": (3, 585)}
    o = am.Octree(uniform[tree][1] if tree in uniform else cases.EDGE_SLOTS.get(tree, hgen.SLOTS))
    if tree in uniform:
        cases.tree_uniform(o, uniform[tree][0])
    else:
        cases.ALL_TREES[tree](o)
    st = o.state()
    for k in ("positions", "parent", "children", "boundaries", "lifetime"):
        assert np.array_equal(st[k], hg[f"tree/{tree}/{k}"]), f"{tree}: {k}"
    assert np.array_equal(np.array([st["timer"], st["max_depth"], st["first_free"], st["used_slots"]], np.uint32),
                          hg[f"tree/{tree}/scalars"])
    o.close()


def test_octree_script_matches_reference(am, hg):
    """400 random add / remove / increment_timer / find operations: the state after every one of
    them equals the reference octree's."""
    o = am.Octree(hgen.SLOTS)
    digests, finds = hgen.run_script(o, hg["tree/script/ops"])
    want = hg["tree/script/digests"]
    bad = np.nonzero(digests != want)[0]
    assert bad.size == 0, f"first divergent operation: {bad[0]} {tuple(hg['tree/script/ops'][bad[0]])}"
    assert np.array_equal(finds, hg["tree/script/finds"])
    st = o.state()
    for k in ("positions", "parent", "children", "boundaries", "lifetime"):
        assert np.array_equal(st[k], hg[f"tree/script/final/{k}"]), k
    o.close()


def test_oracle_scan_and_reductions_on_integers(orc):
    """The oracle's restatement of parallel.h on integers: an inclusive scan is the cumulative sum
    (wrapping), the maximum is the maximum, and the minimum counts a partial block's missing
    elements as 0, as the reference's kernel does (parallel.h:389)."""
    rng = np.random.default_rng(7)
    for n in (1, 5, 512, 513, 1000, 262144, 262145):
        for nc in (1, 3):
            a = rng.integers(-1000, 1000, size=n * nc).astype(np.int32)
            b = a.copy()
            orc.lib().orc_scan(1, nc, b.ctypes.data, n)
            assert np.array_equal(b, np.cumsum(a.reshape(n, nc), axis=0).astype(np.int32).ravel())
            r = np.zeros(nc, np.int32)
            work = a.copy()   # named: the oracle writes into it
            orc.lib().orc_extreme(1, nc, 1, work.ctypes.data, n, r.ctypes.data)
            assert np.array_equal(r, a.reshape(n, nc).max(axis=0))
            pos = np.abs(a) + 1
            work = pos.copy()
            orc.lib().orc_extreme(1, nc, 0, work.ctypes.data, n, r.ctypes.data)
            full = n in (1, 512, 262144)   # every pass's blocks are whole
            assert np.array_equal(r, pos.reshape(n, nc).min(axis=0) if full else np.zeros(nc, np.int32)), (n, nc)


def _random_regrid_ops(rng, o, n_ops, max_slots):
    """A random sequence of runs of add_node and of remove_node calls on the octree `o` (applied
    one by one), returned as [(kind, list of arguments)] for replay."""
    runs = []
    for _ in range(n_ops):
        st = o.state()
        live = [i for i in range(st["used_slots"]) if st["positions"][i] != 0xFFFFFFFF]
        if rng.random() < 0.7 or len(live) < 3:
            k = int(rng.integers(1, 12))
            args = []
            for _ in range(k):
                st = o.state()
                live = [i for i in range(st["used_slots"]) if st["positions"][i] != 0xFFFFFFFF]
                parent = int(rng.choice(live)) if rng.random() < 0.9 else int(rng.integers(0, st["used_slots"]))
                args.append((parent, int(rng.integers(0, 8))))
                o.add_node(*args[-1])
            runs.append(("add", args))
        else:
            k = int(rng.integers(1, 4))
            args = []
            for _ in range(k):
                st = o.state()
                live = [i for i in range(1, st["used_slots"]) if st["positions"][i] != 0xFFFFFFFF]
                node = int(rng.choice(live)) if live else 0
                args.append(node)
                o.remove_node(node)
            runs.append(("remove", args))
        if rng.random() < 0.3:
            o.increment_timer()
            runs.append(("timer", []))
    return runs


def test_octree_batches_equal_single_calls(am):
    """amr_octree_add_nodes / amr_octree_remove_nodes leave exactly the state the same calls one
    by one leave (boundaries of every slot, removed ones included, lifetimes, counters)."""
    rng = np.random.default_rng(3)
    for trial in range(6):
        slots = 300
        single = am.Octree(slots)
        runs = _random_regrid_ops(rng, single, 40, slots)
        batched = am.Octree(slots)
        for kind, args in runs:
            if kind == "add":
                batched.add_nodes([a[0] for a in args], [a[1] for a in args])
            elif kind == "remove":
                batched.remove_nodes(args)
            else:
                batched.increment_timer()
            a, b = single.state(), batched.state()
        for k in a:
            assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), (trial, k)
        single.close()
        batched.close()
