"""Generate the host-side golden fixture from the reference's own host code.

Runs on a machine with the reference sources (the reference-build library oracle/_ref/libamr_ref_n28p2.so
is built from them by oracle/build_ref.py; no GPU is needed: only its refh_* entry points, which
run the reference's __host__ code, are called).  Writes <out>/host_golden.npz with

  prng/*       fast_prng streams (AdaptiveMesh/tensors.h:276-304) for a set of seeds
  codec/*      compressed_float3 host encodes and decodes (tensors.h:305-394) of
               tests/golden/cases.codec_inputs: a shared-generator stream, per-element seeds, the
               deterministic encoder, and random words decoded
  morton/*     yield_sum_coordinates / yield_diff_coordinates / reverse_bits on random operands
  boundary/*   domain_boundary words between every pair of nodes of the 'bssn' and 'uneven' trees
  inverse/*    float3x3_sym::inverse on random symmetric positive-definite matrices
  tree/<name>/*  the octree arrays (AMR.h:118-294) after building each tree of cases.TREES and
               cases.EDGE_TREES (depth limit, full slot array), uniform depth-2 and depth-3 trees and a random
               script of add / remove / timer / find
               operations; for the script also the state digest after every operation

The committed copy is tests/golden/host_golden.npz, checked on the CPU by
tests/test_oracle_golden.py against the oracle and against this library's host octree.

usage: python tests/golden/gen_host_golden.py <out_dir>
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import cases  # noqa: E402

SLOTS = 64
PRNG_SEEDS = np.array([0, 1, -1, 7, 12894712, 2 ** 31 - 1, -2 ** 31, 123456789, -987654321], np.int32)
RANGES = [(0, 8), (-5, 5), (0, 1), (100, 100000), (-2 ** 30, 2 ** 30)]


def state_digest(st: dict) -> str:
    h = hashlib.sha256()
    for k in ("positions", "parent", "children", "boundaries", "lifetime"):
        h.update(np.ascontiguousarray(st[k]).tobytes())
    h.update(np.array([st["timer"], st["max_depth"], st["first_free"], st["used_slots"]], np.uint32).tobytes())
    return h.hexdigest()


def put_state(out: dict, key: str, st: dict):
    for k in ("positions", "parent", "children", "boundaries", "lifetime"):
        out[f"{key}/{k}"] = np.ascontiguousarray(st[k]).copy()
    out[f"{key}/scalars"] = np.array([st["timer"], st["max_depth"], st["first_free"], st["used_slots"]], np.uint32)


def octree_script(seed: int, n_ops: int) -> np.ndarray:
    """A random but valid operation script, as rows (op, a, b): 0 add(parent a, offset b),
    1 remove(node a), 2 increment_timer, 3 find(packed a, max depth b).  Node indices refer to
    the tree as it stands when the row runs, so the script is replayed against a live octree
    (run_script resolves them)."""
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(n_ops):
        r = rng.random()
        op = 0 if r < 0.55 else 1 if r < 0.7 else 2 if r < 0.9 else 3
        rows.append((op, int(rng.integers(0, 2 ** 31)), int(rng.integers(0, 2 ** 31))))
    return np.array(rows, np.int64)


def run_script(o, script: np.ndarray):
    """Replay a script on an octree object (the reference's or this library's).  Random draws
    are mapped onto the live tree deterministically, so both replays take the same choices as long
    as their states agree.  Returns (per-op state digests, find results)."""
    digests, finds = [], []
    for op, a, b in script:
        st = o.state()
        live = [i for i in range(st["used_slots"]) if st["positions"][i] != 0xFFFFFFFF]
        if op == 0:
            parents = [i for i in live if (int(st["positions"][i]) >> 27) < 5]
            o.add_node(parents[a % len(parents)], b & 7)
        elif op == 1:
            nodes = [i for i in live if i != 0]
            if nodes:
                o.remove_node(nodes[a % len(nodes)])
        elif op == 2:
            o.increment_timer()
        else:
            finds.append(o.find_node_idx(a & ((1 << 27) - 1), b % 8 if b % 5 else 0xFFFFFFFF))
        digests.append(state_digest(o.state()))
    return np.array(digests), np.array(finds, np.uint32)


def main(out_dir: str):
    from oracle import reflib
    lib = reflib.load("n28p2")
    out: dict = {}
    # prng
    out["prng/seeds"] = PRNG_SEEDS
    ints = np.zeros((len(PRNG_SEEDS), 64), np.int32)
    floats = np.zeros((len(PRNG_SEEDS), 64), np.float32)
    ranged = np.zeros((len(PRNG_SEEDS), len(RANGES), 32), np.int32)
    for i, s in enumerate(PRNG_SEEDS):
        lib.refh_prng_ints(int(s), 64, ints[i].ctypes.data)
        lib.refh_prng_floats(int(s), 64, floats[i].ctypes.data)
        for j, (lo, hi) in enumerate(RANGES):
            lib.refh_prng_ranged(int(s), 32, lo, hi, ranged[i, j].ctypes.data)
    out["prng/ints"], out["prng/floats"], out["prng/ranged"] = ints, floats, ranged
    out["prng/ranges"] = np.array(RANGES, np.int32)
    # codec (host build: no flush-to-zero, no contraction)
    xyz, seeds = cases.codec_inputs(12_000, 4321)
    n = len(seeds)
    enc = np.zeros(n, np.uint32)
    lib.refh_cf3_encode_seeded(xyz.ctypes.data, seeds.ctypes.data, n, enc.ctypes.data)
    det = np.zeros(n, np.uint32)
    lib.refh_cf3_encode_det(xyz.ctypes.data, n, det.ctypes.data)
    stream = np.zeros(n, np.uint32)
    final = lib.refh_cf3_encode_stream(xyz.ctypes.data, n, 77, stream.ctypes.data)
    words = cases.codec_words(n, 4322)
    dec = np.zeros(3 * n, np.float32)
    lib.refh_cf3_decode(words.ctypes.data, n, dec.ctypes.data)
    out.update({"codec/seeded": enc, "codec/det": det, "codec/stream": stream,
                "codec/stream_final_seed": np.array([final], np.int32), "codec/decoded": dec})
    # Morton arithmetic
    rng = np.random.default_rng(31)
    a = rng.integers(0, 2 ** 27, 8_000).astype(np.uint32)
    b = rng.integers(0, 2 ** 27, 8_000).astype(np.uint32)
    b[::3] &= np.uint32(0o1111111111 * 7 & ((1 << 27) - 1))   # sparse offsets, like face directions
    out["morton/a"], out["morton/b"] = a, b
    for ov in (0, 1):
        out[f"morton/sum{ov}"] = np.array([lib.refh_sum_coordinates(int(x), int(y), ov) for x, y in zip(a, b)], np.uint32)
        out[f"morton/diff{ov}"] = np.array([lib.refh_diff_coordinates(int(x), int(y), ov) for x, y in zip(a, b)], np.uint32)
    r = rng.integers(0, 2 ** 32, 8_000, dtype=np.uint64).astype(np.uint32)
    out["morton/rev_in"] = r
    out["morton/rev"] = np.array([lib.refh_reverse_bits(int(x)) for x in r], np.uint32)
    # octrees
    for name in ("wave", "bssn", "uneven"):
        o = reflib.RefOctree(lib, SLOTS)
        cases.TREES[name](o)
        put_state(out, f"tree/{name}", o.state())
        if name in ("bssn", "uneven"):
            st = o.state()
            used = st["used_slots"]
            pos = st["positions"][:used]
            pairs = [(i, j) for i in range(used) for j in range(used)]
            out[f"boundary/{name}/pairs"] = np.array(pairs, np.int32)
            out[f"boundary/{name}/words"] = np.array(
                [lib.refh_boundary(int(pos[i]), int(pos[j]), j) for i, j in pairs], np.uint64)
        o.close()
    for name, build in cases.EDGE_TREES.items():
        o = reflib.RefOctree(lib, cases.EDGE_SLOTS[name])
        build(o)
        put_state(out, f"tree/{name}", o.state())
        o.close()
    o = reflib.RefOctree(lib, 80)
    cases.tree_uniform(o, 2)
    put_state(out, "tree/uniform2", o.state())
    o.close()
    # the benchmark's octree (uniform depth 3: 585 slots), also read by the benchmark's CPU legs
    o = reflib.RefOctree(lib, 585)
    cases.tree_uniform(o, 3)
    put_state(out, "tree/uniform3", o.state())
    o.close()
    script = octree_script(2024, 400)
    o = reflib.RefOctree(lib, SLOTS)
    digests, finds = run_script(o, script)
    out["tree/script/ops"], out["tree/script/digests"], out["tree/script/finds"] = script, digests, finds
    put_state(out, "tree/script/final", o.state())
    o.close()
    # symmetric inverse
    m = (rng.standard_normal((6_000, 6)) * 0.2).astype(np.float32)
    m[:, [0, 3, 5]] += 1.0
    inv = np.zeros_like(m)
    lib.refh_sym_inverse(m.ctypes.data, len(m), inv.ctypes.data)
    out["inverse/in"], out["inverse/out"] = m, inv
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, "host_golden.npz")
    np.savez_compressed(path, **out)
    print(f"{len(out)} arrays -> {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
