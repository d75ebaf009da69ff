"""Generate codec_fused_probe_inputs.npz: codec inputs that tell apart the two ways of adding the
stochastic-rounding noise.

compressed_float3's encoder adds `prng.generate_float() * .95f` to each scaled component before
truncating (AdaptiveMesh/tensors.h:350-372, the stochastic constructor).  Whether that product is
rounded before the add or fused into it changes the word only when the scaled value sits within an
ulp of a rounding boundary.  This script builds triples whose first component lands there (the
other two pin the shared exponent at 15), keeps those on which the oracle's two variants
(FTZ vs FTZ|FUSED_NOISE) disagree, and stores the first 4000 inputs with their seeds.  The device
tests run them through the reference's kernel and through this library's: both must give the
unfused words.

usage: python tests/golden/gen_codec_probe.py   (writes tests/golden/codec_fused_probe_inputs.npz)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as orc  # noqa: E402


def first_draw(seeds: np.ndarray) -> np.ndarray:
    """fast_prng's first generate_float() for each seed, vectorised (the scalar form is
    orc_prng_float; AdaptiveMesh/tensors.h:292-297)."""
    v = (seeds.view(np.uint32).astype(np.uint64) + 1124781675) & 0xFFFFFFFF
    v = v ^ (v.astype(np.uint32).view(np.int32) >> 7).view(np.uint32).astype(np.uint64)
    v = (v * 1246477263) & 0xFFFFFFFF
    return v.astype(np.uint32).view(np.int32).astype(np.float32) * np.float32(2.3283064e-10)


def main(out: str = os.path.join(HERE, "codec_fused_probe_inputs.npz")):
    rng = np.random.default_rng(5)
    seeds = rng.integers(-2 ** 31, 2 ** 31, 200_000, dtype=np.int64).astype(np.int32)
    noise = (first_draw(seeds) * np.float32(0.95)).astype(np.float32)
    k = rng.integers(0, 250, len(seeds)).astype(np.float32)
    boundary = (k + np.float32(0.5) - noise).astype(np.float32)          # scaled value at a rounding edge
    cands = [(boundary.view(np.uint32).astype(np.int64) + d).astype(np.uint32).view(np.float32) for d in range(-3, 4)]
    x = np.concatenate(cands)
    s = np.tile(seeds, 7)
    a = (x / np.float32(128)).astype(np.float32)                          # exponent 15 scales by 2^7
    xyz = np.stack([a, np.full_like(a, 1.5), np.full_like(a, -1.25)], 1).reshape(-1)
    unfused = orc.cf3_encode_seeded(xyz, s, orc.FTZ)
    fused = orc.cf3_encode_seeded(xyz, s, orc.FTZ | orc.FUSED_NOISE)
    sel = np.nonzero(unfused != fused)[0][:4000]
    np.savez(out, xyz=xyz.reshape(-1, 3)[sel].reshape(-1), seeds=s[sel])
    print(f"{len(sel)} inputs -> {out}")


if __name__ == "__main__":
    orc.build()
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "codec_fused_probe_inputs.npz"))
