"""ctypes wrapper of the C oracle (oracle/amr_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline / reference legs.  Build recipe: build() below (gcc, OpenMP).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborc.so")
SRC = [os.path.join(HERE, "amr_oracle.c"), os.path.join(HERE, "fp64_path.c"), os.path.join(HERE, "bssn_evolve.c"),
       os.path.join(HERE, "amr_oracle.h")]

FUSED_NOISE = 1
FTZ = 2
DEVICE_FLAGS = FTZ                 # the reference's device build, its standalone encoder (fast-math:
                                   # flush-to-zero; the noise product is rounded before the add, see
                                   # test_codec_noise_rounding)
STENCIL_FLAGS = FTZ | FUSED_NOISE  # the encodes inlined into its stencil and Christoffel kernels: the
                                   # noise product is fused into the add (pinned against the reference's
                                   # plugin on a GB300: tests/test_gpu_workload.py)
HOST_FLAGS = 0                     # the reference's host build (no contraction, no flush)

VP = ctypes.c_void_p
U32 = ctypes.c_uint32
I32 = ctypes.c_int32
I64 = ctypes.c_int64


class Evo(ctypes.Structure):
    """orc_evo: physics, gauge and initial data of the evolution oracle."""
    _fields_ = [("n", U32), ("p", U32), ("outer_size", ctypes.c_float), ("physics", ctypes.c_int),
                ("slicing", ctypes.c_int), ("shift", ctypes.c_int), ("eta", ctypes.c_float),
                ("ko_sigma", ctypes.c_float), ("cfl", ctypes.c_float), ("chi_floor", ctypes.c_float),
                ("id_kind", ctypes.c_int), ("amplitude", ctypes.c_float), ("wavelength", ctypes.c_float),
                ("n_punctures", ctypes.c_int), ("mass", ctypes.c_float * 4), ("pos", (ctypes.c_float * 3) * 4),
                ("width", ctypes.c_float)]


class Cfg(ctypes.Structure):
    _fields_ = [("n", U32), ("p", U32), ("outer_size", ctypes.c_float), ("inv_dx", ctypes.c_float * 9),
                ("outer_dt", ctypes.c_float), ("outer_dx", ctypes.c_float), ("flags", U32)]


_SIGS = {
    "orc_cfg_init": (None, [VP, U32, U32, ctypes.c_float, U32]),
    "orc_prng_int": (I32, [VP]),
    "orc_prng_float": (ctypes.c_float, [VP]),
    "orc_prng_ranged": (I32, [VP, I32, I32]),
    "orc_cf3_encode": (U32, [ctypes.c_float, ctypes.c_float, ctypes.c_float, VP, U32]),
    "orc_cf3_encode_seeded": (None, [VP, VP, I64, VP, U32]),
    "orc_cf3_encode_stream": (I32, [VP, I64, I32, VP, U32]),
    "orc_cf3_encode_det": (None, [VP, I64, VP, U32]),
    "orc_cf3_decode_n": (None, [VP, I64, VP]),
    "orc_sym_inverse": (None, [VP, VP]),
    "orc_sym_determinant": (ctypes.c_float, [VP]),
    "orc_trace_contra_sym": (ctypes.c_float, [VP, VP]),
    "orc_sym_times_vec": (None, [VP, VP, VP]),
    "orc_reverse_bits": (U32, [U32]),
    "orc_sum_coordinates": (U32, [U32, U32, ctypes.c_int]),
    "orc_diff_coordinates": (U32, [U32, U32, ctypes.c_int]),
    "orc_boundary": (ctypes.c_uint64, [U32, U32, I32]),
    "orc_differentiate": (None, [VP, VP, VP, VP, VP, U32, U32, U32, I32]),
    "orc_mixed_partials": (None, [VP, VP, VP, VP, U32, U32, U32, I32]),
    "orc_deriv_trace": (None, [VP, VP, VP, VP, VP, VP, U32, U32, U32]),
    "orc_christoffel": (None, [VP, VP, VP, I32, VP, VP, U32, U32, U32, ctypes.c_int]),
    "orc_copy_boundaries": (None, [VP, VP, VP, VP, U32, U32, U32, ctypes.c_int]),
    "orc_copy_new_to_old": (None, [VP, VP, VP, VP, VP, U32, U32, U32]),
    "orc_copy_to_child": (None, [VP, VP, U32, I32, I32]),
    "orc_wave_step": (None, [VP, ctypes.c_int, VP, VP, VP, VP, VP, U32, U32, U32]),
    "orc_criterion": (None, [VP, VP, VP, VP, VP, U32, U32, U32]),
    "orc_rasterise": (None, [VP, VP, VP, U32, U32, ctypes.c_float, ctypes.c_int, VP]),
    "orc_scan": (None, [ctypes.c_int, ctypes.c_int, VP, U32]),
    "orc_extreme": (None, [ctypes.c_int, ctypes.c_int, ctypes.c_int, VP, U32, VP]),
    "orc_differentiate_f64": (None, [VP, VP, VP, VP, VP, VP, U32]),
    "orc_bssn_timestep": (None, [VP, VP, VP, VP, VP, VP, VP, VP, VP, U32, U32, VP, VP, U32, U32]),
    "orc_bssn_timestep_f64": (None, [VP, VP, VP, VP, VP, VP, VP, VP, VP, U32, U32, VP]),
    "orc_evo_initial_data": (None, [VP, VP, VP, U32]),
    "orc_evo_timestep": (None, [VP, VP, VP, VP, VP, VP, VP, VP, U32, U32, VP]),
    "orc_evo_constraints": (None, [VP, VP, VP, VP, U32, ctypes.c_double, VP, VP]),
    "orc_periodic_boundaries": (None, [VP, VP, U32, VP]),
    "orc_num_threads": (ctypes.c_int, []),
    "orc_set_num_threads": (None, [ctypes.c_int]),
}

_lib = None


def build() -> str:
    """Compile oracle/_build/liborc.so if it is missing or older than its sources."""
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           "-o", LIB + ".tmp", *SRC[:-1], "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def P(a):
    """Argument for a pointer parameter: a numpy array's address (the caller keeps the array
    alive), or a ctypes pointer table from ptrs() passed through as is."""
    if isinstance(a, ctypes.Array):
        return a
    return a.ctypes.data


def ptrs(arrs) -> ctypes.Array:
    """A C table of the arrays' addresses.  Pass the returned object itself to the call so it
    stays alive until the call returns."""
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def cfg(n: int, p: int, outer_size: float = 100.0, flags: int = STENCIL_FLAGS, inv_dx=None) -> Cfg:
    c = Cfg()
    lib().orc_cfg_init(ctypes.byref(c), n, p, outer_size, flags)
    if inv_dx is not None:
        for i, v in enumerate(inv_dx):
            c.inv_dx[i] = float(v)
    return c


# ---------------------------------------------------------------- convenience wrappers (numpy in, numpy out)

def cf3_encode_seeded(xyz: np.ndarray, seeds: np.ndarray, flags: int = DEVICE_FLAGS) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, np.float32)
    seeds = np.ascontiguousarray(seeds, np.int32)
    out = np.zeros(len(seeds), np.uint32)
    lib().orc_cf3_encode_seeded(P(xyz), P(seeds), len(seeds), P(out), flags)
    return out


def cf3_encode_det(xyz: np.ndarray, flags: int = DEVICE_FLAGS) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, np.float32)
    out = np.zeros(len(xyz) // 3, np.uint32)
    lib().orc_cf3_encode_det(P(xyz), len(out), P(out), flags)
    return out


def cf3_decode(words: np.ndarray) -> np.ndarray:
    words = np.ascontiguousarray(words, np.uint32)
    out = np.zeros(len(words) * 3, np.float32)
    lib().orc_cf3_decode_n(P(words), len(words), P(out))
    return out


def prng_ints(seed: int, n: int) -> np.ndarray:
    s = ctypes.c_int32(seed)
    return np.array([lib().orc_prng_int(ctypes.byref(s)) for _ in range(n)], np.int32)
