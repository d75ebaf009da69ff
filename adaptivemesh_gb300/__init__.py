"""adaptivemesh_gb300 -- GB300 (sm_103a) implementation of AdaptiveMesh's per-timestep hot path.

The compute path is the C-ABI library libamr_gb300.so (include/amr_gb300.h): hand-written CUDA
kernels plus the C++ host octree and the reference's two plugins.  This module loads it with
ctypes and mirrors the reference's interfaces for Python callers (tests, benchmarks):

  Octree  -- AMR<T>'s host octree (AdaptiveMesh/AMR.h:118-294)
  Sim     -- a plugin (BSSN_AMR_data, BSSN.h:104-171, or wave_AMR_data, SimpleWave.h:191-279)
             with its timestep loop (AMR.h:324-333)
  ops     -- one function per reference operator (AMR.h:880-1310, BSSN.h:24-102,
             SimpleWave.h:48-150) on caller-owned device buffers

There is no CPU fallback: if the library is missing or fails to load, import-time use raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB

OK = 0
ERR_INVALID, ERR_UNSUPPORTED, ERR_CUDA, ERR_NO_DEVICE, ERR_CAPACITY, ERR_TIMEOUT = 1, 2, 3, 4, 5, 6
SIM_BSSN, SIM_WAVE, SIM_BSSN_EVOLVE, SIM_WAVE_RK4 = 1, 2, 3, 4
SLICING_1PLUSLOG, SLICING_HARMONIC = 0, 1
ID_FLAT, ID_GAUGE_WAVE, ID_BRILL_LINDQUIST, ID_GAUSSIAN_PULSE = 0, 1, 2, 3
# BSSN evolution fields (amr_sim_buffer components)
F_CHI, F_GXX, F_K, F_AXX, F_GAMX, F_ALPHA, F_BETAX, F_BX = 0, 1, 7, 8, 14, 17, 18, 21
# the BSSN evolution stores these fields less 1 (chi, gt_xx, gt_yy, gt_zz, alpha)
BSSN_OFFSETS = tuple(1.0 if f in (0, 1, 4, 6, 17) else 0.0 for f in range(24))
DTYPE_UINT32, DTYPE_INT32, DTYPE_FLOAT32 = 0, 1, 2
MODE_PLAIN, MODE_BATCHED, MODE_GRAPH = 0, 1, 2
# the plugin interface's phases, in the order of the reference's timestep loop (AMR.h:324-333)
PHASE_COPY_BACK, PHASE_MODIFY_NODES, PHASE_PREDICTOR, PHASE_COPY_BOUNDS, PHASE_CORRECTOR, PHASE_INCREMENT_TIMER = range(6)
CHRISTOFFEL_REFERENCE, CHRISTOFFEL_RAISED = 0, 1

VP = ctypes.c_void_p
U32, I32, U64 = ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64


class Config(ctypes.Structure):
    """amr_config: the reference's domain constants (AMR.h:9-20) as run-time values."""
    _fields_ = [("size_domain", U32), ("padding_domain", U32), ("outer_size", ctypes.c_float)]

    def __init__(self, size_domain: int = 28, padding_domain: int = 2, outer_size: float = 100.0):
        super().__init__(size_domain, padding_domain, outer_size)

    @property
    def total(self) -> int:
        return self.size_domain + 2 * self.padding_domain

    @property
    def padded_cells(self) -> int:
        return self.total ** 3

    @property
    def inner_cells(self) -> int:
        return self.size_domain ** 3


CP = ctypes.POINTER(Config)


class Evolution(ctypes.Structure):
    """amr_evolution: physics and gauge of an evolution simulation."""
    _fields_ = [("slicing", ctypes.c_int), ("shift", ctypes.c_int), ("eta", ctypes.c_float),
                ("ko_sigma", ctypes.c_float), ("cfl", ctypes.c_float), ("periodic", ctypes.c_int)]

    def __init__(self, slicing=0, shift=0, eta=2.0, ko_sigma=0.1, cfl=0.25, periodic=0):
        super().__init__(slicing, shift, eta, ko_sigma, cfl, periodic)


class Regrid(ctypes.Structure):
    """amr_regrid: thresholds of the refinement decision (plain criterion and learned estimator)."""
    _fields_ = [("refine_threshold", ctypes.c_float), ("coarsen_threshold", ctypes.c_float),
                ("learned_refine", ctypes.c_float), ("learned_coarsen", ctypes.c_float),
                ("judge_factor", ctypes.c_float), ("max_depth", U32), ("min_depth", U32)]

    def __init__(self, refine_threshold=0.02, coarsen_threshold=0.005, learned_refine=-5.0, learned_coarsen=-6.5,
                 judge_factor=4.0, max_depth=6, min_depth=1):
        super().__init__(refine_threshold, coarsen_threshold, learned_refine, learned_coarsen, judge_factor,
                         max_depth, min_depth)


class InitialData(ctypes.Structure):
    """amr_initial_data: analytic initial data of an evolution simulation."""
    _fields_ = [("kind", ctypes.c_int), ("amplitude", ctypes.c_float), ("wavelength", ctypes.c_float),
                ("n_punctures", ctypes.c_int), ("mass", ctypes.c_float * 4), ("position", (ctypes.c_float * 3) * 4),
                ("width", ctypes.c_float)]

    def __init__(self, kind=0, amplitude=0.0, wavelength=1.0, punctures=(), width=0.1):
        super().__init__()
        self.kind, self.amplitude, self.wavelength, self.width = kind, amplitude, wavelength, width
        self.n_punctures = len(punctures)
        for i, (m, pos) in enumerate(punctures):
            self.mass[i] = m
            for k in range(3):
                self.position[i][k] = pos[k]

EXPORTS = {
    "amr_version": (ctypes.c_char_p, []),
    "amr_config_supported": (ctypes.c_int, [CP]),
    "amr_last_cuda_error": (ctypes.c_int, []),
    "amr_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "amr_device_status": (ctypes.c_int, [VP]),
    "amr_cf3_encode": (ctypes.c_int, [VP, VP, U64, VP, VP]),
    "amr_cf3_decode": (ctypes.c_int, [VP, U64, VP, VP]),
    "amr_differentiate": (ctypes.c_int, [CP, VP, VP, VP, VP, U32, U32, U32, I32, VP]),
    "amr_mixed_partials": (ctypes.c_int, [CP, VP, VP, VP, U32, U32, U32, I32, VP]),
    "amr_deriv_trace": (ctypes.c_int, [CP, VP, VP, VP, VP, VP, U32, U32, U32, VP]),
    "amr_christoffel": (ctypes.c_int, [CP, VP, VP, I32, VP, VP, U32, U32, U32, ctypes.c_int, VP]),
    "amr_copy_boundaries": (ctypes.c_int, [CP, VP, VP, VP, U32, U32, U32, ctypes.c_int, VP]),
    "amr_copy_boundaries_noalloc": (ctypes.c_int, [CP, VP, VP, VP, U32, U32, U32, ctypes.c_int, VP]),
    "amr_rasterise": (ctypes.c_int, [CP, VP, VP, U32, U32, U32, ctypes.c_float, ctypes.c_int, VP, VP]),
    "amr_partition_morton": (ctypes.c_int, [VP, U32, U32, VP]),
    "amr_ghost_exchange_plan": (ctypes.c_int, [CP, VP, VP, U32, U32, U32, U32, VP, U32, VP]),
    "amr_restriction_exchange_plan": (ctypes.c_int, [CP, VP, VP, VP, U32, U32, U32, U32, VP, U32, VP]),
    "amr_pack_boxes": (ctypes.c_int, [CP, VP, U32, VP, VP, U32, VP, VP]),
    "amr_unpack_boxes": (ctypes.c_int, [CP, VP, U32, VP, VP, U32, VP, VP]),
    "amr_copy_new_to_old": (ctypes.c_int, [CP, VP, VP, VP, VP, U32, U32, U32, VP]),
    "amr_copy_to_child": (ctypes.c_int, [CP, VP, U32, I32, I32, VP]),
    "amr_wave_predictor": (ctypes.c_int, [CP, VP, VP, VP, VP, VP, U32, U32, U32, VP]),
    "amr_wave_corrector": (ctypes.c_int, [CP, VP, VP, VP, VP, VP, U32, U32, U32, VP]),
    "amr_criterion": (ctypes.c_int, [CP, VP, VP, VP, VP, U32, U32, U32, VP]),
    "amr_octree_create": (ctypes.c_int, [U32, ctypes.POINTER(VP)]),
    "amr_octree_destroy": (ctypes.c_int, [VP]),
    "amr_octree_add_node": (ctypes.c_int, [VP, I32, I32]),
    "amr_octree_remove_node": (ctypes.c_int, [VP, I32]),
    "amr_octree_add_nodes": (ctypes.c_int, [VP, VP, VP, U32]),
    "amr_octree_remove_nodes": (ctypes.c_int, [VP, VP, U32]),
    "amr_octree_increment_timer": (ctypes.c_int, [VP]),
    "amr_octree_find_node_idx": (U32, [VP, U32, U32]),
    "amr_octree_state": (ctypes.c_int, [VP, VP, VP, VP, VP, VP, VP]),
    "amr_sim_create": (ctypes.c_int, [CP, ctypes.c_int, U32, ctypes.c_int, ctypes.POINTER(VP)]),
    "amr_sim_destroy": (ctypes.c_int, [VP]),
    "amr_sim_set_mode": (ctypes.c_int, [VP, ctypes.c_int]),
    "amr_sim_add_node": (ctypes.c_int, [VP, I32, I32]),
    "amr_sim_remove_node": (ctypes.c_int, [VP, I32]),
    "amr_sim_add_nodes": (ctypes.c_int, [VP, VP, VP, U32]),
    "amr_sim_remove_nodes": (ctypes.c_int, [VP, VP, U32]),
    "amr_sim_octree_state": (ctypes.c_int, [VP, VP, VP, VP, VP, VP, VP]),
    "amr_sim_buffer": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(VP), ctypes.POINTER(U64)]),
    "amr_sim_copy_to_device": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int, VP, U64]),
    "amr_sim_copy_to_host": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int, VP, U64]),
    "amr_sim_copy_to_host_side": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int, VP, U64]),
    "amr_sim_stage_to_device": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int, VP, U64]),
    "amr_sim_snapshot_to_host": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int, VP, U64]),
    "amr_sim_stage_many": (ctypes.c_int, [VP, U32, VP, VP, VP, VP]),
    "amr_sim_snapshot_many": (ctypes.c_int, [VP, U32, VP, VP, VP, VP]),
    "amr_sim_event_record": (ctypes.c_int, [VP, ctypes.c_int]),
    "amr_sim_event_elapsed": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "amr_sim_save": (ctypes.c_int, [VP, ctypes.c_char_p]),
    "amr_sim_load": (ctypes.c_int, [VP, ctypes.c_char_p]),
    "amr_sim_timestep": (ctypes.c_int, [VP]),
    "amr_sim_copy_bounds": (ctypes.c_int, [VP]),
    "amr_sim_phase": (ctypes.c_int, [VP, I32]),
    "amr_sim_set_octree": (ctypes.c_int, [VP, VP, VP, VP, VP, VP, VP]),
    "amr_sim_rng": (ctypes.c_int, [VP, ctypes.POINTER(I32)]),
    "amr_sim_set_rng": (ctypes.c_int, [VP, I32]),
    "amr_sim_stream": (ctypes.c_int, [VP, ctypes.POINTER(VP)]),
    "amr_sim_set_stream": (ctypes.c_int, [VP, VP]),
    "amr_sim_synchronize": (ctypes.c_int, [VP]),
    "amr_sim_kernel_launches": (U64, [VP]),
    "amr_sim_set_stencil_ctas": (ctypes.c_int, [VP, U32]),
    "amr_sim_autotune": (ctypes.c_int, [VP, U32, VP]),
    "amr_sim_tuned_shapes": (ctypes.c_int, [VP, U32, VP, VP, VP]),
    "amr_sim_set_fault_injection": (ctypes.c_int, [VP, U32, U32]),
    "amr_sim_set_evolution": (ctypes.c_int, [VP, VP]),
    "amr_sim_initial_data": (ctypes.c_int, [VP, VP]),
    "amr_sim_constraint_norms": (ctypes.c_int, [VP, ctypes.c_float, VP]),
    "amr_octree_set_periodic": (ctypes.c_int, [VP, ctypes.c_int]),
    "amr_estimator_create": (ctypes.c_int, [U32, U64, ctypes.POINTER(VP)]),
    "amr_estimator_destroy": (ctypes.c_int, [VP]),
    "amr_estimator_param_count": (U64, []),
    "amr_estimator_get_params": (ctypes.c_int, [VP, VP]),
    "amr_estimator_set_params": (ctypes.c_int, [VP, VP]),
    "amr_estimator_forward": (ctypes.c_int, [VP, VP, U32, VP]),
    "amr_estimator_gradients": (ctypes.c_int, [VP, VP, VP, U32, VP, ctypes.POINTER(ctypes.c_float)]),
    "amr_estimator_train_step": (ctypes.c_int, [VP, VP, VP, U32, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]),
    "amr_sim_tile_features": (ctypes.c_int, [VP, VP, VP, VP, U32, ctypes.POINTER(U32)]),
    "amr_sim_regrid": (ctypes.c_int, [VP, VP, VP, VP]),
    "amr_sim_enable_kernel_timing": (ctypes.c_int, [VP, ctypes.c_int]),
    "amr_sim_kernel_timing": (ctypes.c_int, [VP, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(U64)]),
    "amr_inclusive_scan": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, VP, U64, VP]),
    "amr_reduce_max": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, VP, U64, VP, VP]),
    "amr_reduce_min": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, VP, U64, VP, VP]),
    "amr_field_norms": (ctypes.c_int, [CP, VP, VP, VP, U32, VP, VP]),
}

_LIB = None


class AmrError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        lib = _LIB
        msg = lib.amr_status_string(status).decode() if lib else str(status)
        cuda = lib.amr_last_cuda_error() if lib else 0
        super().__init__(f"{what}: {msg} (status {status}, last CUDA error {cuda})")
        self.status = status


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libamr_gb300.so (compiling it first if it is absent and nvcc is available)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH) and build_if_missing:
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run adaptivemesh_gb300.build.build()")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise AmrError(status, what)


def _p(t) -> int:
    """Address of a torch tensor / numpy array / int / None."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def _ptr_array(ts) -> ctypes.Array:
    arr = (VP * len(ts))()
    for i, t in enumerate(ts):
        arr[i] = _p(t)
    return arr


from . import ops  # noqa: E402
from .octree import Octree, Sim  # noqa: E402
from .estimator import Estimator  # noqa: E402

__all__ = ["Config", "Evolution", "InitialData", "Regrid", "Octree", "Sim", "Estimator", "ops", "load", "check",
           "AmrError", "LIB_PATH", "EXPORTS"]
