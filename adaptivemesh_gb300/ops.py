"""Operator-level entry points on caller-owned device buffers (torch tensors or raw addresses).

Each function forwards to the C ABI entry point of the same name (include/amr_gb300.h) and
raises AmrError on a non-zero status.  Argument order and meaning follow the reference's
operator wrappers, cited per function.
"""
from __future__ import annotations

import ctypes

from . import Config, _p, _ptr_array, check, load


def _s(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream   # torch.cuda.Stream


def cf3_encode(xyz, out, seeds=None, stream=None) -> None:
    """compressed_float3 encode of n triples (tensors.h:350-393); seeds=None: deterministic."""
    n = out.numel()
    check(load().amr_cf3_encode(_p(xyz), _p(seeds), n, _p(out), _s(stream)), "amr_cf3_encode")


def cf3_decode(words, xyz, stream=None) -> None:
    """compressed_float3 decode (tensors.h:335-348)."""
    check(load().amr_cf3_decode(_p(words), words.numel(), _p(xyz), _s(stream)), "amr_cf3_decode")


def differentiate(cfg: Config, field, dif, d2if, positions, used: int, substep: int, max_depth: int, seed: int,
                  stream=None) -> None:
    """differentiate() (AMR.h:1280-1302)."""
    check(load().amr_differentiate(ctypes.byref(cfg), _p(field), _p(dif), _p(d2if), _p(positions), used, substep,
                                   max_depth, seed, _s(stream)), "amr_differentiate")


def mixed_partials(cfg: Config, field, off, positions, used: int, substep: int, max_depth: int, seed: int,
                   stream=None) -> None:
    """mixed_partials() (AMR.h:1268-1278)."""
    check(load().amr_mixed_partials(ctypes.byref(cfg), _p(field), _p(off), _p(positions), used, substep, max_depth,
                                    seed, _s(stream)), "amr_mixed_partials")


def deriv_trace(cfg: Config, hess_diag, hess_off, metric6, out, positions, used: int, substep: int, max_depth: int,
                stream=None) -> None:
    """__deriv_trace launch of scalar_laplacian_noncovariant (BSSN.h:31-35)."""
    check(load().amr_deriv_trace(ctypes.byref(cfg), _p(hess_diag), _p(hess_off), _ptr_array(metric6), _p(out),
                                 _p(positions), used, substep, max_depth, _s(stream)), "amr_deriv_trace")


def christoffel(cfg: Config, metric6, derivs6, seed: int, out6, positions, used: int, substep: int, max_depth: int,
                mode: int = 0, stream=None) -> None:
    """compute_raised_christoffel_symbols() (BSSN.h:93-102)."""
    check(load().amr_christoffel(ctypes.byref(cfg), _ptr_array(metric6), _ptr_array(derivs6), seed, _ptr_array(out6),
                                 _p(positions), used, substep, max_depth, mode, _s(stream)), "amr_christoffel")


def copy_boundaries(cfg: Config, old, new, boundaries, used: int, substep: int, max_depth: int,
                    copy_only_new: bool = True, stream=None) -> None:
    """copy_boundaries() (AMR.h:880-900)."""
    check(load().amr_copy_boundaries(ctypes.byref(cfg), _p(old), _p(new), _p(boundaries), used, substep, max_depth,
                                     1 if copy_only_new else 0, _s(stream)), "amr_copy_boundaries")


def copy_new_to_old(cfg: Config, old, new, positions, children, used: int, substep: int, max_depth: int,
                    stream=None) -> None:
    """copy_new_to_old() (AMR.h:998-1018)."""
    check(load().amr_copy_new_to_old(ctypes.byref(cfg), _p(old), _p(new), _p(positions), _p(children), used, substep,
                                     max_depth, _s(stream)), "amr_copy_new_to_old")


def copy_to_child(cfg: Config, field, offset: int, child: int, parent: int, stream=None) -> None:
    """copy_to_child() (AMR.h:1075-1082)."""
    check(load().amr_copy_to_child(ctypes.byref(cfg), _p(field), offset, child, parent, _s(stream)), "amr_copy_to_child")


def wave_step(cfg: Config, corrector: bool, old, derivs, hess, new, positions, used: int, substep: int,
              max_depth: int, stream=None) -> None:
    """wave_equation_predictor() / wave_equation_corrector() (SimpleWave.h:48-72)."""
    fn = load().amr_wave_corrector if corrector else load().amr_wave_predictor
    check(fn(ctypes.byref(cfg), _p(old), _p(derivs), _p(hess), _p(new), _p(positions), used, substep, max_depth,
             _s(stream)), "amr_wave_step")


def criterion(cfg: Config, derivs, hess, crit, positions, used: int, substep: int, max_depth: int, stream=None) -> None:
    """The device half of amr_criterion() (SimpleWave.h:142-150)."""
    check(load().amr_criterion(ctypes.byref(cfg), _p(derivs), _p(hess), _p(crit), _p(positions), used, substep,
                               max_depth, _s(stream)), "amr_criterion")


def rasterise(cfg: Config, field, children, used: int, width: int, height: int, raster, z_slice: float = 1e-9,
              bounding_boxes: bool = True, stream=None) -> None:
    """Slice image of a padded field (rasterise_to_image, AdaptiveMesh/AMR.h:1313-1365): `raster`
    holds width * height RGBA floats; the reference's default slice is z = 1e-9 and its build draws
    the leaves' bounding boxes (AMR.h:1312)."""
    check(load().amr_rasterise(ctypes.byref(cfg), _p(field), _p(children), used, width, height, z_slice,
                               1 if bounding_boxes else 0, _p(raster), _s(stream)))



def _dtype_of(t) -> int:
    import torch
    from . import DTYPE_FLOAT32, DTYPE_INT32, DTYPE_UINT32
    return {torch.float32: DTYPE_FLOAT32, torch.int32: DTYPE_INT32, torch.uint32: DTYPE_UINT32}[t.dtype]


def inclusive_scan(data, ncomp: int = 1, stream=None) -> None:
    """In-place inclusive cumulative sum (apply_incl_cum_sum, AdaptiveMesh/parallel.h:62-82) of a
    contiguous CUDA tensor of elements of `ncomp` values (float32, int32 or uint32)."""
    check(load().amr_inclusive_scan(_dtype_of(data), ncomp, _p(data), data.numel() // ncomp, _s(stream)),
          "amr_inclusive_scan")


def reduce_max(data, ncomp: int = 1, stream=None):
    """Component-wise maximum (find_maximum_val, AdaptiveMesh/parallel.h:239-251); the tensor is
    used as scratch as by the reference.  Returns a list of `ncomp` values."""
    return _extreme(load().amr_reduce_max, "amr_reduce_max", data, ncomp, stream)


def reduce_min(data, ncomp: int = 1, stream=None):
    """Component-wise minimum (find_minimum_val, AdaptiveMesh/parallel.h:409-421), with the
    reference's treatment of a partial last block (its missing elements count as 0)."""
    return _extreme(load().amr_reduce_min, "amr_reduce_min", data, ncomp, stream)


def _extreme(fn, name, data, ncomp, stream):
    import numpy as np
    import torch
    out = np.zeros(ncomp, {torch.float32: np.float32, torch.int32: np.int32, torch.uint32: np.uint32}[data.dtype])
    check(fn(_dtype_of(data), ncomp, _p(data), data.numel() // ncomp, out.ctypes.data, _s(stream)), name)
    return out.tolist()


def field_norms(cfg: Config, field, positions, children, used: int, stream=None) -> dict:
    """FP64 sum, sum of squares, largest magnitude and cell count of a padded field over the leaf
    domains' interior cells (amr_field_norms)."""
    import numpy as np
    out = np.zeros(4, np.float64)
    check(load().amr_field_norms(ctypes.byref(cfg), _p(field), _p(positions), _p(children), used, out.ctypes.data,
                                 _s(stream)), "amr_field_norms")
    return {"sum": float(out[0]), "sum_sq": float(out[1]), "max_abs": float(out[2]), "cells": int(out[3])}
