"""The C ABI library loads without a GPU and exports exactly what include/amr_gb300.h declares.

No compute is launched here: argument validation happens before any CUDA call.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "amr_gb300.h")


def declared_functions() -> set[str]:
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(amr_[a-z0-9_]+)\s*\(", text))


def test_header_declarations_are_exported(am):
    lib = am.load()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_no_undeclared_exports(am):
    out = subprocess.run(["nm", "-D", "--defined-only", am.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line and line.split()[-1].startswith("amr_")}
    assert exported == declared_functions()


def test_python_bindings_cover_the_header(am):
    assert set(am.EXPORTS) == declared_functions()


def test_version_and_status_strings(am):
    lib = am.load()
    assert b"sm_103a" in lib.amr_version()
    for s in range(6):
        assert lib.amr_status_string(s)
    assert lib.amr_status_string(0) == b"ok"


@pytest.mark.parametrize("n,p,ok", [(16, 3, 1), (28, 2, 1), (32, 3, 1), (8, 2, 1), (16, 2, 0), (30, 3, 0)])
def test_config_supported(am, n, p, ok):
    assert am.load().amr_config_supported(ctypes.byref(am.Config(n, p, 100.0))) == ok


def test_config_rejects_bad_outer_size(am):
    assert am.load().amr_config_supported(ctypes.byref(am.Config(16, 3, 0.0))) == 0
    assert am.load().amr_config_supported(None) == 0


def test_invalid_arguments_fail_before_cuda(am):
    lib = am.load()
    cfg = am.Config(16, 3, 100.0)
    assert lib.amr_differentiate(ctypes.byref(cfg), None, None, None, None, 1, 0, 0, 0, None) == am.ERR_INVALID
    assert lib.amr_differentiate(ctypes.byref(am.Config(16, 2, 100.0)), 1, 1, None, 1, 1, 0, 0, 0, None) == am.ERR_UNSUPPORTED
    # max_depth beyond the 4-bit depth field of domain_boundary (AMR.h:9)
    assert lib.amr_mixed_partials(ctypes.byref(cfg), 1, 1, 1, 1, 0, 9, 0, None) == am.ERR_INVALID
    assert lib.amr_copy_to_child(ctypes.byref(cfg), 1, 8, 1, 0, None) == am.ERR_INVALID
    assert lib.amr_christoffel(ctypes.byref(cfg), None, None, 0, None, None, 1, 0, 0, 7, None) == am.ERR_INVALID
    assert lib.amr_criterion(ctypes.byref(cfg), None, 1, 1, 1, 1, 0, 0, None) == am.ERR_INVALID
    assert lib.amr_copy_new_to_old(ctypes.byref(cfg), None, 1, 1, 1, 1, 0, 0, None) == am.ERR_INVALID
    assert lib.amr_sim_create(ctypes.byref(cfg), 9, 4, 0, ctypes.byref(ctypes.c_void_p())) == am.ERR_INVALID
    assert lib.amr_sim_timestep(None) == am.ERR_INVALID
    assert lib.amr_cf3_encode(None, None, 4, None, None) == am.ERR_INVALID


def test_octree_entry_points_need_no_device(am):
    o = am.Octree(16)
    o.add_node(0, 3)
    s = o.state()
    assert s["used_slots"] == 2 and s["max_depth"] == 1
    assert s["positions"][1] == (1 << 27) | 3
    with pytest.raises(am.AmrError):
        o.add_node(99, 0)
    o.close()


def test_product_does_not_link_the_oracle(am):
    out = subprocess.run(["nm", "-D", am.LIB_PATH], capture_output=True, text=True, check=True).stdout
    assert "orc_" not in out and "refh_" not in out and "refd_" not in out
    deps = subprocess.run(["ldd", am.LIB_PATH], capture_output=True, text=True).stdout
    assert "liborc" not in deps and "libamr_ref" not in deps
    assert np.uint32  # numpy is importable for the tests
