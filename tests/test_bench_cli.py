"""The benchmark script's command line and its CPU arm (no GPU needed).

The GPU arm runs only where a GPU is visible; here the script must at least compile, and `--impl reference`
(the oracle's restatement of the timestep on the host cores) must print one JSON line with the
benchmark contract's keys.
"""
from __future__ import annotations

import json
import os
import py_compile
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_scripts_compile():
    for name in ("bench.py", "__graft_entry__.py"):
        py_compile.compile(os.path.join(ROOT, name), doraise=True)


def test_reference_arm_prints_one_contract_line():
    """Whole timesteps of the reference path on the host cores (the depth-2 tree keeps it short); the
    line carries the contract's keys and the same config dict as the GPU arm would print."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--depth", "2"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 1
    assert d["config"]["leaf_domains"] == 64 and d["config"]["zones_per_domain"] == 16 ** 3
    assert "64 leaf + 9 parent domains of 16^3, padding 3" in d["config"]["workload"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.config_dict(2, 1)
