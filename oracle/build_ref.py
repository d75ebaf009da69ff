"""Build recipe for the reference-build libraries under oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  The libraries built here wrap the reference's own code
(oracle/ref_harness.cu) and are loaded only by tests, the smoke check and the
benchmark's reference leg.

Two steps:
  stage()  -- when the reference checkout is present (this container), copy the
              reference headers the hot path needs into oracle/_ref/src/<cfg>/.
              Files are copied byte-for-byte except, for the non-native
              configurations, the two `constexpr` domain-size lines
              (AdaptiveMesh/AMR.h:11-12), which the reference documents as its
              compile-time configuration.  oracle/_ref/ is git-ignored.
  build()  -- compile oracle/_ref/libamr_ref_<cfg>.so from the staged headers with
              the reference's Release flags (--use_fast_math) for sm_103a.  This
              also works where the checkout is absent, as long as a previous
              stage() left the headers in oracle/_ref/src/.

The reference checkout's AdaptiveMesh/ folder is taken from the AMR_REFERENCE_DIR environment
variable, or from the `--ref DIR` argument when run as a script; its default is the checkout's
location in the build container, /root/reference/AdaptiveMesh.

Configurations: "n28p2" is the reference as shipped (size_domain 28, padding 2);
"n16p3" is size_domain 16 with padding 3 (the workload size of the benchmarks).
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF_ROOT = "/root/reference/AdaptiveMesh"
REF_ROOT = os.environ.get("AMR_REFERENCE_DIR", DEFAULT_REF_ROOT)
OUT = os.path.join(HERE, "_ref")
HEADERS = ["helper_math.h", "tensors.h", "AMR.h", "BSSN.h", "SimpleWave.h", "CUDA_memory.h", "image_process.h",
           "parallel.h"]
CONFIGS = {"n28p2": (28, 2), "n16p3": (16, 3)}
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")


def stage(ref_root: str | None = None) -> bool:
    """Copy reference headers into oracle/_ref/src/<cfg>; returns False if no checkout."""
    ref_root = ref_root or REF_ROOT
    if not os.path.isdir(ref_root):
        return False
    for cfg, (n, p) in CONFIGS.items():
        dst = os.path.join(OUT, "src", cfg)
        os.makedirs(dst, exist_ok=True)
        for h in HEADERS:
            src = os.path.join(ref_root, h)
            with open(src, "rb") as f:
                data = f.read()
            if h == "AMR.h" and cfg != "n28p2":
                text = data.decode("latin-1")
                text, k1 = re.subn(r"(constexpr uint size_domain = )28u;", rf"\g<1>{n}u;", text)
                text, k2 = re.subn(r"(constexpr uint padding_domain = )2u;", rf"\g<1>{p}u;", text)
                if k1 != 1 or k2 != 1:
                    raise RuntimeError("AMR.h constants not found; reference layout changed")
                data = text.encode("latin-1")
            out = os.path.join(dst, h)
            if not os.path.exists(out) or open(out, "rb").read() != data:
                with open(out, "wb") as f:
                    f.write(data)
    return True


def _build_one(cfg: str) -> str:
    src_dir = os.path.join(OUT, "src", cfg)
    lib = os.path.join(OUT, f"libamr_ref_{cfg}.so")
    harness = os.path.join(HERE, "ref_harness.cu")
    shim = os.path.join(HERE, "ref_shim.h")
    deps = [harness, shim] + [os.path.join(src_dir, h) for h in HEADERS]
    if os.path.exists(lib) and all(os.path.getmtime(lib) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return lib
    cmd = [NVCC, "-std=c++17", "-O3", "--use_fast_math", "-w",
           "-gencode", "arch=compute_103a,code=sm_103a",
           "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
           "-cudart", "shared", "-shared", "-o", lib + ".tmp", harness, "-I", HERE, "-I", src_dir]
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


def build(configs=None, ref_root: str | None = None) -> list[str]:
    """Build every configuration whose staged headers exist; returns the library paths."""
    stage(ref_root)
    configs = configs or list(CONFIGS)
    todo = [c for c in configs if os.path.isdir(os.path.join(OUT, "src", c))]
    with ThreadPoolExecutor(max_workers=len(todo) or 1) as ex:
        return list(ex.map(_build_one, todo))


def lib_path(cfg: str) -> str:
    return os.path.join(OUT, f"libamr_ref_{cfg}.so")


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--ref", default=None, help="the reference checkout's AdaptiveMesh/ folder")
    ap.add_argument("configs", nargs="*", help=f"configurations to build (default: all of {list(CONFIGS)})")
    args = ap.parse_args()
    print("\n".join(build(args.configs or None, args.ref)))
