"""Builds ``libpcrp.so`` (all CUDA/C++ sources in ``csrc/``) for sm_103a, in tree.

One nvcc invocation per translation unit, run in parallel, then one link; a
unit is rebuilt only when it or a header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # pcr-penta_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_PATH = os.path.join(PKG_ROOT, "libpcrp.so")
CMP_SRC = os.path.join(PKG_ROOT, "compare", "cusparse_gpsv.cpp")
CMP_LIB = os.path.join(PKG_ROOT, "compare", "libpcrp_cmp.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + INCLUDE, "-I" + CSRC]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    cmd = [NVCC] + ARCH + COMMON + (["-Xptxas", "-v"] if verbose and src.endswith(".cu") else []) + \
        ["-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        print(res.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile every source and link ``libpcrp.so``; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force:
        for o in glob.glob(os.path.join(BUILD_DIR, "*.o")):
            os.remove(o)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB_PATH] + objs + ["-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{res.stdout}\n{res.stderr}")
    build_compare()
    return LIB_PATH


def build_compare() -> str:
    """The cuSPARSE comparison library (benchmark only, not part of libpcrp)."""
    if not os.path.exists(CMP_LIB) or os.path.getmtime(CMP_LIB) < os.path.getmtime(CMP_SRC):
        cmd = [NVCC] + ARCH + ["-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", CMP_SRC,
                               "-o", CMP_LIB, "-lcusparse"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on the cuSPARSE comparison:\n{res.stdout}\n{res.stderr}")
    return CMP_LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
