"""ctypes wrapper of oracle/refrun.c: the reference's own kernels on the GPU.

TEST INFRASTRUCTURE ONLY (golden-output generation and live parity tests).
Needs oracle/_ref/kernel_{nofma,fma}.ptx (oracle/build_ref.sh, built where
the reference sources exist) and oracle/_ref/librefrun.so (make -C oracle refrun).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "librefrun.so")
_lib = None

VARIANT_SMALL = 0            # pcr_penta                                   kernel.cu:32-154
VARIANT_GLOBAL_SHARED = 2    # global_cached_shared_tile_splitting + stage 2  kernel.cu:325-526, 665-791
VARIANT_GLOBAL_GLOBAL = 3    # global_cached_global_tile_splitting + stage 2  kernel.cu:530-659, 665-791


def ptx_path(fma: bool) -> str:
    return os.path.join(REF_DIR, "kernel_fma.ptx" if fma else "kernel_nofma.ptx")


def available() -> bool:
    return os.path.exists(ptx_path(False)) and os.path.exists(ptx_path(True))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(["make", "-s", "-C", HERE, "refrun"], check=True)
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        L.refrun_solve.argtypes = [ctypes.c_char_p, ctypes.c_int] + [dp] * 7 + [ctypes.c_int, ctypes.c_int]
        L.refrun_solve.restype = ctypes.c_int
        L.refrun_time.argtypes = [ctypes.c_char_p, ctypes.c_int] + [dp] * 7 + [ctypes.c_int, ctypes.c_int,
                                                                               ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
        L.refrun_time.restype = ctypes.c_int
        L.refrun_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def solve(arrs, m: int, n: int, variant: int, fma: bool = False) -> np.ndarray:
    """Run the reference kernels on (a,b,c,d,e,y) (contiguous host arrays); return x."""
    L = lib()
    dp = ctypes.POINTER(ctypes.c_double)
    ins = [np.ascontiguousarray(v, dtype=np.float64) for v in arrs]
    x = np.zeros(m * n, dtype=np.float64)
    rc = L.refrun_solve(ptx_path(fma).encode(), variant, *[v.ctypes.data_as(dp) for v in ins],
                        x.ctypes.data_as(dp), m, n)
    if rc != 0:
        raise RuntimeError(f"refrun_solve rc={rc}: {L.refrun_last_error().decode()}")
    return x


def time_solve(arrs, m: int, n: int, variant: int, fma: bool = False, reps: int = 3):
    """Run the reference kernels once (returning x) and time `reps` more solves
    on the GPU (CUDA events around the launches, inputs restored before each):
    (x, mean milliseconds per solve)."""
    L = lib()
    dp = ctypes.POINTER(ctypes.c_double)
    ins = [np.ascontiguousarray(v, dtype=np.float64) for v in arrs]
    x = np.zeros(m * n, dtype=np.float64)
    ms = ctypes.c_float(0.0)
    rc = L.refrun_time(ptx_path(fma).encode(), variant, *[v.ctypes.data_as(dp) for v in ins],
                       x.ctypes.data_as(dp), m, n, reps, ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError(f"refrun_time rc={rc}: {L.refrun_last_error().decode()}")
    return x, float(ms.value)
