"""ctypes wrapper around the CPU oracle (``oracle/pcrp_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline / reference leg of ``bench.py``; never by the product.

* :func:`pcr` -- the restatement of the reference's PCR-Penta algorithm
  (PCR-Penta kernel.cu:32-154, stride count from main.cu:38-39).
* :func:`ge`  -- FP64 pentadiagonal Gaussian elimination (ground truth for
  diagonally dominant systems; no counterpart in the reference).
* :func:`residual` -- r = y - A x with long-double accumulation.
* :func:`generate` -- the seeded benchmark inputs (same values as the
  library's generator, checked bit for bit in tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)

CONTIGUOUS = 0
INTERLEAVED = 1


def build(force: bool = False) -> str:
    """Compile ``liboracle.so`` with the Makefile beside this file."""
    src = os.path.join(_HERE, "pcrp_oracle.c")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        six = [_dp] * 6
        L.oracle_ref_strides.argtypes = [ctypes.c_int64]
        L.oracle_ref_strides.restype = ctypes.c_int
        for name in ("oracle_pcr_batch", "oracle_ge_batch"):
            f = getattr(L, name)
            f.argtypes = six + [_dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
            f.restype = ctypes.c_int
        L.oracle_ragged_batch.argtypes = six + [_dp, _i64p, _i64p, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
        L.oracle_ragged_batch.restype = ctypes.c_int
        L.oracle_residual_batch.argtypes = six + [_dp, _dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
        L.oracle_residual_batch.restype = ctypes.c_int
        L.oracle_generate.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_int] + six + [ctypes.c_int]
        L.oracle_generate.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(x: np.ndarray):
    assert x.dtype == np.float64 and x.flags.c_contiguous
    return x.ctypes.data_as(_dp)


def ref_strides(n: int) -> int:
    """Strides the reference runs for a system of n rows."""
    return int(lib().oracle_ref_strides(n))


def _bands(a, b, c, d, e, y):
    return [np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c, d, e, y)]


def pcr(a, b, c, d, e, y, m: int, n: int, layout: int = CONTIGUOUS, threads: int = 0) -> np.ndarray:
    """Reference PCR-Penta algorithm on a batch; returns x (same layout as y)."""
    arrs = _bands(a, b, c, d, e, y)
    x = np.zeros(m * n, dtype=np.float64)
    rc = lib().oracle_pcr_batch(*[_ptr(v) for v in arrs], _ptr(x), m, n, layout, threads)
    if rc:
        raise MemoryError("oracle_pcr_batch failed")
    return x


def ge(a, b, c, d, e, y, m: int, n: int, layout: int = CONTIGUOUS, threads: int = 0) -> np.ndarray:
    """Banded Gaussian elimination (no pivoting) on a batch; returns x."""
    arrs = _bands(a, b, c, d, e, y)
    x = np.zeros(m * n, dtype=np.float64)
    rc = lib().oracle_ge_batch(*[_ptr(v) for v in arrs], _ptr(x), m, n, layout, threads)
    if rc:
        raise MemoryError("oracle_ge_batch failed")
    return x


def ragged(a, b, c, d, e, y, offsets, sizes, kind: str = "ge", threads: int = 0) -> np.ndarray:
    """Ragged batch (systems contiguous at ``offsets``); kind 'pcr' or 'ge'."""
    arrs = _bands(a, b, c, d, e, y)
    offs = np.ascontiguousarray(offsets, dtype=np.int64)
    szs = np.ascontiguousarray(sizes, dtype=np.int64)
    x = np.zeros_like(arrs[5])
    rc = lib().oracle_ragged_batch(*[_ptr(v) for v in arrs], _ptr(x),
                                   offs.ctypes.data_as(_i64p), szs.ctypes.data_as(_i64p),
                                   len(szs), 0 if kind == "pcr" else 1, threads)
    if rc:
        raise MemoryError("oracle_ragged_batch failed")
    return x


def residual(a, b, c, d, e, y, x, m: int, n: int, layout: int = CONTIGUOUS) -> np.ndarray:
    """r = y - A x (long-double accumulation)."""
    arrs = _bands(a, b, c, d, e, y)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    r = np.zeros(m * n, dtype=np.float64)
    lib().oracle_residual_batch(*[_ptr(v) for v in arrs], _ptr(xx), _ptr(r), m, n, layout)
    return r


def generate(kind: int, seed: int, m: int, n: int, layout: int = CONTIGUOUS, threads: int = 0):
    """The seeded benchmark inputs (a, b, c, d, e, y), restated in C beside the
    solvers so that CPU-only runs need not load the product library."""
    arrs = [np.zeros(m * n, dtype=np.float64) for _ in range(6)]
    rc = lib().oracle_generate(kind, seed & 0xFFFFFFFFFFFFFFFF, m, n, layout, *[_ptr(v) for v in arrs],
                                threads)
    if rc:
        raise ValueError(f"oracle_generate: bad arguments (kind={kind}, m={m}, n={n})")
    return arrs


def fwd_err(x, xref, m: int, n: int, layout: int = CONTIGUOUS) -> float:
    """max over systems of ||x - xref||_inf / ||xref||_inf."""
    X = np.asarray(x, dtype=np.float64)
    R = np.asarray(xref, dtype=np.float64)
    if layout == CONTIGUOUS:
        X = X.reshape(m, n); R = R.reshape(m, n)
    else:
        X = X.reshape(n, m).T; R = R.reshape(n, m).T
    num = np.abs(X - R).max(axis=1)
    den = np.abs(R).max(axis=1)
    den = np.where(den == 0, 1.0, den)
    return float((num / den).max()) if m else 0.0
