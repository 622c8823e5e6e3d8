"""cuSPARSE gpsvInterleavedBatch as a timed comparison point (library call).

Used by ``bench.py --cusparse`` and its GPU test; not part of the solver.
The arrays use the interleaved layout (i*m + j); gpsv overwrites the bands.
"""
from __future__ import annotations

import ctypes

from .build import CMP_LIB, build_compare

_lib = None


def lib():
    global _lib
    if _lib is None:
        build_compare()
        L = ctypes.CDLL(CMP_LIB)
        vp = ctypes.c_void_p
        L.cmp_gpsv_buffer_size.argtypes = [vp] * 6 + [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
        L.cmp_gpsv_solve.argtypes = [vp] * 6 + [ctypes.c_int, ctypes.c_int, vp, vp]
        _lib = L
    return _lib


def gpsv_solve(a, b, c, d, e, y, m: int, n: int, stream=None):
    """Solve in place on y (interleaved layout) with cusparseDgpsvInterleavedBatch.
    Overwrites a..e.  Returns the scratch tensor (reuse it across calls)."""
    import torch
    L = lib()
    ptrs = [t.data_ptr() for t in (a, b, c, d, e, y)]
    nbytes = ctypes.c_size_t(0)
    rc = L.cmp_gpsv_buffer_size(*ptrs, n, m, ctypes.byref(nbytes))
    if rc:
        raise RuntimeError(f"gpsv buffer size: status {rc}")
    buf = torch.empty(max(1, int(nbytes.value)), dtype=torch.uint8, device=y.device)
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = L.cmp_gpsv_solve(*ptrs, n, m, buf.data_ptr(), s)
    if rc:
        raise RuntimeError(f"gpsv solve: status {rc}")
    return buf
