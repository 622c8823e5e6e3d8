"""pcrp -- Python host binding of the GB300 batched pentadiagonal PCR solver.

The product is ``libpcrp.so`` behind the C ABI in ``include/pcrp.h``; this
module binds it with ctypes so tests, the benchmark and Python users call the
same entry points a C/C++ caller would.  Device memory is passed as raw
pointers (``int``) or as CUDA ``torch.Tensor`` objects (float64, contiguous);
streams as raw handles or ``torch.cuda.Stream``.

The functions mirror the reference's interface for the hot path
(PCR-Penta main.cu:46-87 dispatching kernel.cu:32-154 for n <= 1024 and
kernel.cu:158-791 for n > 1024): five bands a..e plus the right-hand side y,
batch size m, system size n; the solution overwrites y.  Errors raise
:class:`PcrpError` carrying the library's status code.  There is no CPU
fallback: if the library is missing, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

from . import build as _build

CONTIGUOUS = 0
INTERLEAVED = 1

GEN_DOMINANT = 0
GEN_ADI = 1
GEN_WEAK = 2
GEN_TOEPLITZ = 3

STATUS = {0: "PCRP_OK", 1: "PCRP_EINVAL", 2: "PCRP_ECUDA", 3: "PCRP_ENOMEM",
          4: "PCRP_ETIMEOUT", 5: "PCRP_ENOCONV", 6: "PCRP_ENOTSUP"}


class PcrpError(RuntimeError):
    """A C-ABI call returned a status other than PCRP_OK."""

    def __init__(self, status: int, func: str, msg: str):
        super().__init__(f"{func}: {STATUS.get(status, status)}: {msg}")
        self.status = status
        self.func = func


class Opts(ctypes.Structure):
    """Mirror of ``pcrp_opts``."""
    _fields_ = [("size", ctypes.c_uint32), ("smem_rows", ctypes.c_int32),
                ("fuse_strides", ctypes.c_int32), ("tile_rows", ctypes.c_int32),
                ("threads", ctypes.c_int32), ("reserved0", ctypes.c_int32),
                ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t),
                ("window_levels", ctypes.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        self.size = ctypes.sizeof(Opts)
        for k, v in kw.items():
            setattr(self, k, v)


class MixedInfo(ctypes.Structure):
    """Mirror of ``pcrp_mixed_info``."""
    _fields_ = [("sweeps", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("fwd_err_est", ctypes.c_double), ("resid", ctypes.c_double)]


_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_lib: Optional[ctypes.CDLL] = None

# name -> argtypes (restype is always the int status unless listed in _RESTYPE)
_SIGS = {
    "pcrp_solve_f64": [_vp] * 6 + [_i64, _i64, _i32, _vp, _vp],
    "pcrp_solve_f64_small": [_vp] * 6 + [_i64, _i64, _i32, _vp, _vp],
    "pcrp_solve_f64_split": [_vp] * 6 + [_i64, _i64, _i32, _vp, _vp],
    "pcrp_solve_f64_noalloc": [_vp] * 6 + [_i64, _i64, _i32, _vp],
    "pcrp_solve_mixed": [_vp] * 6 + [_i64, _i64, _i32, ctypes.c_double, _i32, _vp, _vp, _vp],
    "pcrp_residual_f64": [_vp] * 8 + [_i64, _i64, _i32, _vp],
    "pcrp_solve_host": [_vp] * 6 + [_i64, _i64, _i32, _i32, ctypes.c_double, _i32, _vp, _vp],
    "pcrp_solve_ragged": [_vp] * 6 + [_vp, _i64, _i64, _i32, ctypes.c_double, _i32, _vp, _vp],
    "pcrp_workspace_size": [_i64, _i64, _i32, _i32, _vp, ctypes.POINTER(ctypes.c_size_t)],
    "pcrp_release_workspace": [],
    "pcrp_get_last_error_string": [],
    "pcrp_version": [],
    "pcrp_kernel_launches": [],
    "pcrp_measure_fp64": [_vp, _vp, _vp],
    "pcrp_measure_pipes": [_vp, _vp],
    "pcrp_check_quotients": [_i32, ctypes.c_uint64, _i64, _vp, _vp, _vp],
    "pcrp_generate": [_i32, ctypes.c_uint64, _i64, _i64, _i32] + [_vp] * 6 + [_i32],
    "pcrp_generate_device": [_i32, ctypes.c_uint64, _i64, _i64, _i32] + [_vp] * 6 + [_vp],
    "pcrp_ragged_sizes": [ctypes.c_uint64, _i64, _i64, _i64, _vp],
    "pcrp_generate_ragged": [_i32, ctypes.c_uint64, _vp, _i64] + [_vp] * 6 + [_i32],
}
_RESTYPE = {"pcrp_get_last_error_string": ctypes.c_char_p, "pcrp_version": _i32,
            "pcrp_kernel_launches": _i64}


def lib_path() -> str:
    return _build.LIB_PATH


def lib() -> ctypes.CDLL:
    """Load ``libpcrp.so`` (built in tree by :func:`pcrp.build.build`)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with pcrp.build.build() "
                               "(there is no CPU fallback)")
        L = ctypes.CDLL(path)
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = L
    return _lib


def exported_symbols() -> Sequence[str]:
    return list(_SIGS)


def last_error() -> str:
    s = lib().pcrp_get_last_error_string()
    return s.decode() if s else ""


def _check(rc: int, func: str) -> None:
    if rc != 0:
        raise PcrpError(rc, func, last_error())


def _check_tensor(x, count: int, dtype: str) -> None:
    # the library reads count elements of this type through the raw pointer
    if str(x.dtype).replace("torch.", "") != dtype:
        raise TypeError(f"expected a {dtype} tensor, got {x.dtype}")
    if not x.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    if x.numel() < count:
        raise ValueError(f"tensor of {x.numel()} elements where {count} are read")


def _ptr(x, count: int = 0, dtype: str = "float64") -> Optional[int]:
    """Raw device pointer of a CUDA tensor (contiguous, of `dtype`, at least
    `count` elements) or an int (an address, taken as it is)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("expected a CUDA tensor")
        _check_tensor(x, count, dtype)
        return x.data_ptr()
    raise TypeError(f"cannot take a device pointer of {type(x)}")


def _count(m: int, n: int) -> int:
    return m * n if m > 0 and n > 0 else 0


def _stream(s) -> Optional[int]:
    if s is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except Exception:
            pass
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream


def _opts(opts: Optional[Opts]):
    return ctypes.byref(opts) if opts is not None else None


def solve_f64(a, b, c, d, e, y, m: int, n: int, layout: int = CONTIGUOUS,
              opts: Optional[Opts] = None, stream=None, path: str = "auto") -> None:
    """FP64 PCR-Penta solve in place on y (pcrp_solve_f64 / _small / _split)."""
    fn = {"auto": "pcrp_solve_f64", "small": "pcrp_solve_f64_small", "split": "pcrp_solve_f64_split"}[path]
    rc = getattr(lib(), fn)(*[_ptr(v, _count(m, n)) for v in (a, b, c, d, e, y)], m, n, layout,
                            _opts(opts), _stream(stream))
    _check(rc, fn)


def solve_f64_noalloc(a, b, c, d, e, y, m: int, n: int, layout: int = CONTIGUOUS, stream=None) -> None:
    """pcrp_solve_f64 without any device allocation (scratch is a fixed array
    inside the library; m*n <= 524288)."""
    rc = lib().pcrp_solve_f64_noalloc(*[_ptr(v, _count(m, n)) for v in (a, b, c, d, e, y)], m, n, layout,
                                      _stream(stream))
    _check(rc, "pcrp_solve_f64_noalloc")


def solve_mixed(a, b, c, d, e, y, m: int, n: int, layout: int = CONTIGUOUS, tol: float = 1e-12,
                max_sweeps: int = 8, opts: Optional[Opts] = None, stream=None,
                report: bool = True) -> Optional[MixedInfo]:
    """FP32 PCR + FP64 refinement in place on y; returns the info when report=True."""
    info = MixedInfo() if report else None
    rc = lib().pcrp_solve_mixed(*[_ptr(v, _count(m, n)) for v in (a, b, c, d, e, y)], m, n, layout, tol, max_sweeps,
                                _opts(opts), _stream(stream), ctypes.byref(info) if info is not None else None)
    _check(rc, "pcrp_solve_mixed")
    return info


def _host_ptr(x, count: int = 0) -> Optional[int]:
    """Address of a host array (numpy or CPU tensor: contiguous float64, at
    least `count` elements) or an int (an address, taken as it is)."""
    if x is None:
        return None
    if hasattr(x, "ctypes"):
        if str(x.dtype) != "float64":
            raise TypeError(f"expected a float64 array, got {x.dtype}")
        if not x.flags.c_contiguous:
            raise ValueError("expected a contiguous array")
        if x.size < count:
            raise ValueError(f"array of {x.size} elements where {count} are read")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if x.is_cuda:
            raise ValueError("expected a host tensor")
        _check_tensor(x, count, "float64")
        return x.data_ptr()
    return int(x)


def solve_host(a, b, c, d, e, y, m: int, n: int, layout: int = CONTIGUOUS, precision: int = 0,
               tol: float = 1e-12, max_sweeps: int = 8, opts: Optional[Opts] = None, stream=None) -> None:
    """Solve a batch held in host memory (numpy arrays or CPU tensors, float64):
    chunks stream through the GPU with copies overlapping solves (pcrp_solve_host).
    Asynchronous on `stream`; synchronise before reading y."""
    rc = lib().pcrp_solve_host(*[_host_ptr(v, _count(m, n)) for v in (a, b, c, d, e, y)], m, n, layout, precision, tol,
                               max_sweeps, _opts(opts), _stream(stream))
    _check(rc, "pcrp_solve_host")


def residual_f64(a, b, c, d, e, y, x, r, m: int, n: int, layout: int = CONTIGUOUS, stream=None) -> None:
    rc = lib().pcrp_residual_f64(*[_ptr(v, _count(m, n)) for v in (a, b, c, d, e, y, x, r)], m, n, layout,
                                 _stream(stream))
    _check(rc, "pcrp_residual_f64")


def solve_ragged(a, b, c, d, e, y, offsets, nsys: int, max_rows: int, mode: int = 0,
                 tol: float = 1e-12, max_sweeps: int = 8, opts: Optional[Opts] = None, stream=None) -> None:
    # (the arrays' length is offsets[nsys], on the device: only their type is checked here)
    rc = lib().pcrp_solve_ragged(*[_ptr(v) for v in (a, b, c, d, e, y)], _ptr(offsets, nsys + 1, "int64"),
                                 nsys, max_rows,
                                 mode, tol, max_sweeps, _opts(opts), _stream(stream))
    _check(rc, "pcrp_solve_ragged")


def workspace_size(m: int, n: int, layout: int = CONTIGUOUS, which: int = 0,
                   opts: Optional[Opts] = None) -> int:
    out = ctypes.c_size_t(0)
    rc = lib().pcrp_workspace_size(m, n, layout, which, _opts(opts), ctypes.byref(out))
    _check(rc, "pcrp_workspace_size")
    return int(out.value)


def release_workspace() -> None:
    _check(lib().pcrp_release_workspace(), "pcrp_release_workspace")


def version() -> int:
    return int(lib().pcrp_version())


def kernel_launches() -> int:
    """Kernels launched by libpcrp in this process so far."""
    return int(lib().pcrp_kernel_launches())


def measure_fp64(stream=None):
    """(DFMA/s, IEEE FP64 divisions/s) of this GPU, from two throughput
    kernels (pcrp_measure_fp64); synchronous."""
    f, d = ctypes.c_double(0.0), ctypes.c_double(0.0)
    _check(lib().pcrp_measure_fp64(ctypes.byref(f), ctypes.byref(d), _stream(stream)), "pcrp_measure_fp64")
    return f.value, d.value


def measure_pipes(stream=None) -> dict:
    """Milliseconds of the pipe-sharing probe (pcrp_measure_pipes): FP64,
    FP32 and integer chains alone, and FP64 beside FP32 or integer work on
    the other warps of the same SMs; synchronous."""
    ms = (ctypes.c_float * 5)()
    _check(lib().pcrp_measure_pipes(ms, _stream(stream)), "pcrp_measure_pipes")
    return dict(zip(("fp64", "fp32", "int", "fp64+fp32", "fp64+int"), list(ms)))


def check_quotients(mode: int, seed: int, samples: int, stream=None):
    """(mismatches, pairs inside the guard) of the FP64 kernels' phase-B
    quotient against IEEE division on `samples` random pairs of operand class
    `mode` (pcrp_check_quotients); synchronous."""
    bad, fast = ctypes.c_uint64(0), ctypes.c_uint64(0)
    _check(lib().pcrp_check_quotients(mode, seed, samples, ctypes.byref(bad), ctypes.byref(fast), _stream(stream)),
           "pcrp_check_quotients")
    return int(bad.value), int(fast.value)


# ----------------------------------------------------------------------------
# generators (host numpy arrays)
# ----------------------------------------------------------------------------

def generate(kind: int, seed: int, m: int, n: int, layout: int = CONTIGUOUS, threads: int = 0):
    """Six float64 numpy arrays (a, b, c, d, e, y) of m*n values."""
    import numpy as np
    arrs = [np.empty(m * n, dtype=np.float64) for _ in range(6)]
    rc = lib().pcrp_generate(kind, seed, m, n, layout, *[v.ctypes.data for v in arrs], threads)
    _check(rc, "pcrp_generate")
    return arrs


def generate_into(kind: int, seed: int, m: int, n: int, layout: int, arrs, threads: int = 0) -> None:
    """Fill six preallocated host float64 arrays (numpy or pinned CPU tensors)."""
    ptrs = [_host_ptr(v, _count(m, n)) for v in arrs]
    rc = lib().pcrp_generate(kind, seed, m, n, layout, *ptrs, threads)
    _check(rc, "pcrp_generate")


def generate_device(kind: int, seed: int, m: int, n: int, layout: int, arrs, stream=None) -> None:
    """Fill six device float64 arrays with the same values as :func:`generate`."""
    rc = lib().pcrp_generate_device(kind, seed, m, n, layout, *[_ptr(v, _count(m, n)) for v in arrs],
                                    _stream(stream))
    _check(rc, "pcrp_generate_device")


def ragged_sizes(seed: int, nsys: int, nmin: int, nmax: int):
    import numpy as np
    out = np.empty(nsys, dtype=np.int64)
    rc = lib().pcrp_ragged_sizes(seed, nsys, nmin, nmax, out.ctypes.data)
    _check(rc, "pcrp_ragged_sizes")
    return out


def generate_ragged(kind: int, seed: int, offsets, threads: int = 0):
    """Six float64 arrays holding the ragged systems contiguous at offsets (nsys+1 int64)."""
    import numpy as np
    offs = np.ascontiguousarray(offsets, dtype=np.int64)
    total = int(offs[-1])
    arrs = [np.empty(total, dtype=np.float64) for _ in range(6)]
    rc = lib().pcrp_generate_ragged(kind, seed, offs.ctypes.data, len(offs) - 1,
                                    *[v.ctypes.data for v in arrs], threads)
    _check(rc, "pcrp_generate_ragged")
    return arrs


def ref_strides(n: int) -> int:
    """Strides the reference runs for n rows (main.cu:38-39, see pcrp_internal.h)."""
    if n <= 1:
        return 0
    lg = (n - 1).bit_length()
    return lg if (1 << lg) == n else lg - 1
