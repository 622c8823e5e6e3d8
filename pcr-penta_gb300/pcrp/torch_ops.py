"""PyTorch operators over the C ABI: ``torch.ops.pcrp.solve_f64`` and
``torch.ops.pcrp.solve_mixed``.

Each takes the five bands and the right-hand side as CUDA float64 tensors of
shape (m, n) (contiguous layout) or (n, m) with ``interleaved=True``, and
returns the solution as a new tensor (the inputs are not modified).  The work
runs on the current CUDA stream.  No autograd: the solve is a batched linear
solve used inside larger pipelines, not a differentiable layer.
"""
from __future__ import annotations

import torch

from . import CONTIGUOUS, INTERLEAVED, solve_f64, solve_mixed


def _shape(y: torch.Tensor, interleaved: bool):
    if y.dim() != 2:
        raise ValueError("expected (m, n) tensors (or (n, m) when interleaved)")
    return (y.shape[1], y.shape[0]) if interleaved else (y.shape[0], y.shape[1])


def _check(ts):
    for t in ts:
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise ValueError("bands and rhs must be contiguous CUDA float64 tensors")
    if len({tuple(t.shape) for t in ts}) != 1:
        raise ValueError("bands and rhs must have the same shape")


@torch.library.custom_op("pcrp::solve_f64", mutates_args=())
def solve_f64_op(a: torch.Tensor, b: torch.Tensor, c: torch.Tensor, d: torch.Tensor, e: torch.Tensor,
                 y: torch.Tensor, interleaved: bool = False) -> torch.Tensor:
    _check((a, b, c, d, e, y))
    m, n = _shape(y, interleaved)
    x = y.clone()
    solve_f64(a, b, c, d, e, x, m, n, INTERLEAVED if interleaved else CONTIGUOUS,
              stream=torch.cuda.current_stream().cuda_stream)
    return x


@solve_f64_op.register_fake
def _(a, b, c, d, e, y, interleaved=False):
    return torch.empty_like(y)


@torch.library.custom_op("pcrp::solve_mixed", mutates_args=())
def solve_mixed_op(a: torch.Tensor, b: torch.Tensor, c: torch.Tensor, d: torch.Tensor, e: torch.Tensor,
                   y: torch.Tensor, interleaved: bool = False, tol: float = 1e-12,
                   max_sweeps: int = 8) -> torch.Tensor:
    _check((a, b, c, d, e, y))
    m, n = _shape(y, interleaved)
    x = y.clone()
    solve_mixed(a, b, c, d, e, x, m, n, INTERLEAVED if interleaved else CONTIGUOUS, tol=tol,
                max_sweeps=max_sweeps, stream=torch.cuda.current_stream().cuda_stream, report=False)
    return x


@solve_mixed_op.register_fake
def _(a, b, c, d, e, y, interleaved=False, tol=1e-12, max_sweeps=8):
    return torch.empty_like(y)
