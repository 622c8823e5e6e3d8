"""The allocation-free solve, pcrp_solve_f64_noalloc.

It exists for callers that may not call the CUDA allocator (host callbacks,
plugin hooks, hosts whose device memory is fixed at start-up): its scratch is
an array compiled into the library.  These tests call it through the C ABI
and check, on two calls in a row, that it returns exactly what
pcrp_solve_f64 returns (the faithful path's tolerance is bit equality), that
batches of short systems (no scratch needed) have no size limit, and that a
batch of long systems larger than its fixed scratch is refused with an
error.  The file is named to be collected last and also passes when run on
its own."""
import numpy as np
import pytest

import pcrp
from helpers import assert_bitexact, dd_bands, to_device

pytestmark = pytest.mark.gpu


def test_noalloc_matches_solve_f64_twice(cuda):
    import torch
    for k, (m, n, layout) in enumerate(((4, 65536, pcrp.CONTIGUOUS), (6, 3000, pcrp.INTERLEAVED))):
        arrs = dd_bands(np.random.default_rng(500 + k), m, n)
        ref = to_device(arrs, cuda)
        pcrp.solve_f64(*ref, m, n, layout)
        got = to_device(arrs, cuda)
        pcrp.solve_f64_noalloc(*got, m, n, layout)
        torch.cuda.synchronize()
        assert_bitexact(got[5].cpu().numpy(), ref[5].cpu().numpy(), f"noalloc call {k}")


def test_noalloc_tridiagonal_null_outer_bands(cuda):
    import torch
    m, n = 4, 65536
    arrs = dd_bands(np.random.default_rng(9), m, n)
    arrs[0][:] = 0.0
    arrs[4][:] = 0.0
    ref = to_device(arrs, cuda)
    pcrp.solve_f64(*ref, m, n)
    got = to_device(arrs, cuda)
    pcrp.solve_f64_noalloc(None, got[1], got[2], got[3], None, got[5], m, n)
    torch.cuda.synchronize()
    assert_bitexact(got[5].cpu().numpy(), ref[5].cpu().numpy(), "noalloc tridiagonal")


def test_noalloc_short_systems_have_no_batch_limit(cuda):
    """Systems that fit the shared-memory tile touch no scratch: a batch of
    them far beyond the split path's limit is solved, bit-identically."""
    import torch
    m, n = 4096, 512                                   # 2^21 unknowns > 524288
    arrs = dd_bands(np.random.default_rng(77), m, n)
    ref = to_device(arrs, cuda)
    pcrp.solve_f64(*ref, m, n)
    got = to_device(arrs, cuda)
    pcrp.solve_f64_noalloc(*got, m, n)
    torch.cuda.synchronize()
    assert_bitexact(got[5].cpu().numpy(), ref[5].cpu().numpy(), "noalloc short systems")


def test_noalloc_refuses_batches_beyond_its_scratch(cuda):
    L = pcrp.lib()
    rc = L.pcrp_solve_f64_noalloc(1, 1, 1, 1, 1, 1, 16, 65536, 0, None)
    assert rc == 1
    assert "524288" in pcrp.last_error()
