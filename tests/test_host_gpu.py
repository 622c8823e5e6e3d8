"""pcrp_solve_host: batches in host memory streamed through the GPU in chunks.
FP64 results must equal the device entry point bit for bit; mixed results
must meet the 1e-12 bar."""
import numpy as np
import pytest

import oracle as O
import pcrp
from helpers import assert_bitexact, dd_bands, gpu_f64, to_layout

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,layout", [(1, 100, 0), (13, 700, 0), (13, 700, 1), (9, 5000, 0), (9, 5000, 1), (64, 512, 0)])
def test_host_f64_equals_device(cuda, m, n, layout):
    import torch
    arrs = to_layout(dd_bands(np.random.default_rng(m * n), m, n, garbage=True), m, n, layout)
    xd, _ = gpu_f64(arrs, m, n, layout)
    h = [torch.from_numpy(v.copy()).pin_memory() for v in arrs]
    pcrp.solve_host(*h, m, n, layout, precision=0)
    torch.cuda.synchronize()
    assert_bitexact(h[5].numpy(), xd, f"host m={m} n={n} layout={layout}")
    for u, v in zip(h[:5], arrs[:5]):
        assert np.array_equal(u.numpy(), v)


@pytest.mark.parametrize("layout", [0, 1])
def test_host_tridiagonal_null_outer_bands(cuda, layout):
    """NULL a and e through the host entry point: not copied, same bits as
    explicit +0.0 bands on the device."""
    import torch
    m, n = 10, 3000
    arrs = dd_bands(np.random.default_rng(5), m, n)
    arrs[0][:] = 0.0
    arrs[4][:] = 0.0
    arrs = to_layout(arrs, m, n, layout)
    xd, _ = gpu_f64(arrs, m, n, layout)
    h = [None if k in (0, 4) else torch.from_numpy(v.copy()).pin_memory() for k, v in enumerate(arrs)]
    pcrp.solve_host(*h, m, n, layout, precision=0)
    torch.cuda.synchronize()
    assert_bitexact(h[5].numpy(), xd, f"host tridiagonal layout={layout}")
    hm = [None if k in (0, 4) else v.copy() for k, v in enumerate(arrs)]
    pcrp.solve_host(*hm, m, n, layout, precision=1)
    torch.cuda.synchronize()
    xr = O.ge(*arrs, m, n, layout)
    assert O.fwd_err(hm[5], xr, m, n, layout) <= 1e-12


def test_host_mixed_meets_tolerance_pageable(cuda):
    import torch
    m, n = 11, 3000
    arrs = dd_bands(np.random.default_rng(1), m, n)
    h = [v.copy() for v in arrs]                      # pageable numpy memory
    pcrp.solve_host(*h, m, n, precision=1)
    torch.cuda.synchronize()
    assert O.fwd_err(h[5], O.ge(*arrs, m, n), m, n) <= 1e-12


def test_host_concurrent_calls_on_two_streams(cuda):
    """Two host threads call pcrp_solve_host at once, each on its own caller
    stream, each right after queueing a device->host copy that fills its host
    right-hand side.  Each call must wait for its own stream's earlier work
    (its join events belong to the call) and return the device solve's bits."""
    import threading

    import torch
    m, n = 12, 3000
    cases = []
    for k in range(2):
        arrs = dd_bands(np.random.default_rng(100 + k), m, n)
        xd, _ = gpu_f64(arrs, m, n)
        h = [torch.from_numpy(v.copy()).pin_memory() for v in arrs]
        h[5].zero_()                                    # filled by the stream copy below
        y_dev = torch.from_numpy(arrs[5]).to(cuda)
        cases.append((h, y_dev, xd, torch.cuda.Stream()))
    errors = []

    def worker(k):
        h, y_dev, xd, st = cases[k]
        try:
            for _ in range(4):
                with torch.cuda.stream(st):
                    torch.cuda._sleep(2000000)          # the copy below lands late
                    h[5].copy_(y_dev, non_blocking=True)
                    pcrp.solve_host(*h, m, n, precision=0, stream=st)
                st.synchronize()
                assert_bitexact(h[5].numpy(), xd, f"thread {k}")
        except Exception as ex:                         # reported by the main thread
            errors.append(ex)

    th = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors[0]
