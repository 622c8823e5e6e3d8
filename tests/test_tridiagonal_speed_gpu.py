"""Tridiagonal batches (a = e = 0) through pcrp_solve_f64, timed three ways on
the same GB300: the outer bands passed as NULL (not read; every pass runs the
zero-operand strides), passed as explicit +0.0 arrays (read; only the passes
of long strides vote on the zero state), and, for scale, the dense
pentadiagonal batch the zeros were cut from.  The NULL-band solve must give
the explicit-band solve's bits; the mixed solver's NULL-band time is printed
beside them.  Inputs are restored before every timed solve; CUDA events on
the current stream time the solve only; times are printed (run with -s)."""
import numpy as np
import pytest

import pcrp

pytestmark = pytest.mark.gpu

CASES = [(256, 65536), (1024, 512), (64, 1 << 20)]


def time_solve(dev, m, n, drop=(), solver="f64", reps=5):
    import torch
    args = [None if k in drop else v for k, v in enumerate(dev)]
    rhs = dev[5].clone()

    def run():
        if solver == "f64":
            pcrp.solve_f64(*args, m, n)
        else:
            pcrp.solve_mixed(*args, m, n, report=False)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for k in range(reps + 2):
        dev[5].copy_(rhs)
        torch.cuda.synchronize()
        e0.record()
        run()
        e1.record()
        e1.synchronize()
        if k >= 2:
            times.append(e0.elapsed_time(e1))
    x = dev[5].clone()
    dev[5].copy_(rhs)
    return x, float(np.median(times))


@pytest.mark.parametrize("m,n", CASES)
def test_tridiagonal_null_bands_timed(cuda, m, n):
    import torch
    dev = [torch.empty(m * n, dtype=torch.float64, device=cuda) for _ in range(6)]
    pcrp.generate_device(pcrp.GEN_DOMINANT, 7, m, n, pcrp.CONTIGUOUS, dev)
    torch.cuda.synchronize()
    _, ms_dense = time_solve(dev, m, n)
    dev[0].zero_()
    dev[4].zero_()
    x_zero, ms_zero = time_solve(dev, m, n)
    x_null, ms_null = time_solve(dev, m, n, drop=(0, 4))
    _, ms_mixed = time_solve(dev, m, n, drop=(0, 4), solver="mixed")
    assert torch.equal(x_null.view(torch.int64), x_zero.view(torch.int64))
    g = m * n / 1e6
    print(f"\n[m={m} n={n}] pcrp_solve_f64: pentadiagonal {ms_dense:.3f} ms ({g / ms_dense:.3f} Gunk/s), "
          f"tridiagonal with +0.0 bands {ms_zero:.3f} ms ({g / ms_zero:.3f}), "
          f"with NULL a, e {ms_null:.3f} ms ({g / ms_null:.3f}); "
          f"pcrp_solve_mixed with NULL a, e {ms_mixed:.3f} ms ({g / ms_mixed:.3f})")
