"""The reference's own CUDA kernels (PCR-Penta kernel.cu, compiled unmodified
by oracle/build_ref.sh and launched with main.cu's geometry by
oracle/refrun.c) timed beside pcrp_solve_f64 on the same GB300 and the same
inputs: both results are checked bit for bit (the reference built without
FMA contraction), and the times are printed (run with -s) as the record of
the drop-in's speed-up over the code it replaces.  Inputs are restored
before every timed solve; CUDA events time the launches only."""
import numpy as np
import pytest

import pcrp

R = pytest.importorskip("refrun")

pytestmark = pytest.mark.gpu

CASES = [  # (workload, m, n, reference variant): the shared-memory and the large-n workloads
    ("n=512 (shared-memory path)", 1024, 512, 0),
    ("n=65536, global_cached_shared_tile_splitting + 2nd stage", 256, 65536, 2),
    ("n=65536, global_cached_global_tile_splitting + 2nd stage", 256, 65536, 3),
]


def time_pcrp(arrs, m, n, reps=3):
    import torch
    dev = [torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in arrs]
    rhs = dev[5].clone()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pcrp.solve_f64(*dev, m, n)
    torch.cuda.synchronize()
    x = dev[5].cpu().numpy()
    total = 0.0
    for _ in range(reps):
        dev[5].copy_(rhs)
        torch.cuda.synchronize()
        e0.record()
        pcrp.solve_f64(*dev, m, n)
        e1.record()
        e1.synchronize()
        total += e0.elapsed_time(e1)
    return x, total / reps


@pytest.mark.skipif(not R.available(), reason="the reference's PTX is built where its sources exist")
@pytest.mark.parametrize("name,m,n,variant", CASES)
def test_reference_kernels_beside_pcrp(cuda, name, m, n, variant):
    arrs = pcrp.generate(pcrp.GEN_DOMINANT, 7, m, n)
    x_ref, ms_ref = R.time_solve(arrs, m, n, variant, fma=False)
    _, ms_ref_fma = R.time_solve(arrs, m, n, variant, fma=True)
    x, ms = time_pcrp(arrs, m, n)
    assert np.array_equal(x.view(np.uint64), x_ref.view(np.uint64))
    print(f"\n[{name}] m={m}: reference kernels {ms_ref:.3f} ms (as shipped, FMA contraction: {ms_ref_fma:.3f} ms), "
          f"pcrp_solve_f64 {ms:.3f} ms -> {ms_ref / ms:.1f}x ({ms_ref_fma / ms:.1f}x); "
          f"{m * n / ms / 1e6:.3f} vs {m * n / ms_ref / 1e6:.3f} Gunknowns/s")
