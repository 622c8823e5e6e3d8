"""Parity pinned to the reference's OWN kernels.

tests/golden/reference_outputs.npz holds the solutions computed on a GB300 by
the reference's kernel.cu (compiled unmodified to PTX: once with -fmad=false,
once with nvcc's default FMA contraction) with the reference's launch
geometry, for the seeded cases in tests/golden/cases.json
(generated by tests/golden/make_golden.py through oracle/refrun.c).

* CPU: the oracle restatement equals the -fmad=false outputs bit for bit, and
  the default (FMA) build differs from it only by the reference's own
  contraction sensitivity, which grows with n: FMA_BOUND below gives, per
  system size, the relative forward distance allowed between pcrp (the
  -fmad=false bits) and the reference as shipped, about twice the largest
  distance measured on these cases.
* GPU: pcrp_solve_f64 equals the -fmad=false outputs bit for bit.

The large cases (n = 16384 ... 2^19, m = 4, splitting variants 2 and 3) keep
the sha256 of each build's output, the per-system max |x|, the measured
distances and row samples (tests/golden/large_cases.json, large_samples.npz),
since whole outputs would be tens of megabytes.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as O
import pcrp
from helpers import assert_bitexact

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = json.load(open(os.path.join(HERE, "cases.json")))
OUT = np.load(os.path.join(HERE, "reference_outputs.npz"))
LARGE = json.load(open(os.path.join(HERE, "large_cases.json")))
SAMPLES = np.load(os.path.join(HERE, "large_samples.npz"))
SAMPLE = 512

# Relative forward distance allowed between the -fmad=false bits (pcrp, the
# oracle) and the reference's default FMA build, by system size.  Measured
# on the golden cases: <= 4.4e-14 up to n = 1024, 1.0e-12 at 4096, 7.5e-13
# at 8192, 1.3e-12 at 16384, 4.7e-12 at 65536, 2.3e-11 (dominant) and
# 4.5e-11 (weakly dominant) at 2^19 -- the PCR-Penta arithmetic's own
# sensitivity to contraction; each build is as far from the banded
# elimination (1.4e-11 / 3.4e-11 at 2^19).
FMA_BOUND = [(1024, 1e-13), (8192, 2.5e-12), (16384, 3e-12), (65536, 1e-11), (1 << 19, 1e-10)]


def fma_bound(n: int) -> float:
    return next(b for nmax, b in FMA_BOUND if n <= nmax)


def sample_rows(n: int) -> np.ndarray:
    mid = n // 2 - SAMPLE // 2
    return np.concatenate([np.arange(SAMPLE), np.arange(mid, mid + SAMPLE), np.arange(n - SAMPLE, n)])


def output_digest(x) -> str:
    return hashlib.sha256(np.ascontiguousarray(x, dtype="<f8").tobytes()).hexdigest()


def sample_err(xs, ref, xmax) -> float:
    """max over systems of max |x - ref| on the sampled rows / max |x| of the system."""
    return float((np.abs(xs - ref).max(axis=1) / np.asarray(xmax)).max())


def inputs(c):
    arrs = pcrp.generate(c["kind"], c["seed"], c["m"], c["n"])
    h = hashlib.sha256()
    for v in arrs:
        h.update(np.ascontiguousarray(v, dtype="<f8").tobytes())
    assert h.hexdigest() == c["inputs_sha256"], "generator output changed: regenerate the goldens"
    return arrs


@pytest.mark.parametrize("c", CASES, ids=lambda c: f"case{c['case']}-n{c['n']}-v{c['variant']}")
def test_oracle_equals_reference_kernels(built_lib, c):
    arrs = inputs(c)
    m, n = c["m"], c["n"]
    xo = O.pcr(*arrs, m, n)
    assert_bitexact(xo, OUT[f"case{c['case']}_nofma"], "oracle vs reference (-fmad=false)")
    # the reference's default build contracts products into FMAs; its results
    # move by the algorithm's own rounding sensitivity, which grows with n
    fma = OUT[f"case{c['case']}_fma"]
    assert O.fwd_err(fma, xo, m, n) <= fma_bound(n)


@pytest.mark.parametrize("c", LARGE, ids=lambda c: f"large{c['case']}-n{c['n']}-v{c['variant']}")
def test_oracle_equals_reference_kernels_large(built_lib, c):
    """The restatement holds bit for bit to the reference's -fmad=false
    kernels up to n = 2^19 (the digest of every output bit); the FMA build
    stays within the per-n bound, on the samples and over the whole output."""
    arrs = inputs(c)
    m, n = c["m"], c["n"]
    xo = O.pcr(*arrs, m, n)
    assert output_digest(xo) == c["nofma_sha256"]
    i = c["case"]
    assert np.array_equal(xo.reshape(m, n)[:, sample_rows(n)].view(np.uint64), SAMPLES[f"large{i}_nofma"].view(np.uint64))
    assert c["fma_vs_nofma"] <= fma_bound(n)
    assert sample_err(SAMPLES[f"large{i}_fma"], SAMPLES[f"large{i}_nofma"], c["xmax"]) <= c["fma_vs_nofma"]


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=lambda c: f"case{c['case']}-n{c['n']}-v{c['variant']}")
def test_gpu_equals_reference_kernels(cuda, c):
    from helpers import gpu_f64
    arrs = inputs(c)
    x, _ = gpu_f64(arrs, c["m"], c["n"])
    assert_bitexact(x, OUT[f"case{c['case']}_nofma"], "pcrp_solve_f64 vs reference (-fmad=false)")


@pytest.mark.gpu
@pytest.mark.parametrize("c", LARGE, ids=lambda c: f"large{c['case']}-n{c['n']}-v{c['variant']}")
def test_gpu_equals_reference_kernels_large(cuda, c):
    """pcrp_solve_f64 gives every bit of the reference's -fmad=false output up
    to n = 2^19, so its distance to the reference as shipped is the
    reference's own (per-n bound)."""
    from helpers import gpu_f64
    arrs = inputs(c)
    m, n = c["m"], c["n"]
    x, _ = gpu_f64(arrs, m, n)
    assert output_digest(x) == c["nofma_sha256"], "pcrp_solve_f64 vs reference (-fmad=false) digest"
    xs = x.reshape(m, n)[:, sample_rows(n)]
    assert sample_err(xs, SAMPLES[f"large{c['case']}_fma"], c["xmax"]) <= fma_bound(n)


@pytest.mark.gpu
@pytest.mark.parametrize("c", LARGE, ids=lambda c: f"large{c['case']}-n{c['n']}-v{c['variant']}")
def test_gpu_mixed_within_reference_build_distance(cuda, c):
    """The mixed solver against the reference as shipped: its distance to the
    FMA build's output stays within that build's own distance from the banded
    elimination plus the mixed solver's 1e-12 bar (triangle inequality), on
    the sampled rows; and its own distance from the elimination meets the bar."""
    import torch
    from helpers import to_device
    arrs = inputs(c)
    m, n = c["m"], c["n"]
    t = to_device(arrs, cuda)
    pcrp.solve_mixed(*t, m, n, max_sweeps=16)
    torch.cuda.synchronize()
    xs = t[5].cpu().numpy().reshape(m, n)[:, sample_rows(n)]
    i, xmax = c["case"], c["xmax"]
    ge, fma = SAMPLES[f"large{i}_ge"], SAMPLES[f"large{i}_fma"]
    # (the ADI case is ill-conditioned: FP64 elimination itself is only good to
    # about cond*eps there, so it gets the 1e-11 bar of the other ADI tests)
    bar = 1e-12 if c["kind"] != pcrp.GEN_ADI else 1e-11
    assert sample_err(xs, ge, xmax) <= bar
    assert sample_err(xs, fma, xmax) <= sample_err(fma, ge, xmax) + bar
