"""Generates the golden outputs of the reference's OWN kernels.

Runs on a GPU machine that holds oracle/_ref/kernel_{nofma,fma}.ptx (compiled
from the reference's kernel.cu by oracle/build_ref.sh) and libpcrp.so (for the
seeded input generator).  For every case in CASES it regenerates the inputs,
runs the reference kernels with the reference's launch geometry
(oracle/refrun.c), and writes

  <out>/cases.json              the cases with the sha256 of their inputs
  <out>/reference_outputs.npz   x of every case from both builds

and, for the large cases (whole outputs would be tens of megabytes), per
case the sha256 of each build's output bits, the per-system max |x|, the
distances between the builds and to the FMA-free banded elimination
(oracle), and row samples (the first, middle and last SAMPLE rows of every
system) of both builds and of the elimination:

  <out>/large_cases.json
  <out>/large_samples.npz

which are committed under tests/golden/.

  python tests/golden/make_golden.py --out tests/golden [--large-only]
"""
import argparse
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "pcr-penta_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pcrp  # noqa: E402
import refrun  # noqa: E402

# (kind, seed, m, n, variant)
CASES = [
    (pcrp.GEN_DOMINANT, 101, 4, 512, refrun.VARIANT_SMALL),
    (pcrp.GEN_DOMINANT, 102, 2, 1024, refrun.VARIANT_SMALL),
    (pcrp.GEN_DOMINANT, 103, 3, 100, refrun.VARIANT_SMALL),
    (pcrp.GEN_DOMINANT, 108, 8, 5, refrun.VARIANT_SMALL),
    (pcrp.GEN_TOEPLITZ, 0, 1, 256, refrun.VARIANT_SMALL),
    (pcrp.GEN_DOMINANT, 104, 2, 4096, refrun.VARIANT_GLOBAL_SHARED),
    (pcrp.GEN_DOMINANT, 104, 2, 4096, refrun.VARIANT_GLOBAL_GLOBAL),
    (pcrp.GEN_ADI, 105, 2, 4096, refrun.VARIANT_GLOBAL_SHARED),
    (pcrp.GEN_WEAK, 107, 1, 8192, refrun.VARIANT_GLOBAL_GLOBAL),
    (pcrp.GEN_DOMINANT, 106, 1, 65536, refrun.VARIANT_GLOBAL_SHARED),
]


# (kind, seed, m, n, variant): the reference's splitting kernels hold up to
# n = 2^19 (every stage-1 kernel looks one 512-row tile back)
LARGE_CASES = [
    (pcrp.GEN_DOMINANT, 201, 4, 16384, refrun.VARIANT_GLOBAL_SHARED),
    (pcrp.GEN_ADI, 202, 4, 16384, refrun.VARIANT_GLOBAL_GLOBAL),
    (pcrp.GEN_DOMINANT, 203, 4, 65536, refrun.VARIANT_GLOBAL_GLOBAL),
    (pcrp.GEN_DOMINANT, 204, 4, 1 << 19, refrun.VARIANT_GLOBAL_SHARED),
    (pcrp.GEN_WEAK, 205, 4, 1 << 19, refrun.VARIANT_GLOBAL_GLOBAL),
]
SAMPLE = 512


def sample_rows(n: int) -> np.ndarray:
    """Row indices of the samples kept for every system of a large case."""
    mid = n // 2 - SAMPLE // 2
    return np.concatenate([np.arange(SAMPLE), np.arange(mid, mid + SAMPLE), np.arange(n - SAMPLE, n)])


def output_digest(x) -> str:
    return hashlib.sha256(np.ascontiguousarray(x, dtype="<f8").tobytes()).hexdigest()


def input_digest(arrs) -> str:
    h = hashlib.sha256()
    for v in arrs:
        h.update(np.ascontiguousarray(v, dtype="<f8").tobytes())
    return h.hexdigest()


def large(out_dir: str) -> None:
    import oracle as O
    manifest, samples = [], {}
    for i, (kind, seed, m, n, variant) in enumerate(LARGE_CASES):
        arrs = pcrp.generate(kind, seed, m, n)
        xs = {b: refrun.solve(arrs, m, n, variant, fma=(b == "fma")) for b in ("nofma", "fma")}
        xg = O.ge(*arrs, m, n)
        rows = sample_rows(n)
        entry = dict(case=i, kind=kind, seed=seed, m=m, n=n, variant=variant, inputs_sha256=input_digest(arrs),
                     nofma_sha256=output_digest(xs["nofma"]), fma_sha256=output_digest(xs["fma"]),
                     xmax=[float(np.abs(xs["nofma"][j * n:(j + 1) * n]).max()) for j in range(m)],
                     fma_vs_nofma=O.fwd_err(xs["fma"], xs["nofma"], m, n),
                     nofma_vs_ge=O.fwd_err(xs["nofma"], xg, m, n), fma_vs_ge=O.fwd_err(xs["fma"], xg, m, n))
        for b, x in list(xs.items()) + [("ge", xg)]:
            samples[f"large{i}_{b}"] = x.reshape(m, n)[:, rows].copy()
        manifest.append(entry)
        print(f"large case {i}: kind={kind} m={m} n={n} variant={variant}: fma vs nofma "
              f"{entry['fma_vs_nofma']:.3e}, vs GE {entry['nofma_vs_ge']:.3e} / {entry['fma_vs_ge']:.3e}", flush=True)
    with open(os.path.join(out_dir, "large_cases.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    np.savez_compressed(os.path.join(out_dir, "large_samples.npz"), **samples)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden"))
    ap.add_argument("--large-only", action="store_true", help="regenerate only the large cases")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    large(args.out)
    if args.large_only:
        return
    manifest, outs = [], {}
    for i, (kind, seed, m, n, variant) in enumerate(CASES):
        arrs = pcrp.generate(kind, seed, m, n)
        entry = dict(case=i, kind=kind, seed=seed, m=m, n=n, variant=variant, inputs_sha256=input_digest(arrs))
        for fma in (False, True):
            outs[f"case{i}_{'fma' if fma else 'nofma'}"] = refrun.solve(arrs, m, n, variant, fma=fma)
        manifest.append(entry)
        print(f"case {i}: kind={kind} m={m} n={n} variant={variant} done", flush=True)
    with open(os.path.join(args.out, "cases.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    np.savez_compressed(os.path.join(args.out, "reference_outputs.npz"), **outs)


if __name__ == "__main__":
    main()
