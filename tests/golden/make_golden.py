"""Generates the golden outputs of the reference's OWN kernels.

Runs on a GPU machine that holds oracle/_ref/kernel_{nofma,fma}.ptx (compiled
from the reference's kernel.cu by oracle/build_ref.sh) and libpcrp.so (for the
seeded input generator).  For every case in CASES it regenerates the inputs,
runs the reference kernels with the reference's launch geometry
(oracle/refrun.c), and writes

  <out>/cases.json              the cases with the sha256 of their inputs
  <out>/reference_outputs.npz   x of every case from both builds

which are committed under tests/golden/.

  python tests/golden/make_golden.py --out tests/golden
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


def input_digest(arrs) -> str:
    h = hashlib.sha256()
    for v in arrs:
        h.update(np.ascontiguousarray(v, dtype="<f8").tobytes())
    return h.hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden"))
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
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
