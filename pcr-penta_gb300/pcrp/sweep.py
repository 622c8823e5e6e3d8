"""Reference-style timing sweep.

Times the solvers over the batch-size x system-size grid the reference's
timing driver uses (main.cu:242-244: 17 batch sizes from 26 to 2080, system
sizes 256 to 131072) and writes the reference's ``.dat`` layout: one line per
(m, n) with the mean time in milliseconds of ``runs`` solves (main.cu:256-287
averages 10), here one column per solver instead of one per splitting variant.
Inputs are the reference's fixture (``initialize``, kernel.cu:5-26) by default:
the fourth-difference stencil (1, -4, 6, -4, 1), whose condition number grows
like n^4, so only the FP64 path is timed on it by default; the mixed solver
(which refines to 1e-12 and stops after max_sweeps otherwise) belongs on a
well-conditioned generator (``--kind dominant``).  Unlike the reference, no
point is skipped for lack of memory; ``--max-unknowns`` bounds the grid instead.

    python -m pcrp.sweep --out sweep_gb300.dat
    python -m pcrp.sweep --solvers f64,mixed --kind dominant --batches 26,260 --sizes 512,65536 --runs 3
"""
from __future__ import annotations

import argparse
import sys

from . import (GEN_ADI, GEN_DOMINANT, GEN_TOEPLITZ, GEN_WEAK, generate_device, solve_f64, solve_mixed)

BATCHES = [26, 52, 104, 156, 208, 260, 312, 364, 416, 624, 832, 1040, 1248, 1456, 1664, 1872, 2080]
SIZES = [256, 512, 1024, 2048, 4096, 8192, 16384, 32768, 65536, 131072]
KINDS = {"toeplitz": GEN_TOEPLITZ, "dominant": GEN_DOMINANT, "adi": GEN_ADI, "weak": GEN_WEAK}


def time_solver(solver: str, m: int, n: int, kind: int, runs: int, seed: int = 1) -> float:
    """Mean milliseconds of `runs` solves (CUDA events around each, the rhs
    restored before each outside the events), after one untimed solve."""
    import torch
    arrs = [torch.empty(m * n, dtype=torch.float64, device="cuda") for _ in range(6)]
    generate_device(kind, seed, m, n, 0, arrs)
    rhs = arrs[5].clone()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def solve():
        if solver == "f64":
            solve_f64(*arrs, m, n)
        else:
            solve_mixed(*arrs, m, n, report=False)

    solve()
    total = 0.0
    for _ in range(runs):
        arrs[5].copy_(rhs)
        e0.record(st)
        solve()
        e1.record(st)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    del arrs, rhs
    torch.cuda.empty_cache()
    return total / runs


def sweep(solvers, batches, sizes, kind_name="toeplitz", runs=10, max_unknowns=1 << 29, out=None, verbose=True):
    """Runs the grid; returns [(m, n, [ms per solver, or None if skipped])]."""
    kind = KINDS[kind_name]
    rows = []
    for m in batches:
        for n in sizes:
            if m * n > max_unknowns:
                rows.append((m, n, [None] * len(solvers)))
                continue
            rows.append((m, n, [time_solver(s, m, n, kind, runs) for s in solvers]))
            if verbose:
                print(" %d \t %d" % (m, n), file=sys.stderr, flush=True)
    if out:
        with open(out, "w") as f:
            f.write(dat_text(rows, solvers, kind_name, runs))
    return rows


def dat_text(rows, solvers, kind_name, runs) -> str:
    names = {"f64": "pcrp_solve_f64 (bit-faithful PCR-Penta, FP64)",
             "mixed": "pcrp_solve_mixed (FP32 block reduction + FP64 refinement to 1e-12)"}
    head = ["Computational times (in milli-seconds) of the pcrp solvers, mean of %d solves." % runs,
            "Inputs: %s generator.  Columns after m and n:" % kind_name]
    head += ["  %s" % names[s] for s in solvers]
    head += ["Points with more unknowns than the sweep's bound are written as 0.", "",
             "m     \t  n    \t" + "\t".join("%-12s" % s for s in solvers)]
    lines = ["%d \t %d \t " % (m, n) + " \t ".join("%f" % (t if t is not None else 0.0) for t in ts)
             for m, n, ts in rows]
    return "\n".join(head + lines) + "\n"


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default="time_perform_analysis_pcrp.dat")
    ap.add_argument("--solvers", default="f64")
    ap.add_argument("--batches", default=",".join(map(str, BATCHES)))
    ap.add_argument("--sizes", default=",".join(map(str, SIZES)))
    ap.add_argument("--kind", default="toeplitz", choices=sorted(KINDS))
    ap.add_argument("--runs", type=int, default=10)
    ap.add_argument("--max-unknowns", type=int, default=1 << 29)
    args = ap.parse_args(argv)
    solvers = [s for s in args.solvers.split(",") if s]
    for s in solvers:
        if s not in ("f64", "mixed"):
            ap.error(f"unknown solver {s}")
    sweep(solvers, [int(v) for v in args.batches.split(",")], [int(v) for v in args.sizes.split(",")],
          args.kind, args.runs, args.max_unknowns, args.out)


if __name__ == "__main__":
    main()
