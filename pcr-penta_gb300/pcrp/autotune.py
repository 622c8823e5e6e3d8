"""Autotuner for the tile sizes, fused-stride depth and shared/global split.

Times every candidate configuration of the faithful FP64 path and of the
mixed-precision path's general passes on representative batch shapes (CUDA
events, median of several solves on a resident batch), keeps the fastest per
size class, times
the plan of the ragged FP64 path (one persistent kernel for every system, so
one plan for all sizes) on a log-uniform ragged batch, and writes

  * a JSON record of every measurement (``--json``), and
  * ``csrc/tuned_params.h`` (``--write``), whose tables the library compiles
    in as its defaults (``pcrp_opts`` fields still override them per call).

The FP64 results do not depend on the choice (every plan is bit-exact with the
reference); the mixed results move only at rounding level.

  python -m pcrp.autotune --json profiles/autotune_gb300.json --write
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import statistics
import time

from . import GEN_DOMINANT, Opts, generate_device, generate_ragged, ragged_sizes, solve_f64, solve_mixed, \
    solve_ragged
from .build import CSRC

# (size-class upper bound n_max, batch m used to time it)
F64_CLASSES = [(512, 1024), (1024, 1024), (8192, 256), (131072, 64), (1 << 21, 8)]
MP_CLASSES = [(1024, 2048), (8192, 1024), (131072, 128), (1 << 21, 16)]
# ragged batch timed for the ragged path's plan: systems, sizes log-uniform in [lo, hi]
RAGGED_BATCH = (512, 32, 65536)


def _timeit(fn, reps=5, warm=1):
    import torch
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(warm):
        fn()
    out = []
    for _ in range(reps):
        e0.record(s)
        fn()
        e1.record(s)
        e1.synchronize()
        out.append(e0.elapsed_time(e1))
    return statistics.median(out)


def _batch(m, n, seed=1):
    import torch
    arrs = [torch.empty(m * n, dtype=torch.float64, device="cuda") for _ in range(6)]
    generate_device(GEN_DOMINANT, seed, m, n, 0, arrs)
    return arrs


def f64_candidates():
    for smem, fuse, threads in itertools.product((480, 512, 640, 960, 1920), (1, 2, 3, 4, 5), (128, 256)):
        H = 2 * ((1 << fuse) - 1)
        if smem - 2 * H < 64:
            continue
        yield dict(smem_rows=smem, fuse_strides=fuse, tile_rows=smem - 2 * H, threads=threads)


def rg_candidates():
    # the persistent kernel runs 256 threads and up to 512 rows per tile
    for smem, fuse in itertools.product((384, 448, 480, 512), (1, 2, 3)):
        H = 2 * ((1 << fuse) - 1)
        yield dict(smem_rows=smem, fuse_strides=fuse, tile_rows=smem - 2 * H, threads=256)


def mp_candidates():
    # The mixed table steers the general block-PCR passes: the path of systems
    # longer than one tile that the windowed reduction leaves coupled.  Dominant
    # systems decouple in the windows, so the candidates run with the windows
    # off (window_levels = -1) to time the passes the table plans.
    for cap, fuse in itertools.product((256, 512, 1024, 2048), (2, 3, 4, 5, 6, 7)):
        if cap - 2 * ((1 << fuse) - 1) < 32:
            continue
        yield dict(smem_rows=2 * cap, fuse_strides=fuse, window_levels=-1)


def tune_ragged(verbose: bool = True):
    """Times the ragged path's plan candidates; returns (measurements, best)."""
    import numpy as np
    import torch
    nsys, lo, hi = RAGGED_BATCH
    sizes = ragged_sizes(1, nsys, lo, hi)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    arrs = [torch.from_numpy(v).cuda() for v in generate_ragged(GEN_DOMINANT, 1, offs)]
    rhs = arrs[5].clone()
    d_off = torch.from_numpy(offs).cuda()
    meas, best = [], None
    for c in rg_candidates():
        o = Opts(**c)

        def run():
            arrs[5].copy_(rhs)
            solve_ragged(*arrs, d_off, nsys, int(sizes.max()), mode=0, opts=o)
        ms = _timeit(run)
        meas.append(dict(n=int(offs[-1]), m=nsys, opts=c, ms=ms, gunk_s=int(offs[-1]) / ms / 1e6))
        if best is None or ms < best["ms"]:
            best = dict(n=int(offs[-1]), m=nsys, ms=ms, opts=c)
        if verbose:
            print(f"ragged rows={int(offs[-1])} systems={nsys} {c} {ms:.3f} ms", flush=True)
    return meas, [best]


def tune(budget_s: float = 600.0, verbose: bool = True, only=None):
    """Times the candidates of both paths and the ragged plan (or only one:
    "f64", "mixed" or "ragged")."""
    import torch
    t_start = time.time()
    rec = {"device": torch.cuda.get_device_name(0), "f64": [], "mixed": []}
    if only in (None, "ragged"):
        rec["ragged"], rec["ragged_best"] = tune_ragged(verbose)
    for kind, classes, cands, solver in (("f64", F64_CLASSES, list(f64_candidates()), solve_f64),
                                         ("mixed", MP_CLASSES, list(mp_candidates()), solve_mixed)):
        if only is not None and kind != only:
            continue
        for n_max, m in classes:
            n = n_max if n_max <= 131072 else n_max // 2
            arrs = _batch(m, n)
            rhs = arrs[5].clone()
            best = None
            for c in cands:
                if time.time() - t_start > budget_s:
                    break
                o = Opts(**c)

                def run():
                    arrs[5].copy_(rhs)
                    if solver is solve_mixed:
                        solver(*arrs, m, n, opts=o, report=False)
                    else:
                        solver(*arrs, m, n, opts=o)
                try:
                    ms = _timeit(run)
                except Exception as exc:          # a candidate the library refuses
                    rec[kind].append(dict(n=n, m=m, opts=c, error=str(exc)))
                    continue
                rec[kind].append(dict(n=n, m=m, opts=c, ms=ms, gunk_s=m * n / ms / 1e6))
                if best is None or ms < best[0]:
                    best = (ms, c)
                if verbose:
                    print(f"{kind} n={n} m={m} {c} {ms:.3f} ms", flush=True)
            if best is None:
                raise RuntimeError(f"autotune: no {kind} candidate ran for n={n} m={m} (time budget or errors)")
            rec.setdefault(kind + "_best", []).append(dict(n_max=n_max, n=n, m=m, ms=best[0], opts=best[1]))
            del arrs, rhs
            torch.cuda.empty_cache()
    return rec


def header_text(rec) -> str:
    f64 = rec["f64_best"]
    mp = rec["mixed_best"]
    rg = rec["ragged_best"][0]["opts"] if rec.get("ragged_best") else f64[-1]["opts"]
    rows_f = ", \\\n    ".join("{%d, %d, %d, %d, %d}" % (b["n_max"], b["opts"]["smem_rows"], b["opts"]["fuse_strides"],
                                                     b["opts"]["tile_rows"], b["opts"]["threads"]) for b in f64)
    rows_m = ", \\\n    ".join("{%d, %d, %d}" % (b["n_max"], b["opts"]["smem_rows"] // 2, b["opts"]["fuse_strides"])
                            for b in mp)
    return f"""// tuned_params.h -- defaults chosen by the autotuner (pcrp/autotune.py) on {rec['device']}.
// Regenerated by `python -m pcrp.autotune --write`; edit there, not here.
#pragma once
#define PCRP_TUNED_SMEM_ROWS {rg['smem_rows']}     // ragged path: shared-memory capacity (rows)
#define PCRP_TUNED_FUSE_STRIDES {rg['fuse_strides']}     // ragged path: strides fused per global pass
#define PCRP_TUNED_TILE_ROWS {rg['tile_rows']}      // ragged path: rows written per CTA in a global pass
#define PCRP_TUNED_THREADS {rg['threads']}        // threads per CTA
#define PCRP_TUNED_MP_SMEM_BLOCKS {mp[-1]['opts']['smem_rows'] // 2}   // mixed: block rows solved whole in shared memory
#define PCRP_TUNED_MP_FUSE {mp[-1]['opts']['fuse_strides']}            // mixed: FP32 block strides fused per global pass
// FP64 path by system size: {{n_max, smem_rows, fuse_strides, tile_rows, threads}}
#define PCRP_TUNED_F64_TABLE {{ \\
    {rows_f} }}
// mixed path by system size: {{n_max, block rows in shared memory, fuse_strides}}
#define PCRP_TUNED_MP_TABLE {{ \\
    {rows_m} }}
"""


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--json", default=None)
    ap.add_argument("--header", default=os.path.join(CSRC, "tuned_params.h"))
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--budget", type=float, default=600.0)
    ap.add_argument("--only", choices=("f64", "mixed", "ragged"), default=None,
                    help="tune one part; the others' results come from --prev")
    ap.add_argument("--prev", default=None, help="earlier JSON record (with --only)")
    args = ap.parse_args()
    rec = tune(args.budget, only=args.only)
    if args.only:
        if not args.prev:
            ap.error("--only needs --prev, the record that holds the other path's results")
        with open(args.prev) as f:
            prev = json.load(f)
        for other in ("f64", "mixed", "ragged"):
            if other != args.only and other + "_best" in prev:
                rec[other], rec[other + "_best"] = prev[other], prev[other + "_best"]
    if args.json:
        with open(args.json, "w") as f:
            json.dump(rec, f, indent=1)
    text = header_text(rec)
    if args.write:
        with open(args.header, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
