"""Benchmark of the batched pentadiagonal PCR-Penta solve on GB300.

Default workload: plain FP64 PCR-Penta through pcrp_solve_f64 on m=64
systems of n=2^20 rows (the HBM-filling weakly dominant stress batch, the
largest single-GPU workload), contiguous (reference) layout, inputs resident
in HBM; the FP32+FP64-refinement solver is timed on the same inputs beside
it.  Prints ONE JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config c0|c1|c2|c3|c4] [--solver f64|mixed]

Metric: Gunknowns/s = (systems x rows, all ranks) / device time per step.
A step solves the whole batch once; it first restores the right-hand side
with one device copy (16 B/unknown, named in `roofline.traffic_note`) because the
solve overwrites y.  The inputs (3.2 GB at m=64, n=2^20) exceed the 129 MB
L2, so no L2 flush is needed between steps.

--impl reference times the CPU restatement of the reference's PCR-Penta
algorithm (oracle/, the reference has no CPU path of its own) on every host
core, on a bounded sample of the same workload; its inputs come from the
oracle's own generator, so that arm never loads the product library.

--gpus N without torchrun re-launches this script under
torch.distributed.run with N ranks (one per GPU, 127.0.0.1 rendezvous).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "pcr-penta_gb300"))

METRIC = "Gunknowns/s, % of 8 TB/s HBM; FP32+IR vs FP64 PCR at ≤1e-12 fwd err"
UNIT = "Gunknowns/s"
BYTES_PER_UNKNOWN = 56          # 5 FP64 bands + FP64 rhs read once, FP64 x written once

# DRAM bytes per unknown of one solve (dram__bytes_read.sum +
# dram__bytes_write.sum over the solve's launches) from ncu captures of a
# smaller batch of the same systems (inputs still larger than L2), scaled to
# the bench's batch by unknowns: systems are independent, so the traffic per
# unknown does not depend on m.  Keyed by (config, solver); used only for the
# config's own layout and the autotuned plan.  The capture commands and the
# raw figures are kept with the ncu summaries in the repository's profiles.
MEASURED_TRAFFIC = {
    ("c1", "f64"): (831.0, "ncu capture m=48 n=65536, the 8 pcr_pass_kernel launches of one solve"),
    ("c1", "mixed"): (117.5, "ncu capture m=48 n=65536, mp_first_kernel + mp_try_kernel of one solve"),
    ("c2", "mixed"): (123.0, "ncu capture m=1024 n=4096, the mp_small_kernel launch of one solve"),
    ("c4", "f64"): (747.7, "ncu capture m=4 n=2^20, the 7 pcr_pass_kernel launches of one solve"),
    ("c4", "mixed"): (139.2, "ncu capture m=4 n=2^20, mp_first_kernel + mp_try_kernel of one solve"),
}


def ref_strides(n: int) -> int:
    """Strides PCR-Penta runs on n rows (main.cu:38-39): log2 n for powers of
    two, ceil(log2 n) - 1 otherwise."""
    if n <= 1:
        return 0
    lg = (n - 1).bit_length()
    return lg if (1 << lg) == n else lg - 1


def fp64_ops(n: int):
    """FP64 operations per unknown of the reference's arithmetic on n rows
    (kernel.cu:63-153, the two neighbour combinations shared as T(m)),
    counted row by row with the boundary rows' shorter forms and nonzero
    pivots: phase A 18 products/sums and up to 2 IEEE divisions per interior
    row (7 and up to 1 with one neighbour), phase B 8 sums plus 5 products and
    1 division per neighbour; then x = y/c (powers of two) or the 2x2 pairs
    (9 products/sums and 2 divisions per pair, 1 division per single row)."""
    import numpy as np
    s = ref_strides(n)
    t = np.arange(n, dtype=np.int64)
    ops = divs = 0
    for k in range(s):
        dl = 1 << k
        hasL, hasR = t - dl >= 0, t + dl <= n - 1
        inner, onlyR, onlyL = hasL & hasR, hasR & ~hasL, hasL & ~hasR
        divL, divR = t - 2 * dl >= 0, t + 2 * dl <= n - 1
        ops += 18 * int(inner.sum()) + 7 * int((onlyR | onlyL).sum())
        divs += int((inner & divL).sum()) + int((inner & divR).sum())
        divs += int((onlyR & divR).sum()) + int((onlyL & divL).sum())
        ops += 8 * n + 5 * int(hasL.sum()) + 5 * int(hasR.sum())
        divs += int(hasL.sum()) + int(hasR.sum())
    if n >= 1 and (1 << s) == n:
        divs += n
    else:
        df = 1 << s
        pairs = max(n - df, 0)
        ops += 9 * pairs
        divs += 2 * pairs + max(min(df, n) - pairs, 0)
    return ops / n, divs / n


GENERATORS = {0: "dominant: a,b,d,e ~ U[-1,1], c = sum|off| + U[1,2], y ~ U[-1,1]",
              1: "ADI convection-diffusion (I - theta dt L), theta=0.5, dt=1e-3, r=0.03, payoff rhs",
              2: "weakly dominant: a,b,d,e ~ U[-1,1], c = +-1.05 sum|off|, y ~ U[-1,1]"}
SEED = 7
L2_BYTES = 129 * 1000 * 1000     # GB300 L2 (inputs below twice this are flushed between steps)

CONFIGS = {
    "c0": dict(m=1024, n=512, kind=0, layout="interleaved",
               name="plain FP64 PCR, shared-memory path, m=1024 n=512, interleaved layout"),
    "c1": dict(m=256, n=65536, kind=0, name="plain FP64 PCR, global tile-splitting path, m=256 n=65536"),
    "c2": dict(m=4096, n=4096, kind=1, name="ADI convection-diffusion, m=4096 n=4096"),
    "c4": dict(m=64, n=1 << 20, kind=2, name="weakly dominant, m=64 n=2^20"),
    "c3": dict(m=4096, n=65536, kind=0, ragged=True,
               name="ragged batch: 4096 systems, n log-uniform in [32, 65536], one persistent kernel"),
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.f is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def config_dict(cfg, world):
    """The workload description; both arms (ours, --impl reference) print the
    same dict for the same --config and --gpus."""
    m, n = cfg["m"], cfg["n"]
    small = 48 * m * n < 2 * L2_BYTES
    return {"workload": cfg["name"], "m": m, "n": n, "layout": cfg.get("layout", "contiguous"),
            "generator": GENERATORS[cfg["kind"]], "seed": SEED,
            "l2": (f"inputs ({48 * m * n / 1e6:.0f} MB) smaller than twice L2: a {2 * L2_BYTES / 1e6:.0f} MB "
                   "write between timed steps, each step timed alone") if small else
                  f"inputs larger than L2 ({48 * m * n / 1e9:.2f} GB vs {L2_BYTES / 1e6:.0f} MB), no flush",
            "parallelism": f"replicas x{world} (independent systems per GPU)"}


def relaunch_distributed(args):
    """--gpus N > 1 outside torchrun: run this script again under
    torch.distributed.run with N ranks on this node; returns its exit code."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def dist_setup(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() and args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def cfg_layout(cfg):
    """The workload's batch layout: 1 interleaved (row-major over systems) or 0
    contiguous (the library's and the oracle's layout codes)."""
    return 1 if cfg.get("layout") == "interleaved" else 0


_CPU_INPUTS = {}


def cpu_sample_gunk(cfg, systems: int, min_s: float = 2.0, solver: str = "pcr"):
    """Oracle PCR restatement (or, solver="ge", the FP64 banded Gaussian
    elimination) on `systems` systems of the workload, in its layout, all
    cores; the sample is solved again until min_s seconds of wall time have
    accumulated.  Returns (Gunknowns/s, cores, seconds, repetitions)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    m, n = systems, cfg["n"]
    lay = cfg_layout(cfg)
    key = (cfg["kind"], m, n, lay)
    if key not in _CPU_INPUTS:          # generated once per sample, outside the timing
        _CPU_INPUTS.clear()
        _CPU_INPUTS[key] = O.generate(cfg["kind"], SEED, m, n, lay)
    arrs = _CPU_INPUTS[key]
    cores = os.cpu_count() or 1
    total, reps = 0.0, 0
    while total < min_s or reps == 0:
        t = time.perf_counter()
        if solver == "ge":
            O.ge(*arrs, m, n, lay, threads=cores)
        else:
            O.pcr(*arrs, m, n, lay, threads=cores)
        total += time.perf_counter() - t
        reps += 1
    return reps * m * n / total / 1e9, cores, total, reps


def run_reference(args, world, rank):
    """--impl reference: the CPU restatement of the reference algorithm on the host cores."""
    if rank != 0:
        return
    cfg = CONFIGS[args.config]
    systems = max(1, min(cfg["m"], args.ref_systems))
    vals = []
    cores = os.cpu_count() or 1
    reps = 1
    for k in range(args.warmup + args.steps):
        v, cores, dt, reps = cpu_sample_gunk(cfg, systems, min_s=0.5 if k < args.warmup else 2.0)
        if k >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    sample = (f"{systems} of {cfg['m']} systems (n={cfg['n']}) solved {reps}x (>= 2 s) per step, "
              f"{cores} host threads")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": cfg["m"] * cfg["n"] / value / 1e6,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded counter-based generator)", "impl": "reference",
        "config": config_dict(cfg, world),
        "solver": "CPU restatement of the reference PCR-Penta algorithm (oracle/pcrp_oracle.c), all host threads",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local, pg):
    import numpy as np
    import torch
    import pcrp

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cfg = CONFIGS[args.config]
    m, n = cfg["m"], cfg["n"]
    stream = torch.cuda.Stream(device=dev)
    hbm, peak_kind = peaks()

    # inputs: this rank's shard of systems (weak scaling: m systems per GPU)
    seed = SEED + rank
    lay = cfg_layout(cfg)
    arrs = [torch.empty(m * n, dtype=torch.float64, device=dev) for _ in range(6)]
    with torch.cuda.stream(stream):
        pcrp.generate_device(cfg["kind"], seed, m, n, lay, arrs, stream=stream)
        rhs = arrs[5].clone()
    stream.synchronize()
    opts = pcrp.Opts(**json.loads(args.opts)) if args.opts else None
    solve = (lambda: pcrp.solve_f64(*arrs, m, n, lay, stream=stream, opts=opts)) if args.solver == "f64" else \
        (lambda: pcrp.solve_mixed(*arrs, m, n, lay, stream=stream, report=False, opts=opts))

    def first_systems(v, k):
        """The first k systems of a batch array, contiguous (for host checks)."""
        return v[: k * n] if lay == pcrp.CONTIGUOUS else v.view(n, m).t()[:k].contiguous().view(-1)

    def step():
        arrs[5].copy_(rhs, non_blocking=True)
        solve()

    def barrier():
        if pg is not None:
            pg.barrier()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    stream.synchronize()
    launches0 = pcrp.kernel_launches()
    barrier()
    torch.cuda.synchronize(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    # inputs that fit in L2 are flushed between timed steps (a write larger
    # than L2), each step then timed alone
    l2 = max(torch.cuda.get_device_properties(dev).L2_cache_size, L2_BYTES)
    small = 48 * m * n < 2 * L2_BYTES
    flush = torch.empty(2 * l2 // 4 + 1024, dtype=torch.float32, device=dev) if small else None
    step_ms = []
    with ClockSampler(local) as clk:
        time.sleep(0.3)
        with torch.cuda.stream(stream):
            if small:
                for _ in range(args.steps):
                    flush.zero_()
                    ev0.record(stream)
                    step()
                    ev1.record(stream)
                    ev1.synchronize()
                    step_ms.append(ev0.elapsed_time(ev1))
            else:
                ev0.record(stream)
                for _ in range(args.steps):
                    step()
                ev1.record(stream)
        ev1.synchronize()
        time.sleep(0.1)
    torch.cuda.synchronize(dev)
    barrier()
    launches = pcrp.kernel_launches() - launches0
    ms = sum(step_ms) / args.steps if small else ev0.elapsed_time(ev1) / args.steps
    if pg is not None:
        t = torch.tensor([ms], dtype=torch.float64, device=dev if pg.get_backend() == "nccl" else "cpu")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    value = world * m * n / (ms * 1e-3) / 1e9

    # kernel-only time of one solve (no RHS restore), for the roofline
    ek0 = torch.cuda.Event(enable_timing=True)
    ek1 = torch.cuda.Event(enable_timing=True)
    kms = []
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.steps)):
            arrs[5].copy_(rhs, non_blocking=True)
            if small:
                flush.zero_()
            ek0.record(stream)
            solve()
            ek1.record(stream)
            ek1.synchronize()
            kms.append(ek0.elapsed_time(ek1))
    kms_med = statistics.median(kms)
    achieved = BYTES_PER_UNKNOWN * m * n / (kms_med * 1e-3) / 1e9

    # accuracy of the headline solve: x of one solve, its normwise residual
    # ||y - A x||_inf / (||A||_inf ||x||_inf) per system on the GPU (worst
    # system), and (below, with the host oracle) its forward error
    with torch.cuda.stream(stream):
        arrs[5].copy_(rhs, non_blocking=True)
        solve()
        x_head = arrs[5].clone()
        r_head = torch.empty_like(x_head)
        pcrp.residual_f64(*arrs[:5], rhs, x_head, r_head, m, n, lay, stream=stream)
    stream.synchronize()

    def per_sys(v):
        return v.view(m, n) if lay == pcrp.CONTIGUOUS else v.view(n, m).t()
    a_norm = sum(per_sys(v).abs() for v in arrs[:5]).amax(dim=1)
    resid = float((per_sys(r_head).abs().amax(dim=1) /
                   (a_norm * per_sys(x_head).abs().amax(dim=1)).clamp_min(1e-300)).max())
    x_head16 = first_systems(x_head, min(m, 16)).cpu().numpy()
    del r_head, x_head

    # FP64-pipe roofline of the faithful path: its FP64 operations at this
    # GPU's measured DFMA and division rates, against the kernel time
    fp64_roof = None
    if args.solver == "f64":
        dfma, ddiv = pcrp.measure_fp64(stream)
        ops, divs = fp64_ops(n)
        t_peak = m * n * (ops / dfma + divs / ddiv)
        fp64_roof = {"bound": "fp64", "ops": "reference", "ops_per_unknown": round(ops, 2),
                     "divisions_per_unknown": round(divs, 3),
                     "dfma_per_s": dfma, "ddiv_per_s": ddiv,
                     "ms_at_peak": t_peak * 1e3, "frac": t_peak / (kms_med * 1e-3),
                     "note": "the reference's FP64 products/sums (exact count on n rows) at the measured "
                             "DFMA rate plus its IEEE divisions at the measured division rate "
                             "(pcrp_measure_fp64), over the solve's kernel time; the kernels form "
                             "operations with a zero operand (late strides, once a and e have "
                             "underflowed) on the integer pipe and finish two quotients from one shared "
                             "reciprocal, so frac is the rate of the reference's operations, not the "
                             "FP64 pipe's busy share (ncu reports that)"}

    # end to end through the public API with host buffers (pinned): pcrp_solve_host
    # (measured before the comparison legs: a long cuSPARSE run leaves the
    # GPU slower for a while, which is no property of this path)
    # copies each step's six input arrays in and the solution out, in chunks
    # that overlap the solves; y is solved in place (the next step's rhs is the
    # previous solution, same work)
    h_in = [torch.empty(m * n, dtype=torch.float64, pin_memory=True) for _ in range(6)]
    pcrp.generate_into(cfg["kind"], seed, m, n, lay, h_in)
    e_steps = max(2, min(args.steps, 5))
    precision = 0 if args.solver == "f64" else 1

    def e2e_step():
        pcrp.solve_host(*h_in, m, n, lay, precision=precision, stream=stream)

    with torch.cuda.stream(stream):
        e2e_step()
    stream.synchronize()
    barrier()
    # each step ends with the host holding y (it waits for the copy out), so
    # the next step's copies do not overlap this step's solve
    ee0 = torch.cuda.Event(enable_timing=True)
    ee1 = torch.cuda.Event(enable_timing=True)
    e_list = []
    with ClockSampler(local) as e_clk:
        with torch.cuda.stream(stream):
            for _ in range(e_steps):
                ee0.record(stream)
                e2e_step()
                ee1.record(stream)
                ee1.synchronize()
                e_list.append(ee0.elapsed_time(ee1))
    e_ms = sum(e_list) / e_steps
    if pg is not None:
        t = torch.tensor([e_ms], dtype=torch.float64, device=dev if pg.get_backend() == "nccl" else "cpu")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e_ms = float(t.item())
    e2e_val = world * m * n / (e_ms * 1e-3) / 1e9

    # comparison legs (cuSPARSE, the other layout) time at most 5 solves: one
    # cuSPARSE solve of the m=64 n=2^20 batch takes ~6 s
    cmp_reps = min(max(3, args.steps), 5)

    # the other precision on the same inputs: FP32 PCR + FP64 refinement when the
    # headline is plain FP64 (and the reverse), for the mixed/FP64 speed ratio
    other = None
    if args.compare:
        other_solver = "mixed" if args.solver == "f64" else "f64"
        osolve = (lambda: pcrp.solve_mixed(*arrs, m, n, lay, stream=stream, report=False)) if other_solver == "mixed" \
            else (lambda: pcrp.solve_f64(*arrs, m, n, lay, stream=stream))
        oms = []
        with torch.cuda.stream(stream):
            for it in range(max(3, args.steps) + 2):
                arrs[5].copy_(rhs, non_blocking=True)
                if small:
                    flush.zero_()
                ek0.record(stream)
                osolve()
                ek1.record(stream)
                ek1.synchronize()
                if it >= 2:
                    oms.append(ek0.elapsed_time(ek1))
        other = {"solver": other_solver, "ms_per_solve": statistics.median(oms),
                 "value": world * m * n / (statistics.median(oms) * 1e-3) / 1e9}
        # mixed: the library's own report (sweeps, estimate, final residual) on one solve
        with torch.cuda.stream(stream):
            arrs[5].copy_(rhs, non_blocking=True)
            info = pcrp.solve_mixed(*arrs, m, n, lay, stream=stream, report=True)
        other["mixed_report"] = {"sweeps": info.sweeps, "converged": info.converged,
                                 "fwd_err_est": info.fwd_err_est, "resid": info.resid}
        x_mixed = first_systems(arrs[5], min(m, 16)).cpu().numpy()
        other["ratio_mixed_over_f64"] = (other["value"] / (world * m * n / (kms_med * 1e-3) / 1e9)
                                         if other_solver == "mixed" else
                                         (world * m * n / (kms_med * 1e-3) / 1e9) / other["value"])

    # library comparison point: cuSPARSE gpsvInterleavedBatch (QR, FP64) on the
    # same systems in the interleaved layout it requires (the transposes and the
    # fresh band copies it needs, since it overwrites them, are outside the timing)
    lib_cmp = None
    if args.cusparse:
        import pcrp.compare as cmpmod
        inter = ([v.view(m, n).t().contiguous().view(-1) for v in arrs[:5]] + [rhs.view(m, n).t().contiguous().view(-1)]
                 if lay == pcrp.CONTIGUOUS else list(arrs[:5]) + [rhs])
        work = [torch.empty_like(v) for v in inter]
        import ctypes
        L = cmpmod.lib()
        nbytes = ctypes.c_size_t(0)
        L.cmp_gpsv_buffer_size(*[w.data_ptr() for w in work], n, m, ctypes.byref(nbytes))
        gbuf = torch.empty(max(1, int(nbytes.value)), dtype=torch.uint8, device=dev)
        gms = []
        with torch.cuda.stream(stream):
            for it in range(cmp_reps + 1):
                for w, v in zip(work, inter):
                    w.copy_(v, non_blocking=True)
                ek0.record(stream)
                rc = L.cmp_gpsv_solve(*[w.data_ptr() for w in work], n, m, gbuf.data_ptr(), stream.cuda_stream)
                ek1.record(stream)
                ek1.synchronize()
                if rc:
                    raise RuntimeError(f"cusparseDgpsvInterleavedBatch status {rc}")
                if it >= 1:
                    gms.append(ek0.elapsed_time(ek1))
        lib_cmp = {"library": "cuSPARSE cusparseDgpsvInterleavedBatch (FP64, interleaved layout)",
                   "ms_per_solve": statistics.median(gms),
                   "value": world * m * n / (statistics.median(gms) * 1e-3) / 1e9}
        x_gpsv = work[5].view(n, m).t()[: min(m, 16)].contiguous().view(-1).cpu().numpy()
        del inter, work, gbuf

    # the headline solver on the same systems in the other batch layout
    # (contiguous <-> interleaved), and whether its solution has the same bits
    alt_layout = None
    if args.other_layout:
        alt_lay = pcrp.INTERLEAVED if lay == pcrp.CONTIGUOUS else pcrp.CONTIGUOUS

        def relayout(v):
            return (v.view(m, n).t() if lay == pcrp.CONTIGUOUS else v.view(n, m).t()).contiguous().view(-1)
        alt = [relayout(v) for v in arrs[:5]] + [torch.empty_like(rhs)]
        alt_rhs = relayout(rhs)
        asolve = (lambda: pcrp.solve_f64(*alt, m, n, alt_lay, stream=stream, opts=opts)) if args.solver == "f64" \
            else (lambda: pcrp.solve_mixed(*alt, m, n, alt_lay, stream=stream, report=False, opts=opts))
        ams = []
        with torch.cuda.stream(stream):
            for it in range(cmp_reps + 1):
                alt[5].copy_(alt_rhs, non_blocking=True)
                if small:
                    flush.zero_()
                ek0.record(stream)
                asolve()
                ek1.record(stream)
                ek1.synchronize()
                if it >= 1:
                    ams.append(ek0.elapsed_time(ek1))
        x_alt = (alt[5].view(m, n) if alt_lay == pcrp.CONTIGUOUS else alt[5].view(n, m).t())[: min(m, 16)]
        same = bool(torch.equal(x_alt.contiguous().view(-1).cpu().view(torch.int64),
                                torch.from_numpy(x_head16).view(torch.int64)))
        alt_layout = {"layout": "interleaved" if alt_lay == pcrp.INTERLEAVED else "contiguous",
                      "ms_per_solve": statistics.median(ams),
                      "value": world * m * n / (statistics.median(ams) * 1e-3) / 1e9,
                      "same_bits_as_headline": same, "checked": f"first {min(m, 16)} systems"}
        del alt, alt_rhs


    if rank != 0:
        return
    # measured DRAM traffic of one solve (bytes), where a capture exists
    mt = MEASURED_TRAFFIC.get((args.config, args.solver))
    if mt is not None and not args.opts and "layout" not in cfg:
        traffic = mt[0] * m * n
        traffic_note = (f"bytes per solve: {mt[0]} B/unknown x {m * n} unknowns, {mt[1]}; "
                        f"each timed step also restores y (one device copy, 16 B/unknown of traffic)")
    else:
        traffic = None
        traffic_note = "no ncu capture of this workload; each timed step also restores y (one device copy)"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.solver == "f64" else "f32+f64",
        "data": "synthetic (seeded counter-based generator, generated on device)",
        "config": config_dict(cfg, world),
        "solver": "pcrp_solve_f64 (bit-faithful PCR-Penta)" if args.solver == "f64"
                  else "pcrp_solve_mixed (FP32 block PCR + FP64 refinement)",
        "gpu_launches": launches,
        "opts": json.loads(args.opts) if args.opts else "autotuned defaults",
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 6 * 8 * m * n,
                "d2h_bytes_per_step": 8 * m * n, "ms_per_step": e_ms,
                "timing": f"pcrp_solve_host on pinned host buffers, each of {e_steps} steps timed alone "
                          "(copies in, solve, copy out; the host waits for y before the next step)",
                "clocks": e_clk.summary()},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "traffic_note": traffic_note,
                     "note": f"algorithmic {BYTES_PER_UNKNOWN} B/unknown over the solve's kernel time "
                             f"({kms_med:.3f} ms); peak {peak_kind}"},
        "clocks": clk.summary(),
    }
    if small and step_ms:
        # steps timed one at a time (after an L2 flush): their spread beside the mean
        q = sorted(step_ms)
        line["step_ms_spread"] = {"min": q[0], "median": statistics.median(q), "max": q[-1]}
    line["accuracy"] = {"resid": resid, "resid_sample": f"all {m} systems, worst system"}
    if fp64_roof is not None:
        line["fp64_roofline"] = fp64_roof
    if other is not None:
        line["compare"] = other
    if lib_cmp is not None:
        line["library_baseline"] = lib_cmp
    if alt_layout is not None:
        line["other_layout"] = alt_layout
    if args.cpu_baseline and world == 1:
        # forward error of the headline solve and of the comparison points
        # against FP64 banded elimination on the first systems
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        ms = min(m, 16)
        host = pcrp.generate(cfg["kind"], seed, ms, n)
        x_ge = O.ge(*host, ms, n)
        xg64 = np.asarray(x_ge, dtype=np.float64).reshape(ms, n)
        xh64 = np.asarray(x_head16, dtype=np.float64).reshape(ms, n)
        line["accuracy"]["fwd_err_vs_ge"] = float((np.abs(xh64 - xg64).max(axis=1) /
                                                   np.maximum(np.abs(xg64).max(axis=1), 1e-300)).max())
        line["accuracy"]["fwd_err_sample"] = f"first {ms} systems vs FP64 banded elimination (oracle)"
        if other is not None:
            xm64 = np.asarray(x_mixed, dtype=np.float64).reshape(ms, n)
            line["compare"]["fwd_err_vs_ge"] = float((np.abs(xm64 - xg64).max(axis=1) /
                                                      np.maximum(np.abs(xg64).max(axis=1), 1e-300)).max())
            line["compare"]["fwd_err_sample"] = f"first {ms} systems vs FP64 banded elimination"
        if lib_cmp is not None:
            xc64 = np.asarray(x_gpsv, dtype=np.float64).reshape(ms, n)
            line["library_baseline"]["fwd_err_vs_ge"] = float((np.abs(xc64 - xg64).max(axis=1) /
                                                               np.maximum(np.abs(xg64).max(axis=1), 1e-300)).max())
        v, cores, dt, reps = cpu_sample_gunk(cfg, min(m, args.ref_systems))
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{min(m, args.ref_systems)} of {m} systems (n={n}) solved {reps}x, "
                                          f"oracle PCR restatement, {dt:.2f} s wall"}
        # the FP64 host solver the accuracy is judged against: banded
        # Gaussian elimination, threads over systems (a reported baseline)
        gv, gcores, gdt, greps = cpu_sample_gunk(cfg, min(m, args.ref_systems), solver="ge")
        line["host_ge"] = {"value": gv, "unit": UNIT, "cores": gcores,
                           "sample": f"{min(m, args.ref_systems)} of {m} systems (n={n}) solved {greps}x, "
                                     f"FP64 banded Gaussian elimination (oracle), {gdt:.2f} s wall"}
    print(json.dumps(line), flush=True)


def run_ragged_bench(args, world, rank, local, pg):
    """Ragged batch (4096 systems, log-uniform sizes 32..65536) through
    pcrp_solve_ragged (FP64 and mixed) against
    the per-size sequence of launches (one pcrp_solve_f64 call per system)."""
    import numpy as np
    import torch
    import pcrp

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cfg = CONFIGS[args.config]
    seed = SEED + rank
    sizes = pcrp.ragged_sizes(seed, cfg["m"], 32, 65536)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    total = int(offs[-1])
    host = pcrp.generate_ragged(cfg["kind"], seed, offs)
    arrs = [torch.from_numpy(v).to(dev) for v in host]
    rhs = arrs[5].clone()
    d_off = torch.from_numpy(offs).to(dev)
    nmax = int(sizes.max())
    stream = torch.cuda.current_stream(dev)

    def timed(fn, steps, warm):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(warm):
            arrs[5].copy_(rhs)
            fn()
        out = []
        for _ in range(steps):
            arrs[5].copy_(rhs)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return statistics.median(out)

    l0 = pcrp.kernel_launches()
    f64_ms = timed(lambda: pcrp.solve_ragged(*arrs, d_off, len(sizes), nmax, mode=0), args.steps, args.warmup)
    launches = (pcrp.kernel_launches() - l0) // (args.steps + args.warmup)
    mixed_ms = timed(lambda: pcrp.solve_ragged(*arrs, d_off, len(sizes), nmax, mode=1), args.steps, args.warmup)
    views = [[v[offs[k]:offs[k + 1]] for v in arrs] for k in range(len(sizes))]

    def per_system():
        for k in range(len(sizes)):
            pcrp.solve_f64(*views[k], 1, int(sizes[k]))
    l1 = pcrp.kernel_launches()
    seq_ms = timed(per_system, max(1, args.steps // 2), 1)
    seq_launches = (pcrp.kernel_launches() - l1) // (max(1, args.steps // 2) + 1)
    if rank != 0:
        return
    value = world * total / (f64_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": f64_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded counter-based generator)",
        "config": {"workload": cfg["name"], "systems": len(sizes), "total_rows": total,
                   "n_min": int(sizes.min()), "n_max": nmax, "layout": "contiguous (ragged offsets)",
                   "solver": "pcrp_solve_ragged mode 0 (bit-faithful PCR-Penta, persistent kernel)"},
        "gpu_launches": launches,
        "per_size_launch_sequence": {"value": world * total / (seq_ms * 1e-3) / 1e9, "ms_per_step": seq_ms,
                                     "gpu_launches": seq_launches,
                                     "note": "pcrp_solve_f64 called once per system"},
        "mixed": {"value": world * total / (mixed_ms * 1e-3) / 1e9, "ms_per_step": mixed_ms,
                  "solver": "pcrp_solve_ragged mode 1 (FP32 block PCR + FP64 refinement)"},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="c4")
    ap.add_argument("--solver", choices=["f64", "mixed"], default="f64")
    ap.add_argument("--ref-systems", type=int, default=64)
    ap.add_argument("--m", type=int, default=0, help="override the number of systems (profiling runs)")
    ap.add_argument("--opts", default="", help='tuning overrides as JSON, e.g. {"smem_rows": 1024}')
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-cusparse", dest="cusparse", action="store_false",
                    help="skip timing cuSPARSE gpsvInterleavedBatch on the same systems")
    ap.add_argument("--no-other-layout", dest="other_layout", action="store_false",
                    help="skip the headline solver on the same systems in the other batch layout")
    ap.add_argument("--no-compare", dest="compare", action="store_false",
                    help="skip timing the other precision on the same inputs")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.m > 0:
        CONFIGS[args.config] = dict(CONFIGS[args.config], m=args.m)
        CONFIGS[args.config]["name"] += f" (m overridden to {args.m})"
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_distributed(args))
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif CONFIGS[args.config].get("ragged"):
        run_ragged_bench(args, world, rank, local, pg)
    else:
        run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
