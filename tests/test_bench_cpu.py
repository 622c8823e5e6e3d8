"""Host-side pieces of bench.py: stride count and the FP64 operation count
of the roofline, checked against a row-by-row walk of the reference's
stride loop (kernel.cu:63-153)."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def walk(n):
    """Products/sums and divisions of the reference's stride arithmetic, one
    row at a time (nonzero pivots), then the final step."""
    s = bench.ref_strides(n)
    ops = divs = 0
    for k in range(s):
        dl = 1 << k
        for t in range(n):
            hasL, hasR = t - dl >= 0, t + dl <= n - 1
            if hasL and hasR:
                ops += 18
                divs += (t - 2 * dl >= 0) + (t + 2 * dl <= n - 1)
            elif hasR:
                ops += 7
                divs += t + 2 * dl <= n - 1
            elif hasL:
                ops += 7
                divs += t - 2 * dl >= 0
            ops += 8
            if hasL:
                ops += 5
                divs += 1
            if hasR:
                ops += 5
                divs += 1
    df = 1 << s
    if df == n:
        divs += n
    else:
        for t in range(n):
            if t < n - df:
                ops += 9
                divs += 2
            if n - df <= t < df:
                divs += 1
    return ops, divs


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 9, 31, 32, 33, 100, 256, 300, 512, 1000])
def test_fp64_ops_matches_row_walk(n):
    ops, divs = walk(n)
    o, d = bench.fp64_ops(n)
    assert o * n == pytest.approx(ops, abs=1e-6)
    assert d * n == pytest.approx(divs, abs=1e-6)


def test_ref_strides():
    assert [bench.ref_strides(n) for n in (1, 2, 3, 4, 5, 8, 9, 1000, 1024, 1025)] == [0, 1, 1, 2, 2, 3, 3, 9, 10, 10]


def dram_mb(path, names):
    """Sum of the MB figures on the profile table rows whose first cell is
    one of `names` (every column of the row)."""
    tot = 0.0
    with open(path) as f:
        for line in f:
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            if cells and cells[0] in names:
                for c in cells[1:]:
                    for v in c.split("/"):
                        v = v.strip()
                        if v.replace(".", "", 1).isdigit():
                            tot += float(v)
    return tot


# the ncu summaries the bench's traffic table was read from
PROFILES = {("c1", "f64"): "profiles/pcr_pass_kernel_f64_m256_n65536.md",
            ("c1", "mixed"): "profiles/mixed_kernels_m256_n65536.md",
            ("c2", "mixed"): "profiles/mixed_small_kernel_c2_m4096_n4096.md",
            ("c4", "f64"): "profiles/pcr_pass_kernel_f64_m64_n1048576.md",
            ("c4", "mixed"): "profiles/mixed_kernels_m64_n1048576.md"}


@pytest.mark.parametrize("key,col_names,units", [
    (("c1", "f64"), ["dram__bytes_read.sum (MB)", "dram__bytes_write.sum (MB)"], 48 * 65536),
    (("c1", "mixed"), ["dram__bytes_read.sum (MB)", "dram__bytes_write.sum (MB)"], 48 * 65536),
    (("c4", "f64"), ["dram__bytes_read.sum (MB)", "dram__bytes_write.sum (MB)"], 4 << 20),
    (("c4", "mixed"), ["dram__bytes_read.sum (MB)", "dram__bytes_write.sum (MB)"], 4 << 20),
])
def test_measured_traffic_matches_profiles(key, col_names, units):
    """The bench's DRAM bytes per unknown equal the committed captures' sums."""
    per, _ = bench.MEASURED_TRAFFIC[key]
    got = dram_mb(os.path.join(bench.ROOT, PROFILES[key]), col_names) * 1e6 / units
    assert abs(got - per) < 0.5, (got, per)


def test_measured_traffic_c2_matches_profile():
    per, _ = bench.MEASURED_TRAFFIC[("c2", "mixed")]
    with open(os.path.join(bench.ROOT, PROFILES[("c2", "mixed")])) as f:
        row = next(line for line in f if line.startswith("| dram__bytes_read / write (MB)"))
    rd, wr = [float(v) for v in row.split("|")[2].split("/")]   # the current kernel's column
    assert abs((rd + wr) * 1e6 / (1024 * 4096) - per) < 0.5


def test_bench_messages_name_no_files():
    """Printed notes describe captures in words, not by repository paths."""
    for per, note in bench.MEASURED_TRAFFIC.values():
        assert "profiles/" not in note and ".md" not in note


def run_bench(*args, timeout=600):
    import json
    import subprocess
    env = dict(os.environ)
    env.pop("WORLD_SIZE", None)
    out = subprocess.run([sys.executable, os.path.join(bench.ROOT, "bench.py"), *args], capture_output=True,
                         text=True, timeout=timeout, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_config_matches_ours_and_default_is_c4():
    """Both arms print the same config dict; the default workload is the
    largest single-GPU configuration (m=64, n=2^20)."""
    ref = bench.config_dict(bench.CONFIGS["c4"], 1)
    assert ref["m"] == 64 and ref["n"] == 1 << 20 and "solver" not in ref
    import argparse  # noqa: F401
    src = open(os.path.join(bench.ROOT, "bench.py")).read()
    assert 'choices=sorted(CONFIGS), default="c4"' in src
    assert src.count('"config": config_dict(cfg, world)') == 2


def test_reference_arm_two_ranks_one_line():
    """--impl reference --gpus 2 outside torchrun launches two gloo ranks
    itself; rank 0 alone prints one line with n_gpus 2 and never loads the
    product library."""
    lines = run_bench("--impl", "reference", "--config", "c0", "--gpus", "2", "--steps", "1", "--warmup", "3",
                      "--ref-systems", "4")
    assert len(lines) == 1
    ln = lines[0]
    assert ln["impl"] == "reference" and ln["n_gpus"] == 2
    assert ln["config"] == bench.config_dict(bench.CONFIGS["c0"], 2)
    assert ln["e2e"]["h2d_bytes_per_step"] == 0 and ln["cpu_baseline"]["kind"] == "port"


def test_reference_arm_does_not_load_libpcrp():
    """The CPU reference arm generates its inputs with the oracle."""
    import subprocess
    code = ("import sys, runpy; sys.argv=['bench.py','--impl','reference','--config','c0','--steps','1',"
            "'--warmup','3','--ref-systems','2']; runpy.run_path('bench.py', run_name='__main__');"
            "maps=open('/proc/self/maps').read(); print('LOADED' if 'libpcrp.so' in maps else 'CLEAN')")
    out = subprocess.run([sys.executable, "-c", code], cwd=bench.ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().splitlines()[-1] == "CLEAN"


def test_tuned_params_header_is_the_autotuners_output():
    """csrc/tuned_params.h is exactly what `python -m pcrp.autotune --write`
    emits from the committed measurement record profiles/autotune_gb300.json."""
    import json
    sys.path.insert(0, os.path.join(bench.ROOT, "pcr-penta_gb300"))
    from pcrp import autotune
    with open(os.path.join(bench.ROOT, "profiles", "autotune_gb300.json")) as f:
        rec = json.load(f)
    with open(os.path.join(bench.ROOT, "pcr-penta_gb300", "csrc", "tuned_params.h")) as f:
        assert f.read() == autotune.header_text(rec)


def test_autotune_record_best_is_the_fastest_measured():
    """Every size class's chosen plan is the fastest measurement of that class
    in the committed record."""
    import json
    with open(os.path.join(bench.ROOT, "profiles", "autotune_gb300.json")) as f:
        rec = json.load(f)
    for kind in ("f64", "mixed", "ragged"):
        for b in rec.get(kind + "_best", []):
            ms = [r["ms"] for r in rec[kind] if r["n"] == b["n"] and r["m"] == b["m"] and "ms" in r]
            assert ms and b["ms"] == min(ms), (kind, b)


def test_autotune_header_ragged_defaults():
    """The ragged path's defaults come from the record's own ragged search
    when it has one, else from the largest FP64 size class (older records)."""
    import copy
    import json
    sys.path.insert(0, os.path.join(bench.ROOT, "pcr-penta_gb300"))
    from pcrp import autotune
    with open(os.path.join(bench.ROOT, "profiles", "autotune_gb300.json")) as f:
        rec = json.load(f)
    rg = rec["ragged_best"][0]["opts"]
    text = autotune.header_text(rec)
    assert f"#define PCRP_TUNED_SMEM_ROWS {rg['smem_rows']} " in text
    assert f"#define PCRP_TUNED_FUSE_STRIDES {rg['fuse_strides']} " in text
    old = copy.deepcopy(rec)
    old.pop("ragged_best")
    last = old["f64_best"][-1]["opts"]
    assert f"#define PCRP_TUNED_TILE_ROWS {last['tile_rows']} " in autotune.header_text(old)


def test_autotune_mixed_candidates_time_the_general_passes(monkeypatch):
    """The mixed table plans the general block-PCR passes, so every mixed
    candidate runs with the windows off; a size class none of whose
    candidates ran is an error, not a silent gap in the table.  (Timing and
    solves are replaced by fakes: no GPU.)"""
    import types
    sys.path.insert(0, os.path.join(bench.ROOT, "pcr-penta_gb300"))
    from pcrp import autotune
    cands = list(autotune.mp_candidates())
    assert cands and all(c["window_levels"] == -1 for c in cands)
    assert all(c["smem_rows"] // 2 - 2 * ((1 << c["fuse_strides"]) - 1) >= 32 for c in cands)

    fake_torch = types.SimpleNamespace(cuda=types.SimpleNamespace(get_device_name=lambda i: "fake",
                                                                  empty_cache=lambda: None))
    monkeypatch.setitem(sys.modules, "torch", fake_torch)

    class FakeArray:
        def clone(self):
            return self

        def copy_(self, other):
            return self

    monkeypatch.setattr(autotune, "_batch", lambda m, n, seed=1: [FakeArray() for _ in range(6)])
    seen = []

    def timeit(fn, reps=5, warm=1):
        fn()
        return 1.0 + len(seen) * 1e-3
    monkeypatch.setattr(autotune, "_timeit", timeit)
    monkeypatch.setattr(autotune, "solve_mixed", lambda *a, **k: seen.append(k["opts"].window_levels))
    rec = autotune.tune(verbose=False, only="mixed")
    assert set(seen) == {-1} and len(rec["mixed_best"]) == len(autotune.MP_CLASSES)
    assert all(b["ms"] == min(r["ms"] for r in rec["mixed"] if r["n"] == b["n"]) for b in rec["mixed_best"])

    def refuse(*a, **k):
        raise RuntimeError("refused")
    monkeypatch.setattr(autotune, "solve_mixed", refuse)
    with pytest.raises(RuntimeError, match="no mixed candidate ran"):
        autotune.tune(verbose=False, only="mixed")
