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


@pytest.mark.parametrize("key,col_names,units", [
    (("c1", "f64"), ["dram__bytes_read.sum (MB)", "dram__bytes_write.sum (MB)"], 48 * 65536),
    (("c1", "mixed"), ["dram__bytes_read.sum (MB)", "dram__bytes_write.sum (MB)"], 48 * 65536),
])
def test_measured_traffic_matches_profiles(key, col_names, units):
    """The bench's DRAM bytes per unknown equal the committed captures' sums."""
    per, note = bench.MEASURED_TRAFFIC[key]
    prof = os.path.join(bench.ROOT, note.split("(")[-1].rstrip(")"))
    got = dram_mb(prof, col_names) * 1e6 / units
    assert abs(got - per) < 0.5, (got, per)


def test_measured_traffic_c2_matches_profile():
    per, note = bench.MEASURED_TRAFFIC[("c2", "mixed")]
    prof = os.path.join(bench.ROOT, note.split("(")[-1].rstrip(")"))
    with open(prof) as f:
        row = next(line for line in f if line.startswith("| dram__bytes_read / write (MB)"))
    rd, wr = [float(v) for v in row.split("|")[2].split("/")]   # the current kernel's column
    assert abs((rd + wr) * 1e6 / (1024 * 4096) - per) < 0.5
