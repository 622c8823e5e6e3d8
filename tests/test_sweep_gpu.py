"""The reference-style timing sweep (pcrp.sweep): grid, .dat layout."""
import pytest


@pytest.mark.gpu
def test_sweep_writes_reference_layout(cuda, tmp_path):
    from pcrp import sweep
    out = tmp_path / "t.dat"
    rows = sweep.sweep(["f64", "mixed"], [26, 52], [256, 2048], "toeplitz", runs=2, max_unknowns=52 * 256,
                       out=str(out), verbose=False)
    assert [(m, n) for m, n, _ in rows] == [(26, 256), (26, 2048), (52, 256), (52, 2048)]
    assert all(t is not None and t > 0 for m, n, ts in rows if m * n <= 52 * 256 for t in ts)
    assert rows[1][2] == [None, None] and rows[3][2] == [None, None]      # beyond the bound
    data = [l.split() for l in out.read_text().splitlines() if l[:1].isdigit()]
    assert len(data) == 4 and all(len(d) == 4 for d in data)
    assert data[1][2:] == ["0.000000", "0.000000"]


def test_sweep_grid_is_the_reference_grid():
    from pcrp import sweep
    assert len(sweep.BATCHES) == 17 and sweep.BATCHES[0] == 26 and sweep.BATCHES[-1] == 2080
    assert sweep.SIZES == [256 << k for k in range(10)]
