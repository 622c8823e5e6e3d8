"""Ragged batches through pcrp_solve_ragged: one persistent kernel (cached
CUDA graph) over systems of uneven size.  FP64 mode must equal the faithful
per-system solve bit for bit; mixed mode must meet the 1e-12 forward-error
bar against elimination."""
import numpy as np
import pytest

import oracle as O
import pcrp
from helpers import assert_bitexact, dd_bands

pytestmark = pytest.mark.gpu


def ragged_batch(sizes, seed, garbage=True):
    rng = np.random.default_rng(seed)
    parts = [dd_bands(rng, 1, int(s), garbage=garbage) for s in sizes]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    arrs = [np.concatenate([p[k] for p in parts]) for k in range(6)]
    return arrs, offs


def run_ragged(arrs, offs, mode=0, opts=None, dev="cuda:0", **kw):
    import torch
    t = [torch.from_numpy(v).to(dev) for v in arrs]
    o = torch.from_numpy(offs).to(dev)
    sizes = np.diff(offs)
    pcrp.solve_ragged(*t, o, len(sizes), int(sizes.max()), mode=mode, opts=opts, **kw)
    torch.cuda.synchronize()
    return t[5].cpu().numpy()


SIZES = [1, 2, 3, 5, 7, 32, 100, 511, 512, 1000, 1024, 1025, 2048, 3000, 4096, 9000, 65536, 17, 1100]


@pytest.mark.parametrize("opts", [None, dict(smem_rows=64), dict(smem_rows=128, fuse_strides=2, tile_rows=50)])
def test_ragged_f64_bitexact_per_system(cuda, opts):
    arrs, offs = ragged_batch(SIZES, 1)
    x = run_ragged(arrs, offs, 0, pcrp.Opts(**opts) if opts else None)
    xo = O.ragged(*arrs, offs[:-1], np.diff(offs), kind="pcr")
    assert_bitexact(x, xo, f"ragged f64 {opts}")


def test_ragged_f64_log_uniform_sizes_match_uniform_path(cuda):
    import torch
    sizes = pcrp.ragged_sizes(3, 256, 32, 65536)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    arrs = pcrp.generate_ragged(pcrp.GEN_DOMINANT, 3, offs)
    x1 = run_ragged(arrs, offs, 0)
    x2 = run_ragged(arrs, offs, 0)                    # graph replay
    assert np.array_equal(x1, x2)
    for k in range(0, len(sizes), 37):
        sl = slice(offs[k], offs[k + 1])
        t = [torch.from_numpy(np.ascontiguousarray(v[sl])).to(cuda) for v in arrs]
        pcrp.solve_f64(*t, 1, int(sizes[k]))
        torch.cuda.synchronize()
        assert_bitexact(x1[sl], t[5].cpu().numpy(), f"system {k} n={sizes[k]}")


@pytest.mark.parametrize("mode", [0, 1])
def test_ragged_tridiagonal_null_outer_bands(cuda, mode):
    """a = e = NULL: FP64 mode gives the oracle's bits on explicit +0.0 bands,
    mixed mode meets the 1e-12 bar against elimination."""
    import torch
    arrs, offs = ragged_batch(SIZES, 11)
    arrs[0][:] = 0.0
    arrs[4][:] = 0.0
    t = [None if k in (0, 4) else torch.from_numpy(v).to(cuda) for k, v in enumerate(arrs)]
    o = torch.from_numpy(offs).to(cuda)
    sizes = np.diff(offs)
    pcrp.solve_ragged(*t, o, len(sizes), int(sizes.max()), mode=mode)
    torch.cuda.synchronize()
    x = t[5].cpu().numpy()
    if mode == 0:
        assert_bitexact(x, O.ragged(*arrs, offs[:-1], sizes, kind="pcr"), "ragged tridiagonal f64")
    else:
        xr = O.ragged(*arrs, offs[:-1], sizes, kind="ge")
        for k in range(len(sizes)):
            sl = slice(offs[k], offs[k + 1])
            assert O.fwd_err(x[sl], xr[sl], 1, int(sizes[k])) <= 1e-12, f"system {k}"


def test_ragged_rejects_bad_offsets(cuda):
    import torch
    arrs, offs = ragged_batch([5, 6], 2)
    bad = offs.copy(); bad[0] = 1
    with pytest.raises(pcrp.PcrpError) as ei:
        run_ragged(arrs, bad)
    assert ei.value.status == 1
    t = [torch.from_numpy(v).to(cuda) for v in arrs]
    o = torch.from_numpy(offs).to(cuda)
    with pytest.raises(pcrp.PcrpError):
        pcrp.solve_ragged(*t, o, 2, 5)                   # max_rows below a system's size


def test_ragged_wait_timeout_is_reported(cuda):
    """Failure detection: the test hook makes one dependency wait unsatisfiable;
    the bounded wait gives up, the kernel returns, the call reports ETIMEOUT and
    the context stays usable."""
    arrs, offs = ragged_batch([5000, 30], 4)
    with pytest.raises(pcrp.PcrpError) as ei:
        run_ragged(arrs, offs, 0, pcrp.Opts(reserved0=0x7E57))
    assert ei.value.status == 4
    x = run_ragged(arrs, offs, 0)                     # still works afterwards
    assert_bitexact(x, O.ragged(*arrs, offs[:-1], np.diff(offs), kind="pcr"), "after timeout")


def test_ragged_mixed_meets_tolerance(cuda):
    arrs, offs = ragged_batch(SIZES, 5)
    x = run_ragged(arrs, offs, 1)
    xg = O.ragged(*arrs, offs[:-1], np.diff(offs), kind="ge")
    for k in range(len(SIZES)):
        sl = slice(offs[k], offs[k + 1])
        assert O.fwd_err(x[sl], xg[sl], 1, int(SIZES[k])) <= 1e-12, k


def test_ragged_mixed_log_uniform(cuda):
    sizes = pcrp.ragged_sizes(9, 300, 32, 65536)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    arrs = pcrp.generate_ragged(pcrp.GEN_DOMINANT, 9, offs)
    x1 = run_ragged(arrs, offs, 1)
    x2 = run_ragged(arrs, offs, 1)                    # graph replay
    assert np.array_equal(x1, x2)
    xg = O.ragged(*arrs, offs[:-1], sizes, kind="ge")
    worst = max(O.fwd_err(x1[offs[k]:offs[k + 1]], xg[offs[k]:offs[k + 1]], 1, int(sizes[k]))
                for k in range(len(sizes)))
    assert worst <= 1e-12


def test_ragged_mixed_reads_no_slot_outside_a_system(cuda):
    """Mixed mode reads each system in place from the caller's arrays: NaN in
    every band slot that lies outside its system (a_0, a_1, b_0, d_{n-1},
    e_{n-2}, e_{n-1}) must not reach any solution.  Sizes sit on both sides
    of the size-class boundaries (quarter octaves)."""
    sizes = np.array([33, 40, 41, 48, 49, 56, 57, 64, 65, 1025, 1280, 1281, 4097, 5120, 5121, 7000, 8192, 8193, 2, 3],
                     dtype=np.int64)
    arrs, offs = ragged_batch(sizes, 12, garbage=False)
    for k, n in enumerate(sizes):
        o = offs[k]
        arrs[0][o:o + min(2, n)] = np.nan
        arrs[1][o] = np.nan
        arrs[3][o + n - 1] = np.nan
        arrs[4][o + max(n - 2, 0):o + n] = np.nan
    x = run_ragged(arrs, offs, 1)
    assert np.isfinite(x).all()
    clean = [np.nan_to_num(v, nan=0.0) for v in arrs]
    xg = O.ragged(*clean, offs[:-1], sizes, kind="ge")
    for k in range(len(sizes)):
        sl = slice(offs[k], offs[k + 1])
        assert O.fwd_err(x[sl], xg[sl], 1, int(sizes[k])) <= 1e-12, (k, sizes[k])


def test_ragged_mixed_replay_after_workspace_growth(cuda):
    """The cached graph of a ragged batch is tied to the workspace it was
    captured on: a larger solve in between (which grows the shared workspace)
    must lead to a fresh capture, with the same answer."""
    import torch
    sizes = np.array([300, 5000, 40, 70000, 1200], dtype=np.int64)
    arrs, offs = ragged_batch(sizes, 21)
    x1 = run_ragged(arrs, offs, 1)
    x2 = run_ragged(arrs, offs, 1)                    # replay
    rng = np.random.default_rng(5)
    big = [torch.from_numpy(v).to(cuda) for v in dd_bands(rng, 64, 1 << 17)]
    pcrp.solve_mixed(*big, 64, 1 << 17)
    torch.cuda.synchronize()
    x3 = run_ragged(arrs, offs, 1)
    assert np.array_equal(x1, x2) and np.array_equal(x1, x3)


@pytest.mark.parametrize("mode", [0, 1])
def test_ragged_replay_with_offsets_rewritten_in_place(cuda, mode):
    """The same arrays, offsets buffer and caller workspace, the offsets
    rewritten between calls to a batch of more rows in total and back: every
    call solves the batch it is given (a cached launch sequence holds the
    workspace layout of the row count it was captured for, so the row count
    is part of its key)."""
    import torch
    s1 = np.array([300, 5000, 40, 1200], dtype=np.int64)
    s2 = np.array([60000, 5000, 70000, 33], dtype=np.int64)
    max_rows = int(max(s1.max(), s2.max()))
    need = pcrp.workspace_size(len(s1), max_rows, which=2)
    ws = torch.empty(need, dtype=torch.uint8, device=cuda)
    opts = pcrp.Opts(workspace=ws.data_ptr(), workspace_bytes=need)
    t = [torch.zeros(int(s2.sum()), dtype=torch.float64, device=cuda) for _ in range(6)]
    off = torch.empty(len(s1) + 1, dtype=torch.int64, device=cuda)
    for sizes, seed in ((s1, 41), (s2, 42), (s1, 43)):
        arrs, offs = ragged_batch(sizes, seed)
        for u, v in zip(t, arrs):
            u[: len(v)].copy_(torch.from_numpy(v))
        off.copy_(torch.from_numpy(offs))
        pcrp.solve_ragged(*t, off, len(sizes), max_rows, mode=mode, opts=opts)
        torch.cuda.synchronize()
        x = t[5][: int(offs[-1])].cpu().numpy()
        if mode == 0:
            assert_bitexact(x, O.ragged(*arrs, offs[:-1], sizes, kind="pcr"), f"batch {list(sizes)}")
        else:
            xg = O.ragged(*arrs, offs[:-1], sizes, kind="ge")
            for k in range(len(sizes)):
                sl = slice(offs[k], offs[k + 1])
                assert O.fwd_err(x[sl], xg[sl], 1, int(sizes[k])) <= 1e-12, (list(sizes), k)


@pytest.mark.parametrize("mode", [0, 1])
def test_ragged_runs_in_the_workspace_it_asks_for(cuda, mode):
    """A caller-owned workspace of pcrp_workspace_size(nsys, max_rows,
    which=2) bytes is enough for either mode."""
    import torch
    sizes = np.array([33, 1000, 5121, 65536, 7, 40000], dtype=np.int64)
    arrs, offs = ragged_batch(sizes, 31)
    need = pcrp.workspace_size(len(sizes), int(sizes.max()), which=2)
    ws = torch.empty(need, dtype=torch.uint8, device=cuda)
    x = run_ragged(arrs, offs, mode, pcrp.Opts(workspace=ws.data_ptr(), workspace_bytes=need))
    if mode == 0:
        assert_bitexact(x, O.ragged(*arrs, offs[:-1], sizes, kind="pcr"), "caller workspace")
    else:
        xg = O.ragged(*arrs, offs[:-1], sizes, kind="ge")
        for k in range(len(sizes)):
            sl = slice(offs[k], offs[k + 1])
            assert O.fwd_err(x[sl], xg[sl], 1, int(sizes[k])) <= 1e-12


def test_ragged_mixed_reports_unconverged_systems(cuda):
    """Mixed mode with one refinement sweep and an unreachable tolerance:
    PCRP_ENOCONV (status 5), never a false success; the same batch then
    solves to the usual bar with the default settings."""
    sizes = np.array([40, 3000, 70000, 900, 2], dtype=np.int64)
    arrs, offs = ragged_batch(sizes, 41)
    with pytest.raises(pcrp.PcrpError) as ei:
        run_ragged(arrs, offs, 1, tol=1e-30, max_sweeps=1)
    assert ei.value.status == 5
    x = run_ragged(arrs, offs, 1)
    xg = O.ragged(*arrs, offs[:-1], sizes, kind="ge")
    for k in range(len(sizes)):
        sl = slice(offs[k], offs[k + 1])
        assert O.fwd_err(x[sl], xg[sl], 1, int(sizes[k])) <= 1e-12
