"""GPU tests of the mixed-precision solver (FP32 2x2-block PCR + FP64
refinement) against the FP64 elimination oracle.

Bar (the solver's contract): relative forward error <= 1e-12 against the FP64
banded Gaussian elimination on diagonally dominant systems, bands untouched,
and an honest report (sweeps, estimate, residual)."""
import numpy as np
import pytest

import oracle as O
import pcrp
from helpers import dd_bands, to_device, to_layout

pytestmark = pytest.mark.gpu
TOL = 1e-12


def run_mixed(arrs, m, n, layout=pcrp.CONTIGUOUS, dev="cuda:0", **kw):
    import torch
    t = to_device(arrs, dev)
    info = pcrp.solve_mixed(*t, m, n, layout, **kw)
    torch.cuda.synchronize()
    return t[5].cpu().numpy(), info, t


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 31, 100, 512, 1000, 1024, 2047, 4096, 5001])
@pytest.mark.parametrize("layout", [pcrp.CONTIGUOUS, pcrp.INTERLEAVED])
def test_mixed_dominant_meets_tolerance(cuda, n, layout):
    m = 6
    arrs = to_layout(dd_bands(np.random.default_rng(n), m, n, garbage=True), m, n, layout)
    x, info, _ = run_mixed(arrs, m, n, layout)
    xg = O.ge(*arrs, m, n, layout)
    assert O.fwd_err(x, xg, m, n, layout) <= TOL
    assert info.converged == 1 and 1 <= info.sweeps <= 4
    # residual of the FP64 answer relative to |A||x|: a few hundred ulps at most
    assert info.resid < 1e-13


@pytest.mark.parametrize("kind,m,n", [
    (pcrp.GEN_DOMINANT, 64, 512), (pcrp.GEN_DOMINANT, 4, 65536), (pcrp.GEN_ADI, 32, 4096),
    (pcrp.GEN_WEAK, 8, 8192), (pcrp.GEN_WEAK, 2, 1 << 20), (pcrp.GEN_DOMINANT, 3, 1 << 20),
])
def test_mixed_benchmark_generators(cuda, kind, m, n):
    arrs = pcrp.generate(kind, 17, m, n)
    x, info, _ = run_mixed(arrs, m, n)
    xg = O.ge(*arrs, m, n)
    assert O.fwd_err(x, xg, m, n) <= TOL, (info.sweeps, info.fwd_err_est)
    assert info.converged == 1


@pytest.mark.parametrize("opts", [
    dict(smem_rows=64), dict(smem_rows=64, window_levels=2), dict(smem_rows=64, window_levels=7),
    dict(smem_rows=64, window_levels=-1), dict(smem_rows=64, fuse_strides=2, window_levels=-1),
    dict(smem_rows=8, fuse_strides=1, window_levels=-1)])
def test_mixed_forced_global_passes(cuda, opts):
    """Systems larger than the shared-memory tile: the windowed cyclic
    reduction (any depth; too shallow a window leaves the systems coupled and
    hands them to the block-PCR passes) and the block-PCR passes alone."""
    m, n = 3, 3000
    arrs = dd_bands(np.random.default_rng(7), m, n)
    x, info, _ = run_mixed(arrs, m, n, opts=pcrp.Opts(**opts))
    assert O.fwd_err(x, O.ge(*arrs, m, n), m, n) <= TOL
    assert info.converged == 1


@pytest.mark.parametrize("n", [4097, 16384, 40000])
def test_mixed_batch_of_decoupling_and_coupled_systems(cuda, n):
    """One batch where the windowed cyclic reduction decouples some systems
    (dominant) and leaves others coupled (ADI: its couplings need ~10 levels
    to vanish); the latter go through the block-PCR passes in the same sweeps."""
    dom = pcrp.generate(pcrp.GEN_DOMINANT, 3, 2, n)
    adi = pcrp.generate(pcrp.GEN_ADI, 4, 2, n)
    arrs = [np.concatenate([np.asarray(u), np.asarray(v)]) for u, v in zip(dom, adi)]
    m = 4
    x, info, _ = run_mixed(arrs, m, n, max_sweeps=16)
    assert info.converged == 1
    xt = O.ge(*arrs, m, n)
    for _ in range(2):
        xt = xt + O.ge(*arrs[:5], O.residual(*arrs, xt, m, n), m, n)
    # dominant systems to the solver's bar; the ADI ones (condition up to
    # ~1e5 at these sizes) to the bar of the ill-conditioned ADI test
    assert O.fwd_err(x[: 2 * n], xt[: 2 * n], 2, n) <= TOL
    assert O.fwd_err(x[2 * n:], xt[2 * n:], 2, n) <= 1e-11


def test_mixed_ill_conditioned_adi(cuda):
    """ADI at n = 65536: entries reach ~1e6 against a unit dominance margin
    (condition ~1e6), so FP32 corrections contract slowly (rho ~ 1e-2) and take
    several sweeps; the refinement must still get there.  FP64 elimination is
    itself only good to ~cond*eps here, so it is refined with long-double
    residuals to give the reference answer."""
    m, n = 4, 65536
    arrs = pcrp.generate(pcrp.GEN_ADI, 17, m, n)
    x, info, _ = run_mixed(arrs, m, n, max_sweeps=16)
    assert info.converged == 1 and info.sweeps >= 3
    xt = O.ge(*arrs, m, n)
    for _ in range(3):
        xt = xt + O.ge(*arrs[:5], O.residual(*arrs, xt, m, n), m, n)
    assert O.fwd_err(x, xt, m, n) <= 1e-11


def test_mixed_solves_what_the_reference_algorithm_cannot(cuda):
    """Exact zeros among the off-diagonals break PCR-Penta's pivots
    (kernel.cu:72-75); the block pivots of the mixed solver do not care."""
    rng = np.random.default_rng(5)
    m, n = 3, 256
    a, b, d, e = [rng.integers(-8, 9, (m, n)) / 8.0 for _ in range(4)]
    a[:, :2] = 0; b[:, :1] = 0; d[:, -1:] = 0; e[:, -2:] = 0
    c = np.abs(a) + np.abs(b) + np.abs(d) + np.abs(e) + 1.0
    xt = rng.integers(-64, 65, (m, n)).astype(np.float64)
    y = c * xt
    y[:, 2:] += a[:, 2:] * xt[:, :-2]; y[:, 1:] += b[:, 1:] * xt[:, :-1]
    y[:, :-1] += d[:, :-1] * xt[:, 1:]; y[:, :-2] += e[:, :-2] * xt[:, 2:]
    arrs = [v.ravel().copy() for v in (a, b, c, d, e, y)]
    x, info, _ = run_mixed(arrs, m, n)
    assert O.fwd_err(x, xt.ravel(), m, n) <= TOL
    assert O.fwd_err(O.pcr(*arrs, m, n), xt.ravel(), m, n) > 1e-3


def test_mixed_async_equals_reported(cuda):
    import torch
    m, n = 5, 9000
    arrs = dd_bands(np.random.default_rng(9), m, n)
    x1, info, _ = run_mixed(arrs, m, n)
    t = to_device(arrs, cuda)
    pcrp.solve_mixed(*t, m, n, report=False)
    torch.cuda.synchronize()
    x2 = t[5].cpu().numpy()
    assert O.fwd_err(x2, O.ge(*arrs, m, n), m, n) <= TOL
    assert O.fwd_err(x1, x2, m, n) <= TOL


def test_mixed_reports_nonconvergence(cuda):
    m, n = 2, 700
    arrs = dd_bands(np.random.default_rng(3), m, n)
    with pytest.raises(pcrp.PcrpError) as ei:
        run_mixed(arrs, m, n, max_sweeps=1)
    assert ei.value.status == 5


def test_mixed_leaves_bands_untouched(cuda):
    import torch
    m, n = 3, 5000
    arrs = dd_bands(np.random.default_rng(4), m, n)
    t = to_device(arrs, cuda)
    before = [v.clone() for v in t[:5]]
    pcrp.solve_mixed(*t, m, n)
    torch.cuda.synchronize()
    for u, v in zip(before, t[:5]):
        assert torch.equal(u, v)


@pytest.mark.parametrize("layout", [pcrp.CONTIGUOUS, pcrp.INTERLEAVED])
def test_residual_f64_matches_oracle(cuda, layout):
    import torch
    m, n = 4, 777
    arrs = to_layout(dd_bands(np.random.default_rng(2), m, n, garbage=True), m, n, layout)
    x = np.random.default_rng(3).uniform(-1, 1, m * n)
    t = to_device(arrs + [x, np.zeros(m * n)], cuda)
    pcrp.residual_f64(*t[:6], t[6], t[7], m, n, layout)
    torch.cuda.synchronize()
    r = t[7].cpu().numpy()
    ro = O.residual(*arrs, x, m, n, layout)
    scale = np.abs(arrs[2]).max() * np.abs(x).max()
    assert np.abs(r - ro).max() <= 8 * np.finfo(float).eps * scale


def test_mixed_unaligned_arrays(cuda):
    """Arrays that start 8 bytes past a 16-byte boundary take the scalar load path."""
    import torch
    m, n = 4, 2000
    arrs = dd_bands(np.random.default_rng(31), m, n)
    bufs = [torch.empty(m * n + 1, dtype=torch.float64, device=cuda) for _ in range(6)]
    views = [b[1:] for b in bufs]
    for v, h in zip(views, arrs):
        v.copy_(torch.from_numpy(h))
    assert views[0].data_ptr() % 16 == 8
    pcrp.solve_mixed(*views, m, n)
    torch.cuda.synchronize()
    assert O.fwd_err(views[5].cpu().numpy(), O.ge(*arrs, m, n), m, n) <= TOL


@pytest.mark.parametrize("kind,m,n", [(pcrp.GEN_DOMINANT, 16, 512), (pcrp.GEN_DOMINANT, 4, 65536),
                                      (pcrp.GEN_ADI, 8, 4096), (pcrp.GEN_ADI, 2, 20000)])
def test_mixed_graph_driven_sweeps_match_host_driven(cuda, kind, m, n, monkeypatch):
    """Repeated calls with one argument set run the sweeps as a CUDA graph
    with a device-side while loop (from the second call on); the results are
    bit-identical to the host-driven launches and every call converges."""
    import torch
    arrs = [torch.as_tensor(np.asarray(v)).cuda() for v in pcrp.generate(kind, 5, m, n)]
    rhs = arrs[5].clone()
    monkeypatch.setenv("PCRP_NO_GRAPH", "1")
    pcrp.solve_mixed(*arrs, m, n, max_sweeps=16, report=False)
    torch.cuda.synchronize()
    host = arrs[5].clone()
    monkeypatch.delenv("PCRP_NO_GRAPH")
    for _ in range(3):
        arrs[5].copy_(rhs)
        pcrp.solve_mixed(*arrs, m, n, max_sweeps=16, report=False)
        torch.cuda.synchronize()
        assert torch.equal(arrs[5], host)
    xg = O.ge(*[v.cpu().numpy() for v in arrs[:5]], rhs.cpu().numpy(), m, n)
    assert O.fwd_err(host.cpu().numpy(), xg, m, n) <= (TOL if kind == pcrp.GEN_DOMINANT else 1e-11)


@pytest.mark.parametrize("n", [7, 512, 5000, 65536])
def test_mixed_tridiagonal_null_outer_bands(cuda, n):
    """a = e = NULL: a tridiagonal batch (the outer bands are neither read nor
    multiplied); same answers as passing zero bands, to the solver's bar."""
    import torch
    m = 4
    rng = np.random.default_rng(n)
    b, d, y = [rng.uniform(-1, 1, (m, n)) for _ in range(3)]
    b[:, 0] = 0.0; d[:, -1] = 0.0
    c = np.abs(b) + np.abs(d) + rng.uniform(1, 2, (m, n))
    z = np.zeros((m, n))
    full = [v.ravel().copy() for v in (z, b, c, d, z, y)]
    t = [torch.as_tensor(v).cuda() for v in full]
    info = pcrp.solve_mixed(None, t[1], t[2], t[3], None, t[5], m, n)
    torch.cuda.synchronize()
    x = t[5].cpu().numpy()
    assert info.converged == 1
    assert O.fwd_err(x, O.ge(*full, m, n), m, n) <= TOL
    t2 = [torch.as_tensor(v).cuda() for v in full]
    pcrp.solve_mixed(*t2, m, n, report=False)
    torch.cuda.synchronize()
    assert O.fwd_err(x, t2[5].cpu().numpy(), m, n) <= TOL


def test_mixed_null_inner_band_rejected(cuda):
    import torch
    t = [torch.zeros(8, dtype=torch.float64, device="cuda") for _ in range(6)]
    with pytest.raises(pcrp.PcrpError):
        pcrp.solve_mixed(t[0], None, t[2], t[3], t[4], t[5], 1, 8)


@pytest.mark.parametrize("mode", ["global", "thread_local", "relaxed"])
def test_mixed_inside_a_caller_graph_capture(cuda, mode):
    """Inside a caller's stream capture the solve (sweep loop included, as a
    while node) becomes part of the caller's graph; replaying that graph
    solves whatever the captured buffers hold, to the solver's bar."""
    import torch
    m, n = 8, 20000
    src = [torch.as_tensor(np.asarray(v)).cuda() for v in pcrp.generate(pcrp.GEN_DOMINANT, 9, m, n)]
    arrs = [v.clone() for v in src]
    ws = torch.empty(pcrp.workspace_size(m, n, which=1), dtype=torch.uint8, device="cuda")
    opts = pcrp.Opts(workspace=ws.data_ptr(), workspace_bytes=ws.numel())
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s, capture_error_mode=mode):
            pcrp.solve_mixed(*arrs, m, n, opts=opts, stream=s, report=False)
    for seed in (9, 10):
        fresh = [torch.as_tensor(np.asarray(v)).cuda() for v in pcrp.generate(pcrp.GEN_DOMINANT, seed, m, n)]
        for dst, v in zip(arrs, fresh):
            dst.copy_(v)
        g.replay()
        torch.cuda.synchronize()
        host = [v.cpu().numpy() for v in fresh]
        assert O.fwd_err(arrs[5].cpu().numpy(), O.ge(*host, m, n), m, n) <= TOL


@pytest.mark.parametrize("m,n", [(5, 512), (3, 4096), (4, 65536), (2, 1000), (40, 1000), (40, 20), (33, 9000)])
def test_mixed_interleaved_adapter_matches_contiguous(cuda, m, n):
    """An interleaved batch is solved through the layout adapter (transposed
    into contiguous copies, solved, transposed back): the same bits as the
    contiguous solve of the same systems, with and without the report, with
    NULL outer bands too, and in a caller workspace sized by
    pcrp_workspace_size for the interleaved layout."""
    import torch
    arrs = dd_bands(np.random.default_rng(m * n), m, n)
    inter = to_layout(arrs, m, n, pcrp.INTERLEAVED)
    xc, _, _ = run_mixed(arrs, m, n, pcrp.CONTIGUOUS, report=False)
    for report in (False, True):
        xi, _, _ = run_mixed(inter, m, n, pcrp.INTERLEAVED, report=report)
        xi_c = np.ascontiguousarray(xi.reshape(n, m).T).ravel()
        assert np.array_equal(xi_c.view(np.uint64), xc.view(np.uint64)), f"report={report}"
    # tridiagonal: NULL outer bands through the adapter
    tri = [np.zeros_like(arrs[0])] + list(arrs[1:4]) + [np.zeros_like(arrs[4]), arrs[5]]
    tc = to_device(tri, "cuda:0")
    pcrp.solve_mixed(None, *tc[1:4], None, tc[5], m, n, pcrp.CONTIGUOUS, report=False)
    ti = to_device(to_layout(tri, m, n, pcrp.INTERLEAVED), "cuda:0")
    pcrp.solve_mixed(None, *ti[1:4], None, ti[5], m, n, pcrp.INTERLEAVED, report=False)
    torch.cuda.synchronize()
    assert torch.equal(ti[5].view(n, m).t().contiguous().view(-1).view(torch.int64), tc[5].view(torch.int64))
    # caller workspace: the size the query gives for the interleaved layout
    # works, a workspace that cannot hold the copies is refused
    need = pcrp.workspace_size(m, n, pcrp.INTERLEAVED, which=1)
    assert need > pcrp.workspace_size(m, n, pcrp.CONTIGUOUS, which=1)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    xw, _, _ = run_mixed(inter, m, n, pcrp.INTERLEAVED, report=True,
                         opts=pcrp.Opts(workspace=ws.data_ptr(), workspace_bytes=need))
    assert np.array_equal(np.ascontiguousarray(xw.reshape(n, m).T).ravel().view(np.uint64), xc.view(np.uint64))
    small = 6 * m * n * 8 - 1
    with pytest.raises(pcrp.PcrpError):
        run_mixed(inter, m, n, pcrp.INTERLEAVED, report=True,
                  opts=pcrp.Opts(workspace=ws.data_ptr(), workspace_bytes=small))


@pytest.mark.parametrize("n", [700, 20000])
def test_mixed_nan_input_reports_nonconvergence(cuda, n):
    """A NaN in the right-hand side of one system poisons that system's norms:
    the stopping rule never accepts it, the call ends after max_sweeps with
    PCRP_ENOCONV (status 5), and the other systems are still solved (the
    whole-system kernel for n = 700, the windowed passes for n = 20000)."""
    import torch
    m = 3
    arrs = dd_bands(np.random.default_rng(11), m, n)
    arrs[5][n + n // 2] = np.nan                       # system 1
    t = to_device(arrs, "cuda:0")
    with pytest.raises(pcrp.PcrpError) as ei:
        pcrp.solve_mixed(*t, m, n, max_sweeps=4)
    assert ei.value.status == 5
    torch.cuda.synchronize()
    x = t[5].cpu().numpy().reshape(m, n)
    xg = np.asarray(O.ge(*arrs, m, n)).reshape(m, n)
    for j in (0, 2):
        assert np.abs(x[j] - xg[j]).max() / np.abs(xg[j]).max() <= TOL
    assert np.isnan(x[1]).any()


# --- sweeps 0 and 1 fused into one pass (mixed_duo.cu) ----------------------

@pytest.mark.parametrize("kind,m,n", [(pcrp.GEN_DOMINANT, 4, 65536), (pcrp.GEN_WEAK, 2, 1 << 20),
                                      (pcrp.GEN_DOMINANT, 3, 5002), (pcrp.GEN_WEAK, 5, 9000),
                                      (pcrp.GEN_DOMINANT, 3, 7682)])   # last window: one core block row
def test_mixed_fused_sweeps_match_general_kernels(cuda, kind, m, n, monkeypatch):
    """Systems longer than one tile run their first two sweeps in one fused
    pass (windows with halos, bulk-staged inputs, the factorisation kept in
    tensor memory; PCRP_DUO=1); the general kernels solve the same systems:
    both meet the bar, in two sweeps."""
    arrs = pcrp.generate(kind, 23, m, n)
    xg = O.ge(*arrs, m, n)
    monkeypatch.setenv("PCRP_DUO", "1")
    x, info, _ = run_mixed(arrs, m, n)
    assert info.converged == 1 and info.sweeps == 2
    assert O.fwd_err(x, xg, m, n) <= TOL
    monkeypatch.delenv("PCRP_DUO")
    xr, info_r, _ = run_mixed(arrs, m, n)
    assert info_r.converged == 1
    assert O.fwd_err(xr, xg, m, n) <= TOL


def test_mixed_systems_left_by_fused_sweeps_run_the_general_kernels(cuda, monkeypatch):
    """A tolerance that two sweeps cannot meet leaves every system to the
    general kernels, which solve it from the start: the same bits as a solve
    that never ran the fused pass, and more than two sweeps reported."""
    import torch
    m, n = 3, 20000
    arrs = dd_bands(np.random.default_rng(41), m, n)
    monkeypatch.setenv("PCRP_DUO", "1")
    t = to_device(arrs, cuda)
    pcrp.solve_mixed(*t, m, n, tol=1e-17, max_sweeps=4, report=False)
    torch.cuda.synchronize()
    fused = t[5].cpu().numpy()
    monkeypatch.delenv("PCRP_DUO")
    t2 = to_device(arrs, cuda)
    pcrp.solve_mixed(*t2, m, n, tol=1e-17, max_sweeps=4, report=False)
    torch.cuda.synchronize()
    assert np.array_equal(fused.view(np.uint64), t2[5].cpu().numpy().view(np.uint64))
    monkeypatch.setenv("PCRP_DUO", "1")
    try:                       # (a correction that is exactly zero at the FP64 floor meets any tol)
        _, info, _ = run_mixed(arrs, m, n, tol=1e-17, max_sweeps=4)
        assert info.sweeps >= 3
    except pcrp.PcrpError as ex:
        assert ex.status == 5


def test_mixed_fused_sweeps_bounded_wait_reports_timeout(cuda, monkeypatch):
    """Failure detection without a fault: the test hook makes every CTA of
    the fused kernel wait for a chunk that is never staged; the wait gives up
    after ~4 ms, the general kernels still solve every system, the report
    says PCRP_ETIMEOUT (status 4), and the context keeps working."""
    m, n = 3, 65536
    arrs = pcrp.generate(pcrp.GEN_DOMINANT, 29, m, n)
    monkeypatch.setenv("PCRP_DUO", "1")
    with pytest.raises(pcrp.PcrpError) as ei:
        run_mixed(arrs, m, n, opts=pcrp.Opts(reserved0=0x7E57))
    assert ei.value.status == 4
    x, info, _ = run_mixed(arrs, m, n)
    assert info.converged == 1 and O.fwd_err(x, O.ge(*arrs, m, n), m, n) <= TOL


@pytest.mark.parametrize("n", [16384, 40000])
def test_mixed_fused_sweeps_mixed_batch_and_nan(cuda, n, monkeypatch):
    """Through the fused pass: a batch where dominant systems decouple and ADI
    systems stay coupled (left to the general kernels), and a NaN in one
    system's rhs that must surface as non-convergence while the others are
    solved."""
    monkeypatch.setenv("PCRP_DUO", "1")
    dom = pcrp.generate(pcrp.GEN_DOMINANT, 3, 2, n)
    adi = pcrp.generate(pcrp.GEN_ADI, 4, 2, n)
    arrs = [np.concatenate([np.asarray(u), np.asarray(v)]) for u, v in zip(dom, adi)]
    x, info, _ = run_mixed(arrs, 4, n, max_sweeps=16)
    assert info.converged == 1
    assert O.fwd_err(x[: 2 * n], O.ge(*dom, 2, n), 2, n) <= TOL
    bad = [np.asarray(v).copy() for v in dom]
    bad[5][n + n // 3] = np.nan
    t = to_device(bad, cuda)
    with pytest.raises(pcrp.PcrpError) as ei:
        pcrp.solve_mixed(*t, 2, n, max_sweeps=4)
    assert ei.value.status == 5
    xs = t[5].cpu().numpy()
    assert O.fwd_err(xs[:n], O.ge(*[v[:n] for v in bad], 1, n), 1, n) <= TOL


def test_pipe_probe_reports_all_five_timings(cuda):
    """pcrp_measure_pipes times FP64, FP32 and integer chains alone and
    FP64 beside each of the others (the measurement behind the mixed
    kernels' split of work between the pipes): five positive, finite
    timings, and a pair never faster than its slower part."""
    import math
    t = pcrp.measure_pipes()
    assert set(t) == {"fp64", "fp32", "int", "fp64+fp32", "fp64+int"}
    assert all(v > 0 and math.isfinite(v) for v in t.values())
    assert t["fp64+fp32"] >= 0.95 * max(t["fp64"], t["fp32"])
    assert t["fp64+int"] >= 0.95 * max(t["fp64"], t["int"])
