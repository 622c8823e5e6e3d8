"""GPU parity of the faithful FP64 PCR-Penta path against the oracle.

The CUDA kernels form every product, sum and quotient of the reference's
stride arithmetic (kernel.cu:63-153) in its order without FMA contraction,
so the bar is BIT-EXACT equality with the CPU restatement, on every size,
layout and pass plan, including garbage in out-of-range band slots."""
import ctypes

import numpy as np
import pytest

import oracle as O
import pcrp
from helpers import assert_bitexact, dd_bands, gpu_f64, to_device, to_layout, zero_bands

pytestmark = pytest.mark.gpu

SMALL_N = [1, 2, 3, 4, 5, 7, 8, 16, 31, 32, 33, 64, 100, 127, 128, 255, 256, 500, 512, 513, 1000, 1023, 1024]


@pytest.mark.parametrize("n", SMALL_N)
@pytest.mark.parametrize("layout", [pcrp.CONTIGUOUS, pcrp.INTERLEAVED])
def test_small_path_bitexact(cuda, n, layout):
    rng = np.random.default_rng(1000 + n)
    m = 5
    arrs = to_layout(dd_bands(rng, m, n, garbage=(n % 2 == 1)), m, n, layout)
    x, _ = gpu_f64(arrs, m, n, layout, path="small")
    assert_bitexact(x, O.pcr(*arrs, m, n, layout), f"small n={n} layout={layout}")


@pytest.mark.parametrize("n,opts", [
    (1025, {}), (2048, {}), (3000, {}), (4096, {}), (5001, {}),
    (4096, dict(fuse_strides=1)), (4096, dict(fuse_strides=2, tile_rows=100)),
    (4096, dict(smem_rows=64, fuse_strides=3, tile_rows=37)),
    (8192, dict(smem_rows=2048)), (8192, dict(smem_rows=256, fuse_strides=4)),
    (3000, dict(smem_rows=16, fuse_strides=5, tile_rows=300, threads=64)),
])
@pytest.mark.parametrize("layout", [pcrp.CONTIGUOUS, pcrp.INTERLEAVED])
def test_split_path_bitexact(cuda, n, opts, layout):
    rng = np.random.default_rng(n + len(opts))
    m = 3
    arrs = to_layout(dd_bands(rng, m, n, garbage=True), m, n, layout)
    x, _ = gpu_f64(arrs, m, n, layout, path="split", opts=pcrp.Opts(**opts) if opts else None)
    assert_bitexact(x, O.pcr(*arrs, m, n, layout), f"split n={n} {opts} layout={layout}")


@pytest.mark.parametrize("n,opts", [(300, dict(smem_rows=32)), (777, dict(smem_rows=8, fuse_strides=2, tile_rows=11))])
def test_auto_path_with_small_tiles_bitexact(cuda, n, opts):
    """pcrp_solve_f64 may split systems below 1024 rows when told to; same bits."""
    rng = np.random.default_rng(n)
    m = 4
    arrs = dd_bands(rng, m, n)
    x, _ = gpu_f64(arrs, m, n, opts=pcrp.Opts(**opts))
    assert_bitexact(x, O.pcr(*arrs, m, n), f"auto n={n} {opts}")


def test_small_config_full_size_bitexact(cuda):
    """Plain FP64 shared-memory path at m=1024, n=512 (dominant generator)."""
    m, n = 1024, 512
    arrs = pcrp.generate(pcrp.GEN_DOMINANT, 2024, m, n)
    x, _ = gpu_f64(arrs, m, n)
    assert_bitexact(x, O.pcr(*arrs, m, n), "m=1024 n=512")
    # the reference algorithm itself is this far from elimination (5.3e-10 observed)
    assert O.fwd_err(x, O.ge(*arrs, m, n), m, n) < 1e-8


def test_large_config_full_size_bitexact(cuda):
    """Plain FP64 global path at m=256, n=65536: every system bit-exact."""
    m, n = 256, 65536
    arrs = pcrp.generate(pcrp.GEN_DOMINANT, 7, m, n)
    x, _ = gpu_f64(arrs, m, n)
    assert_bitexact(x, O.pcr(*arrs, m, n), "m=256 n=65536")


def test_max_size_bitexact(cuda):
    """n = 2^20 (the HBM-filling size; beyond the reference's own n <= 2^19 range)."""
    m, n = 2, 1 << 20
    arrs = pcrp.generate(pcrp.GEN_WEAK, 11, m, n)
    x, _ = gpu_f64(arrs, m, n)
    assert_bitexact(x, O.pcr(*arrs, m, n), "n=2^20 weak")


def test_adi_and_toeplitz_bitexact(cuda):
    for kind, m, n in ((pcrp.GEN_ADI, 64, 4096), (pcrp.GEN_TOEPLITZ, 3, 256), (pcrp.GEN_TOEPLITZ, 3, 1024),
                       (pcrp.GEN_TOEPLITZ, 2, 4096)):
        arrs = pcrp.generate(kind, 5, m, n)
        x, _ = gpu_f64(arrs, m, n)
        assert_bitexact(x, O.pcr(*arrs, m, n), f"kind={kind} n={n}")


@pytest.mark.parametrize("n,path,opts", [
    (64, "small", None), (1000, "small", None), (1024, "small", None),
    (4096, "split", None), (5001, "split", pcrp.Opts(smem_rows=256, fuse_strides=3, tile_rows=100)),
    (1000, "auto", pcrp.Opts(smem_rows=16, fuse_strides=6, tile_rows=50)),
    (300, "auto", pcrp.Opts(smem_rows=8, fuse_strides=3, tile_rows=7)),
    (65536, "auto", None)])
@pytest.mark.parametrize("special", [False, True])
@pytest.mark.parametrize("zero_d", [False, True])
def test_zero_outer_bands_bitexact(cuda, n, path, opts, special, zero_d):
    """Zero outer bands (signed zeros), zeros in b, d, y (or d all zeros: the
    lower-bidiagonal state), and +-inf / NaN entries: the rows whose products
    have zero factors are formed on the integer pipe and must give the bits
    of the IEEE operations, zero signs included; rows with a non-finite
    operand take the FP64 operations."""
    rng = np.random.default_rng(n + 7 * special + 13 * zero_d)
    m = 6
    arrs = zero_bands(rng, m, n, special=special, zero_d=zero_d)
    x, _ = gpu_f64(arrs, m, n, path=path, opts=opts)
    ref = O.pcr(*arrs, m, n)
    if not special and not zero_d:
        assert np.isfinite(ref).all()
    assert_bitexact(x, ref, f"zero bands n={n} path={path} special={special} zero_d={zero_d}")


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_phase_b_quotients_match_ieee_division(cuda, mode):
    """Phase B forms its two quotients from one correctly rounded reciprocal
    of cT (Markstein's correction inside an exponent guard); on 2^28 random
    pairs per operand class every quotient has the bits of __ddiv_rn."""
    bad, fast = pcrp.check_quotients(mode, 1234 + mode, 1 << 28)
    assert bad == 0
    assert fast > (1 << 26)                       # the guard admits most pairs of every class


@pytest.mark.parametrize("n", [700, 5000, 65536])
def test_rows_scaled_across_the_exponent_range_bitexact(cuda, n):
    """Rows scaled by random powers of two up to 2^+-500.  A power-of-two row
    scale commutes exactly with every operation while nothing overflows, so
    the solution keeps the unscaled system's bits; meanwhile numerators and
    divisors of neighbouring rows differ by up to 2^1000, past the 900-octave
    exponent guard of phase B's shared-reciprocal quotients, so the IEEE
    division takes over for those pairs.  Bits equal the oracle's for both the
    scaled and the unscaled system."""
    rng = np.random.default_rng(n)
    m = 4
    arrs = dd_bands(rng, m, n)
    scale = np.ldexp(1.0, rng.integers(-500, 501, m * n))
    scaled = [v * scale for v in arrs]
    x, _ = gpu_f64(scaled, m, n)
    ref = O.pcr(*scaled, m, n)
    assert np.isfinite(ref).all()
    assert_bitexact(x, ref, f"scaled rows n={n}")
    assert_bitexact(x, O.pcr(*arrs, m, n), f"scaled rows vs unscaled n={n}")


def tridiagonal(rng, m, n, special=False):
    """A diagonally dominant tridiagonal batch as five bands (a = e = +0.0);
    `special` puts +-inf and NaN into a few systems."""
    arrs = dd_bands(rng, m, n, garbage=True)
    arrs[0][:] = 0.0
    arrs[4][:] = 0.0
    if special and m >= 3 and n >= 8:
        arrs[2][n // 2] = np.inf
        arrs[5][n + n // 3] = np.nan
        arrs[1][2 * n + n // 4] = -np.inf
    return arrs


def solve_null_outer(arrs, m, n, layout, drop=(0, 4), path="auto", opts=None):
    """pcrp_solve_f64 with the bands at `drop` passed as NULL."""
    import torch
    t = to_device(arrs, "cuda:0")
    args = [None if k in drop else v for k, v in enumerate(t)]
    pcrp.solve_f64(*args, m, n, layout, opts=opts, path=path)
    torch.cuda.synchronize()
    return t[5].cpu().numpy()


@pytest.mark.parametrize("n,path,opts", [
    (1, "small", None), (300, "small", None), (1024, "auto", None), (1025, "split", None),
    (5000, "auto", None), (65536, "auto", None), (70001, "auto", None),
    (3000, "split", dict(smem_rows=16, fuse_strides=5, tile_rows=300, threads=64)),
])
@pytest.mark.parametrize("layout", [pcrp.CONTIGUOUS, pcrp.INTERLEAVED])
@pytest.mark.parametrize("special", [False, True])
def test_tridiagonal_null_outer_bands_bitexact(cuda, n, path, opts, layout, special):
    """a = e = NULL, a tridiagonal batch: the bands are +0.0 and not read, and
    every pass runs the zero-operand strides (the vote still checks every
    tile, so non-finite systems take the FP64 operations).  Bits equal the
    oracle's on explicit +0.0 bands and the solve given those bands."""
    m = 3
    arrs = to_layout(tridiagonal(np.random.default_rng(7 * n + special), m, n, special), m, n, layout)
    o = pcrp.Opts(**opts) if opts else None
    x = solve_null_outer(arrs, m, n, layout, path=path, opts=o)
    assert_bitexact(x, O.pcr(*arrs, m, n, layout), f"tridiagonal n={n} layout={layout}")
    xz, _ = gpu_f64(arrs, m, n, layout, path=path, opts=o)
    assert_bitexact(x, xz, f"tridiagonal NULL vs +0.0 bands n={n}")


@pytest.mark.parametrize("n", [700, 9000])
@pytest.mark.parametrize("drop", [(0,), (4,)])
def test_one_null_outer_band_bitexact(cuda, n, drop):
    """Only a (or only e) NULL: that band is +0.0, the other is read."""
    m = 4
    arrs = dd_bands(np.random.default_rng(n + drop[0]), m, n)
    arrs[drop[0]][:] = 0.0
    x = solve_null_outer(arrs, m, n, pcrp.CONTIGUOUS, drop=drop)
    assert_bitexact(x, O.pcr(*arrs, m, n), f"band {drop} NULL n={n}")


def test_null_inner_band_is_refused(cuda):
    L = pcrp.lib()
    t = to_device(dd_bands(np.random.default_rng(0), 2, 100), "cuda:0")
    p = [v.data_ptr() for v in t]
    rc = L.pcrp_solve_f64(p[0], None, p[2], p[3], p[4], p[5], 2, 100, 0, None, None)
    assert rc == 1 and "only a and e may be null" in pcrp.last_error()   # PCRP_EINVAL


def test_bands_are_not_modified(cuda):
    import torch
    for n in (300, 5000):
        m = 3
        arrs = dd_bands(np.random.default_rng(n), m, n)
        t = to_device(arrs, cuda)
        before = [v.clone() for v in t[:5]]
        pcrp.solve_f64(*t, m, n)
        torch.cuda.synchronize()
        for u, v in zip(before, t[:5]):
            assert torch.equal(u, v)


def test_caller_workspace_and_stream(cuda):
    import torch
    m, n = 4, 9000
    arrs = dd_bands(np.random.default_rng(3), m, n)
    need = pcrp.workspace_size(m, n)
    assert need > 0
    small = torch.empty(need // 8 - 1, dtype=torch.float64, device=cuda)
    t = to_device(arrs, cuda)
    with pytest.raises(pcrp.PcrpError) as ei:
        pcrp.solve_f64(*t, m, n, opts=pcrp.Opts(workspace=small.data_ptr(), workspace_bytes=small.numel() * 8))
    assert ei.value.status == 3
    ws = torch.empty(need // 8, dtype=torch.float64, device=cuda)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        t = to_device(arrs, cuda)
        pcrp.solve_f64(*t, m, n, opts=pcrp.Opts(workspace=ws.data_ptr(), workspace_bytes=need), stream=s)
    s.synchronize()
    assert_bitexact(t[5].cpu().numpy(), O.pcr(*arrs, m, n), "caller workspace")


def test_repeat_calls_are_deterministic(cuda):
    m, n = 8, 3000
    arrs = dd_bands(np.random.default_rng(4), m, n)
    x1, _ = gpu_f64(arrs, m, n)
    x2, _ = gpu_f64(arrs, m, n)
    assert np.array_equal(x1, x2)


def test_device_generator_matches_host(cuda):
    import torch
    for kind in range(4):
        for layout in (pcrp.CONTIGUOUS, pcrp.INTERLEAVED):
            m, n = 6, 1111
            host = pcrp.generate(kind, 99, m, n, layout)
            dev = [torch.empty(m * n, dtype=torch.float64, device=cuda) for _ in range(6)]
            pcrp.generate_device(kind, 99, m, n, layout, dev)
            torch.cuda.synchronize()
            for h, d in zip(host, dev):
                assert np.array_equal(h, d.cpu().numpy())


@pytest.mark.parametrize("n", [2, 64, 512, 1000, 1024])
def test_bulk_staged_tiles_match_thread_loads(cuda, n):
    """Whole systems of even n in contiguous, 16-byte aligned arrays are
    staged into shared memory by bulk asynchronous copies; arrays that start
    8 bytes past a 16-byte boundary take the per-thread loads.  Same bits
    (and the oracle's), with and without the outer bands."""
    import torch
    m = 37
    arrs = dd_bands(np.random.default_rng(n + 5), m, n, garbage=True)
    xo = O.pcr(*arrs, m, n)
    for tri in (False, True):
        src = [np.zeros_like(v) if tri and k in (0, 4) else v for k, v in enumerate(arrs)]
        xo_t = O.pcr(*src, m, n) if tri else xo
        al = [torch.from_numpy(v.copy()).to(cuda) for v in src]
        bufs = [torch.empty(m * n + 1, dtype=torch.float64, device=cuda) for _ in range(6)]
        un = [b[1:] for b in bufs]
        for u, v in zip(un, src):
            u.copy_(torch.from_numpy(v))
        assert al[1].data_ptr() % 16 == 0 and un[1].data_ptr() % 16 == 8
        if tri:
            pcrp.solve_f64(None, *al[1:4], None, al[5], m, n)
            pcrp.solve_f64(None, *un[1:4], None, un[5], m, n)
        else:
            pcrp.solve_f64(*al, m, n)
            pcrp.solve_f64(*un, m, n)
        torch.cuda.synchronize()
        assert_bitexact(al[5].cpu().numpy(), xo_t, f"bulk-staged n={n} tri={tri}")
        assert_bitexact(un[5].cpu().numpy(), xo_t, f"thread loads n={n} tri={tri}")
