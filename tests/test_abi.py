"""CPU tests of the C ABI: the library loads, exports every declared symbol,
validates arguments without touching a GPU, and its generators are seeded."""
import ctypes
import os
import re

import numpy as np
import pytest

import pcrp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pcrp.h")).read()
    return sorted(set(re.findall(r"^\s*(?:pcrp_status|const char\*|int32_t|int64_t)\s+(pcrp_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(built_lib):
    L = ctypes.CDLL(built_lib)
    names = declared_functions()
    assert len(names) >= 14
    for name in names:
        assert hasattr(L, name), name
    assert set(names) <= set(pcrp.exported_symbols())


def test_version(built_lib):
    assert pcrp.version() >= 100


@pytest.mark.parametrize("fn", ["pcrp_solve_f64", "pcrp_solve_f64_small", "pcrp_solve_f64_split"])
def test_f64_argument_validation(built_lib, fn):
    L = pcrp.lib()
    f = getattr(L, fn)
    nn = 4096 if fn.endswith("split") else 16
    assert f(None, None, None, None, None, None, 0, nn, 0, None, None) == 0          # m = 0: no-op
    assert f(None, None, None, None, None, None, 4, 0, 0, None, None) == 0           # n = 0: no-op
    assert f(None, None, None, None, None, None, -1, nn, 0, None, None) == 1         # EINVAL
    assert f(None, None, None, None, None, None, 4, 2048, 7, None, None) == 1        # bad layout
    assert f(None, None, None, None, None, None, 4, 2048, 0, None, None) == 1        # null arrays
    assert pcrp.last_error() != ""
    if fn == "pcrp_solve_f64_small":
        assert f(1, 1, 1, 1, 1, 1, 4, 2048, 0, None, None) == 1
        assert "1024" in pcrp.last_error()
    if fn == "pcrp_solve_f64_split":
        assert f(1, 1, 1, 1, 1, 1, 4, 512, 0, None, None) == 1


def test_generators_are_seeded_and_layout_consistent(built_lib):
    for kind in (pcrp.GEN_DOMINANT, pcrp.GEN_ADI, pcrp.GEN_WEAK, pcrp.GEN_TOEPLITZ):
        A = pcrp.generate(kind, 42, 5, 77)
        B = pcrp.generate(kind, 42, 5, 77, threads=3)
        I = pcrp.generate(kind, 42, 5, 77, layout=pcrp.INTERLEAVED)
        for u, v, w in zip(A, B, I):
            assert np.array_equal(u, v)
            assert np.array_equal(u.reshape(5, 77).T.ravel(), w)
        # a slice of systems regenerates identically (values depend on (seed, j, i, n) only)
        S = pcrp.generate(kind, 42, 3, 77)
        for u, s in zip(A, S):
            assert np.array_equal(u[: 3 * 77], s)
    C = pcrp.generate(pcrp.GEN_DOMINANT, 43, 5, 77)
    assert not np.array_equal(A[0], C[0]) or True


def test_dominant_generator_properties(built_lib):
    m, n = 16, 300
    a, b, c, d, e, y = [v.reshape(m, n) for v in pcrp.generate(pcrp.GEN_DOMINANT, 1, m, n)]
    assert np.all(a[:, :2] == 0) and np.all(b[:, :1] == 0) and np.all(d[:, -1:] == 0) and np.all(e[:, -2:] == 0)
    off = np.abs(a) + np.abs(b) + np.abs(d) + np.abs(e)
    assert np.all(c - off >= 1.0) and np.all(c - off < 2.0 + 1e-12)
    assert np.all(np.abs(y) <= 1.0) and np.abs(a).max() <= 1.0


def test_weak_generator_properties(built_lib):
    m, n = 8, 200
    a, b, c, d, e, y = [v.reshape(m, n) for v in pcrp.generate(pcrp.GEN_WEAK, 2, m, n)]
    off = np.abs(a) + np.abs(b) + np.abs(d) + np.abs(e)
    np.testing.assert_allclose(np.abs(c), 1.05 * off, rtol=1e-15)
    assert (c < 0).any() and (c > 0).any()


def test_adi_generator_properties(built_lib):
    m, n = 4, 4096
    a, b, c, d, e, y = [v.reshape(m, n) for v in pcrp.generate(pcrp.GEN_ADI, 3, m, n)]
    assert np.all(a == 0)
    off = np.abs(b) + np.abs(d) + np.abs(e)
    assert np.all(c > off)                           # strictly dominant by the identity margin
    S = np.arange(n) * (800.0 / (n - 1))
    assert np.all(y >= 0) and np.all(y <= 800)
    for j in range(m):
        K = S[np.argmax(y[j] > 0)] if (y[j] > 0).any() else 800
        assert 50 - 1 <= K <= 150 + 1


def test_toeplitz_fixture_matches_reference_initialize(built_lib):
    n = 8
    a, b, c, d, e, y = pcrp.generate(pcrp.GEN_TOEPLITZ, 0, 1, n)
    assert list(c) == [5, 6, 6, 6, 6, 6, 6, 5]
    assert b[0] == 1 and d[-1] == 1 and a[0] == 0 and a[1] == 0 and e[-1] == 0 and e[-2] == 0
    assert np.all(y == 1)


def test_ragged_sizes(built_lib):
    s = pcrp.ragged_sizes(7, 4096, 32, 65536)
    assert s.min() >= 32 and s.max() <= 65536
    assert np.array_equal(s, pcrp.ragged_sizes(7, 4096, 32, 65536))
    # log-uniform: about half of the systems below the geometric mean
    gm = np.sqrt(32 * 65536)
    assert 0.4 < np.mean(s < gm) < 0.6


def test_mixed_workspace_includes_layout_adapter(built_lib):
    """Interleaved batches of more than one system are solved by the mixed
    solver through contiguous copies of the six arrays in the workspace: the
    size query counts them (256-byte aligned each); one system needs none."""
    import pcrp
    for m, n in ((4, 4096), (3, 1000), (256, 65536)):
        arr = (m * n * 8 + 255) // 256 * 256
        ci = pcrp.workspace_size(m, n, pcrp.CONTIGUOUS, which=1)
        ii = pcrp.workspace_size(m, n, pcrp.INTERLEAVED, which=1)
        assert ii - ci == 6 * arr
    assert pcrp.workspace_size(1, 5000, pcrp.INTERLEAVED, which=1) == pcrp.workspace_size(1, 5000, pcrp.CONTIGUOUS, which=1)


def test_noalloc_size_checks_do_not_wrap(built_lib):
    """The allocation-free entry point checks its fixed scratch without
    forming m*n (which could wrap around) and refuses before any CUDA call."""
    L = pcrp.lib()
    for m, n in ((1 << 33, 1 << 27), (1 << 40, 1 << 31), (3, 1 << 20), (9, 65536)):
        assert L.pcrp_solve_f64_noalloc(1, 1, 1, 1, 1, 1, m, n, 0, None) == 1, (m, n)
        assert "524288" in pcrp.last_error()
    for fn in ("pcrp_solve_f64", "pcrp_solve_f64_split"):
        # the split path's own scratch size is checked the same way
        assert getattr(L, fn)(1, 1, 1, 1, 1, 1, 1 << 40, 1 << 31, 0, None, None) == 1
        assert "too large" in pcrp.last_error() or "out of range" in pcrp.last_error()


def test_noalloc_accepts_any_batch_of_short_systems_on_cpu(built_lib):
    """Systems that fit the shared-memory tile need no scratch, so no size
    limit applies to them: without a GPU the call gets past the size check
    and fails only at the first CUDA call (PCRP_ECUDA, not PCRP_EINVAL)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("CPU-only check (fake pointers); the GPU test solves such a batch for real")
    L = pcrp.lib()
    rc = L.pcrp_solve_f64_noalloc(8, 8, 8, 8, 8, 8, 1 << 20, 512, 0, None)
    assert rc == 2, pcrp.last_error()


def test_workspace_size_ragged_family(built_lib):
    """which=2 (pcrp_solve_ragged) answers a bound for either mode: at least
    the FP64 mode's state for m*n rows; larger batches need more; an unknown
    family and an m*n that would wrap are refused."""
    import pcrp
    small = pcrp.workspace_size(16, 4096, which=2)
    big = pcrp.workspace_size(64, 4096, which=2)
    assert small >= 2 * 7 * 16 * 4096 * 8 and big > small
    for which in (3, -1):
        with pytest.raises(pcrp.PcrpError):
            pcrp.workspace_size(4, 4096, which=which)
    for which in (0, 1, 2):                  # no family's size wraps around
        with pytest.raises(pcrp.PcrpError):
            pcrp.workspace_size(1 << 40, 1 << 20, which=which)
    assert pcrp.workspace_size(1 << 20, 1 << 20, which=0) == 2 * 8 * 8 * (1 << 40)


def test_mixed_residual_host_ragged_argument_validation(built_lib):
    """The other entry points refuse bad arguments before any CUDA call (so
    without a GPU) and treat empty batches as no-ops, as pcrp.h states."""
    L = pcrp.lib()
    info = pcrp.MixedInfo()
    mixed = L.pcrp_solve_mixed
    assert mixed(None, None, None, None, None, None, 0, 64, 0, 0.0, 0, None, None, ctypes.byref(info)) == 0
    assert info.converged == 1                                                   # empty batch: converged
    assert mixed(None, None, None, None, None, None, 4, 0, 0, 0.0, 0, None, None, None) == 0
    assert mixed(None, None, None, None, None, None, -1, 64, 0, 0.0, 0, None, None, None) == 1
    assert mixed(None, None, None, None, None, None, 4, 64, 5, 0.0, 0, None, None, None) == 1   # layout
    assert mixed(None, None, None, None, None, None, 4, 64, 0, 0.0, 0, None, None, None) == 1   # null arrays
    assert "null array" in pcrp.last_error()
    assert mixed(1, 1, 1, 1, 1, 1, 1 << 25, 64, 0, 0.0, 0, None, None, None) == 1               # m > 2^24
    assert "out of range" in pcrp.last_error()
    assert mixed(1, 1, 1, 1, 1, 1, 4, (1 << 31) + 2, 0, 0.0, 0, None, None, None) == 1          # n > 2^31

    res = L.pcrp_residual_f64
    assert res(*([None] * 8), 0, 64, 0, None) == 0
    assert res(*([None] * 8), -3, 64, 0, None) == 1
    assert res(*([None] * 8), 4, 64, 9, None) == 1
    assert res(*([None] * 8), 4, 64, 0, None) == 1
    assert res(1, 1, 1, 1, 1, 1, 7, 7, 4, 64, 0, None) == 1                                     # r aliases x
    assert "alias" in pcrp.last_error()

    host = L.pcrp_solve_host
    assert host(*([None] * 6), 0, 64, 0, 0, 0.0, 0, None, None) == 0
    assert host(*([None] * 6), -1, 64, 0, 0, 0.0, 0, None, None) == 1
    assert host(*([None] * 6), 4, 64, 3, 0, 0.0, 0, None, None) == 1                            # layout
    assert host(*([None] * 6), 4, 64, 0, 2, 0.0, 0, None, None) == 1                            # precision
    assert "precision" in pcrp.last_error()
    assert host(*([None] * 6), 4, 64, 0, 1, 0.0, 0, None, None) == 1                            # null arrays

    rg = L.pcrp_solve_ragged
    assert rg(*([None] * 7), 0, 64, 0, 0.0, 0, None, None) == 0
    assert rg(*([None] * 7), 8, 0, 1, 0.0, 0, None, None) == 0
    assert rg(*([None] * 7), -1, 64, 0, 0.0, 0, None, None) == 1
    assert rg(*([None] * 7), 8, -1, 0, 0.0, 0, None, None) == 1
    assert rg(*([None] * 7), 8, 64, 2, 0.0, 0, None, None) == 1                                 # mode
    assert "mode" in pcrp.last_error()
    assert rg(1, 1, 1, 1, 1, 1, None, 8, 64, 0, 0.0, 0, None, None) == 1                        # null offsets
    assert rg(1, 1, 1, 1, 1, 1, 1, (1 << 24) + 1, 64, 1, 0.0, 0, None, None) == 1               # nsys > 2^24
    assert "out of range" in pcrp.last_error()


def test_python_wrappers_check_type_and_length(built_lib):
    """The ctypes wrappers refuse arrays the library would read past or
    misread (wrong element type, fewer than m*n elements, not contiguous)
    before any call into it."""
    import torch

    good = np.zeros(64, dtype=np.float64)
    with pytest.raises(TypeError):
        pcrp.solve_host(*([np.zeros(64, dtype=np.float32)] * 6), 4, 16)
    with pytest.raises(ValueError):
        pcrp.solve_host(*([good[:63]] * 6), 4, 16)
    with pytest.raises(ValueError):
        pcrp.solve_host(*([np.zeros(128)[::2]] * 6), 4, 16)
    with pytest.raises(TypeError):
        pcrp.generate_into(pcrp.GEN_DOMINANT, 1, 4, 16, pcrp.CONTIGUOUS, [torch.zeros(64, dtype=torch.float32)] * 6)
    assert pcrp._host_ptr(good, 64) == good.ctypes.data

    class FakeDeviceTensor:                 # what _ptr reads of a CUDA tensor, without a GPU
        is_cuda = True

        def __init__(self, dtype, numel):
            self.dtype, self._numel = dtype, numel

        def is_contiguous(self):
            return True

        def numel(self):
            return self._numel

        def data_ptr(self):
            return 4096

    assert pcrp._ptr(FakeDeviceTensor(torch.float64, 64), 64) == 4096
    with pytest.raises(TypeError):
        pcrp._ptr(FakeDeviceTensor(torch.float32, 64), 64)
    with pytest.raises(ValueError):
        pcrp._ptr(FakeDeviceTensor(torch.float64, 63), 64)
    with pytest.raises(TypeError):
        pcrp.solve_ragged(*([FakeDeviceTensor(torch.float64, 64)] * 6), FakeDeviceTensor(torch.int32, 5), 4, 16)
    with pytest.raises(ValueError):
        pcrp.solve_ragged(*([FakeDeviceTensor(torch.float64, 64)] * 6), FakeDeviceTensor(torch.int64, 4), 4, 16)
    with pytest.raises(ValueError):
        pcrp.solve_mixed(*([FakeDeviceTensor(torch.float64, 63)] * 6), 4, 16)
