"""CPU tests of the oracle: ground-truth solver vs SciPy, the PCR restatement's
stride rule and edge cases, known-answer systems.  No GPU."""
import math

import numpy as np
import pytest
import scipy.linalg as sl

import oracle as O
from helpers import dd_bands


def scipy_solve(a, b, c, d, e, y, m, n):
    xs = []
    A, B, C, D, E, Y = [v.reshape(m, n) for v in (a, b, c, d, e, y)]
    for j in range(m):
        ab = np.zeros((5, n))
        if n > 2: ab[0, 2:] = E[j, :-2]
        if n > 1: ab[1, 1:] = D[j, :-1]
        ab[2] = C[j]
        if n > 1: ab[3, :-1] = B[j, 1:]
        if n > 2: ab[4, :-2] = A[j, 2:]
        xs.append(sl.solve_banded((2, 2), ab, Y[j]))
    return np.concatenate(xs)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 31, 64, 100, 512, 1000, 4096])
def test_ge_matches_scipy(n):
    rng = np.random.default_rng(n)
    m = 5
    arrs = dd_bands(rng, m, n)
    xg = O.ge(*arrs, m, n)
    xs = scipy_solve(*arrs, m, n)
    assert O.fwd_err(xg, xs, m, n) < 1e-14


def test_ge_interleaved_equals_contiguous():
    rng = np.random.default_rng(3)
    m, n = 7, 33
    arrs = dd_bands(rng, m, n)
    xc = O.ge(*arrs, m, n, O.CONTIGUOUS)
    il = [v.reshape(m, n).T.ravel().copy() for v in arrs]
    xi = O.ge(*il, m, n, O.INTERLEAVED)
    assert np.array_equal(xi.reshape(n, m).T.ravel(), xc)


def reference_k2(n):
    """main.cu:39 literally: k2 = ceil((float)log(n)/log(2)); pcr_penta loops k2-1 times."""
    return math.ceil(float(np.float32(math.log(n))) / math.log(2))


def test_stride_rule_matches_reference_host_formula():
    # n <= 1024: pcr_penta runs k2-1 strides (kernel.cu:63)
    for n in range(1, 1025):
        assert O.ref_strides(n) == max(reference_k2(n) - 1, 0), n
    # n > 1024, powers of two: log2(G) splitting strides + (k1-1) = 10 second-stage strides
    for k in range(11, 21):
        n = 1 << k
        G = math.ceil(float(np.float32(n)) / 1024)
        num_split = int(math.log(G) / math.log(2.0))
        k1 = math.ceil(float(np.float32(math.log(1024))) / math.log(2))
        assert O.ref_strides(n) == num_split + (k1 - 1) == k


@pytest.mark.parametrize("n", [1, 2, 3, 5, 6, 9, 16, 17, 63, 64, 65, 250, 512, 1024, 2048, 3000])
def test_pcr_restatement_solves_dd_systems(n):
    rng = np.random.default_rng(100 + n)
    m = 6
    arrs = dd_bands(rng, m, n)
    xp = O.pcr(*arrs, m, n)
    xg = O.ge(*arrs, m, n)
    # The reference's stride arithmetic pivots on off-diagonal entries, so its
    # error grows with n; this bounds it well above what is observed.
    assert O.fwd_err(xp, xg, m, n) < 1e-10


def test_pcr_out_of_range_slots_are_ignored_bitexact():
    rng = np.random.default_rng(11)
    for n in (1, 2, 3, 5, 64, 100):
        m = 4
        clean = dd_bands(np.random.default_rng(n), m, n, garbage=False)
        dirty = dd_bands(np.random.default_rng(n), m, n, garbage=True)
        assert not all(np.array_equal(u, v) for u, v in zip(clean, dirty)) or n == 1 and False is False
        assert np.array_equal(O.pcr(*clean, m, n), O.pcr(*dirty, m, n))
        assert np.array_equal(O.ge(*clean, m, n), O.ge(*dirty, m, n))


def dyadic_kat(rng, m, n, allow_zero_offdiag):
    """Bands and x with few mantissa bits: y = A x is exact, so x is the exact answer."""
    def offd():
        v = rng.integers(1, 9, (m, n)) * rng.choice([-1, 1], (m, n))
        if allow_zero_offdiag:
            v = rng.integers(-8, 9, (m, n))
        return v / 8.0
    a, b, d, e = [offd() for _ in range(4)]
    a[:, :2] = 0; b[:, :1] = 0; d[:, -1:] = 0; e[:, -2:] = 0
    c = np.abs(a) + np.abs(b) + np.abs(d) + np.abs(e) + 1.0
    x = rng.integers(-64, 65, (m, n)).astype(np.float64)
    y = c * x
    y[:, 2:] += a[:, 2:] * x[:, :-2]
    y[:, 1:] += b[:, 1:] * x[:, :-1]
    y[:, :-1] += d[:, :-1] * x[:, 1:]
    y[:, :-2] += e[:, :-2] * x[:, 2:]
    return [v.ravel().copy() for v in (a, b, c, d, e, y)], x.ravel()


def test_known_answer_dyadic_system():
    m, n = 3, 256
    arrs, x = dyadic_kat(np.random.default_rng(5), m, n, allow_zero_offdiag=False)
    assert np.all(O.residual(*arrs, x, m, n) == 0)
    assert O.fwd_err(O.ge(*arrs, m, n), x, m, n) < 1e-14


def test_known_answer_random_system():
    """x chosen first, y = A x formed in extended precision: the exact answer is x
    up to the rounding of y."""
    rng = np.random.default_rng(8)
    for n in (7, 64, 512, 2048):
        m = 4
        arrs = dd_bands(rng, m, n)
        x = rng.uniform(-1, 1, m * n)
        a, b, c, d, e, _ = [v.reshape(m, n).astype(np.longdouble) for v in arrs]
        X = x.reshape(m, n).astype(np.longdouble)
        y = c * X
        y[:, 2:] += a[:, 2:] * X[:, :-2]
        y[:, 1:] += b[:, 1:] * X[:, :-1]
        y[:, :-1] += d[:, :-1] * X[:, 1:]
        y[:, :-2] += e[:, :-2] * X[:, 2:]
        arrs[5] = y.astype(np.float64).ravel()
        assert O.fwd_err(O.ge(*arrs, m, n), x, m, n) < 1e-14
        assert O.fwd_err(O.pcr(*arrs, m, n), x, m, n) < 1e-10


def test_reference_algorithm_fails_on_zero_offdiagonal_pivots():
    """The reference guards a zero pivot b[i-2d] (or d[i+2d]) by setting the
    multiplier to 0 (kernel.cu:72-75), which leaves the x_{i-3d} coupling in
    place and drops it: on a strictly dominant system with exact zeros among
    the off-diagonals the PCR-Penta answer is wrong while elimination is exact.
    The same happens when a reduced off-diagonal cancels to exactly zero during
    the strides, which dyadic inputs make likely.  The restatement reproduces
    that behaviour rather than repairing it."""
    m, n = 3, 256
    for zeros in (True, False):
        arrs, x = dyadic_kat(np.random.default_rng(5), m, n, allow_zero_offdiag=zeros)
        assert O.fwd_err(O.ge(*arrs, m, n), x, m, n) < 1e-14
        assert O.fwd_err(O.pcr(*arrs, m, n), x, m, n) > 1e-3


def test_identity_and_diagonal_systems():
    for n in (32, 37):
        m = 2
        z = np.zeros(m * n)
        c = np.linspace(1, 3, m * n)
        y = np.linspace(-1, 1, m * n)
        xp = O.pcr(z, z, c, z, z, y, m, n)
        if n == 32:     # each stride negates the row exactly; x = (-1)^k y / (-1)^k c
            assert np.array_equal(xp, y / c)
        else:           # the pairwise 2x2 finish rounds differently
            np.testing.assert_allclose(xp, y / c, rtol=4e-16, atol=0)
        assert np.array_equal(O.ge(z, z, c, z, z, y, m, n), y / c)
        one = np.ones(m * n)
        assert np.array_equal(O.pcr(z, z, one, z, z, y, m, n), y)


def test_zero_pivot_keeps_last_multiplier():
    """A Reduction-III pivot that is exactly zero reuses the multiplier register
    (kernel.cu:122,129).  Hand-built: row 1 of a 4-row system makes T's pivot 0."""
    n = 4
    a = np.zeros(n); b = np.zeros(n); d = np.zeros(n); e = np.zeros(n)
    c = np.array([1.0, 0.0, 1.0, 1.0]); b[2] = 1.0; d[0] = 1.0
    y = np.array([1.0, 2.0, 3.0, 4.0])
    x = O.pcr(a, b, c, d, e, y, 1, n)
    assert x.shape == (n,)     # finite or not, it must be deterministic
    assert np.array_equal(x, O.pcr(a, b, c, d, e, y, 1, n), equal_nan=True)


def test_ragged_oracle_matches_uniform():
    rng = np.random.default_rng(9)
    sizes = np.array([1, 5, 64, 3, 200])
    offs = np.concatenate([[0], np.cumsum(sizes)])
    parts = [dd_bands(rng, 1, int(s)) for s in sizes]
    arrs = [np.concatenate([p[k] for p in parts]) for k in range(6)]
    for kind, fn in (("pcr", O.pcr), ("ge", O.ge)):
        xr = O.ragged(*arrs, offs[:-1], sizes, kind=kind)
        for k, s in enumerate(sizes):
            sl_ = slice(offs[k], offs[k + 1])
            assert np.array_equal(xr[sl_], fn(*[v[sl_] for v in arrs], 1, int(s)))


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("layout", [0, 1])
def test_oracle_generator_equals_library_generator(kind, layout):
    """The oracle's restated generator (used by the CPU legs of bench.py so
    that they never load libpcrp.so) gives the library generator's bits."""
    pcrp = pytest.importorskip("pcrp")
    for m, n in [(3, 1), (4, 7), (5, 4096), (2, 65536)]:
        ours = pcrp.generate(kind, 7, m, n, layout)
        theirs = O.generate(kind, 7, m, n, layout)
        for u, v in zip(ours, theirs):
            assert np.array_equal(np.asarray(u).view(np.uint64), v.view(np.uint64))
