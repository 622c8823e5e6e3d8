"""Shared helpers for the parity tests (inputs, device copies, comparisons)."""
import numpy as np

import oracle as O
import pcrp


def dd_bands(rng, m, n, garbage=False):
    """Strictly diagonally dominant batch (contiguous), optional garbage in out-of-range slots."""
    a, b, d, e = [rng.uniform(-1, 1, (m, n)) for _ in range(4)]
    for arr, sl in ((a, np.s_[:, :2]), (b, np.s_[:, :1]), (d, np.s_[:, n - 1:]), (e, np.s_[:, max(n - 2, 0):])):
        arr[sl] = 0.0
    c = np.abs(a) + np.abs(b) + np.abs(d) + np.abs(e) + rng.uniform(1, 2, (m, n))
    y = rng.uniform(-1, 1, (m, n))
    if garbage:
        for arr, sl in ((a, np.s_[:, :2]), (b, np.s_[:, :1]), (d, np.s_[:, n - 1:]), (e, np.s_[:, max(n - 2, 0):])):
            arr[sl] = rng.uniform(-1e3, 1e3, arr[sl].shape)
    return [v.ravel().copy() for v in (a, b, c, d, e, y)]


def zero_bands(rng, m, n, special=False, zero_d=False):
    """Batch whose outer bands a, e are zeros of random sign (a pentadiagonal
    system already in the state of the late strides, where every product of
    the multipliers has a zero factor), with zeros of random sign sprinkled
    into b, d and y; `zero_d` makes d all zeros of random sign too (the lower
    bidiagonal state); `special` adds +-inf and NaN entries to a few systems."""
    def signed_zeros(shape):
        return np.where(rng.random(shape) < 0.5, 0.0, -0.0)
    a, e = signed_zeros((m, n)), signed_zeros((m, n))
    b, d, y = [rng.uniform(-1, 1, (m, n)) for _ in range(3)]
    if zero_d:
        d = signed_zeros((m, n))
    for arr in (b, d, y):
        hit = rng.random((m, n)) < 0.05
        arr[hit] = signed_zeros(int(hit.sum()))
    c = np.abs(b) + np.abs(d) + rng.uniform(1, 2, (m, n))
    a[:, :2] = 0.0; b[:, :1] = 0.0; d[:, n - 1:] = 0.0; e[:, max(n - 2, 0):] = 0.0
    if special and m >= 4 and n >= 8:
        c[1, n // 2] = np.inf
        y[2, n // 3] = np.nan
        b[3, n // 4] = -np.inf
        d[0, n // 5] = np.inf
    # one system keeps nonzero outer bands only in its first half, so the
    # rows of one tile mix both kinds
    a[m - 1, 2:n // 2] = rng.uniform(-0.1, 0.1, n // 2 - 2)
    e[m - 1, :n // 2] = rng.uniform(-0.1, 0.1, n // 2)
    return [v.ravel().copy() for v in (a, b, c, d, e, y)]


def to_layout(arrs, m, n, layout):
    if layout == pcrp.CONTIGUOUS:
        return [np.ascontiguousarray(v) for v in arrs]
    return [np.ascontiguousarray(v.reshape(m, n).T.ravel()) for v in arrs]


def to_device(arrs, dev):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in arrs]


def gpu_f64(arrs, m, n, layout=pcrp.CONTIGUOUS, path="auto", opts=None, dev="cuda:0"):
    import torch
    t = to_device(arrs, dev)
    pcrp.solve_f64(*t, m, n, layout, opts=opts, path=path)
    torch.cuda.synchronize()
    return t[5].cpu().numpy(), t


def assert_bitexact(x, xref, what=""):
    """Equal bit patterns (so +0 and -0 differ); any NaN matches any NaN."""
    x = np.ascontiguousarray(x, dtype=np.float64); xref = np.ascontiguousarray(xref, dtype=np.float64)
    same = (x.view(np.uint64) == xref.view(np.uint64)) | (np.isnan(x) & np.isnan(xref))
    if not same.all():
        bad = np.flatnonzero(~same)
        k = bad[0]
        rel = np.nanmax(np.abs(x[bad] - xref[bad]) / np.maximum(np.abs(xref[bad]), 1e-300))
        raise AssertionError(f"{what}: {bad.size} of {x.size} values differ; first at {k}: "
                             f"{x[k]!r} vs {xref[k]!r}; max rel diff {rel:.3e}")


def fwd_err(x, xref, m, n, layout=pcrp.CONTIGUOUS):
    return O.fwd_err(x, xref, m, n, layout)
