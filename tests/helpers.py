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
    x = np.asarray(x); xref = np.asarray(xref)
    same = (x == xref) | (np.isnan(x) & np.isnan(xref))
    if not same.all():
        bad = np.flatnonzero(~same)
        k = bad[0]
        rel = np.nanmax(np.abs(x[bad] - xref[bad]) / np.maximum(np.abs(xref[bad]), 1e-300))
        raise AssertionError(f"{what}: {bad.size} of {x.size} values differ; first at {k}: "
                             f"{x[k]!r} vs {xref[k]!r}; max rel diff {rel:.3e}")


def fwd_err(x, xref, m, n, layout=pcrp.CONTIGUOUS):
    return O.fwd_err(x, xref, m, n, layout)
