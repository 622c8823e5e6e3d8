"""The cuSPARSE comparison harness solves the same systems (sanity of the
benchmark's library baseline): gpsvInterleavedBatch agrees with FP64
elimination and with pcrp_solve_mixed."""
import numpy as np
import pytest

import oracle as O
import pcrp
from helpers import dd_bands, to_device, to_layout

pytestmark = pytest.mark.gpu


def test_cusparse_gpsv_matches_elimination(cuda):
    import torch
    import pcrp.compare as cmpmod
    m, n = 8, 3000
    arrs = dd_bands(np.random.default_rng(21), m, n)
    il = to_layout(arrs, m, n, pcrp.INTERLEAVED)
    t = to_device(il, cuda)
    cmpmod.gpsv_solve(*t, m, n)
    torch.cuda.synchronize()
    x = t[5].cpu().numpy()
    xg = O.ge(*il, m, n, pcrp.INTERLEAVED)
    assert O.fwd_err(x, xg, m, n, pcrp.INTERLEAVED) < 1e-12
