"""torch.ops.pcrp.* operators: same results as the C ABI calls they wrap."""
import numpy as np
import pytest

import oracle as O
import pcrp
from helpers import assert_bitexact, dd_bands

pytestmark = pytest.mark.gpu


def test_torch_ops(cuda):
    import torch
    import pcrp.torch_ops  # noqa: F401  (registers the operators)
    m, n = 6, 3000
    arrs = dd_bands(np.random.default_rng(12), m, n)
    t = [torch.from_numpy(v.reshape(m, n)).to(cuda) for v in arrs]
    x = torch.ops.pcrp.solve_f64(*t)
    assert torch.equal(t[5].cpu(), torch.from_numpy(arrs[5].reshape(m, n)))      # input untouched
    assert_bitexact(x.cpu().numpy().ravel(), O.pcr(*arrs, m, n), "torch.ops.pcrp.solve_f64")
    xm = torch.ops.pcrp.solve_mixed(*t)
    assert O.fwd_err(xm.cpu().numpy().ravel(), O.ge(*arrs, m, n), m, n) <= 1e-12
    ti = [v.t().contiguous() for v in t]                                          # (n, m) interleaved
    xi = torch.ops.pcrp.solve_f64(*ti, interleaved=True)
    assert torch.equal(xi.t().cpu(), x.cpu())
