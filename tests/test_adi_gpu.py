"""The paper's application: batched Black-Scholes time stepping with the
pentadiagonal operator (second-order upwind convection), solved by the mixed
and the faithful FP64 solvers; prices agree with the closed form."""
import pytest

pytestmark = pytest.mark.gpu


def test_adi_european_calls_match_closed_form(cuda):
    import torch
    from pcrp.adi import black_scholes_call, price_call
    m, n, r, T, steps = 6, 2048, 0.03, 1.0, 200
    v = torch.linspace(0.02, 0.2, m, dtype=torch.float64, device=cuda)
    K = torch.linspace(80.0, 120.0, m, dtype=torch.float64, device=cuda)
    um = price_call(K, v, r, T, steps, n=n, solver="mixed")
    uf = price_call(K, v, r, T, steps, n=n, solver="f64")
    torch.cuda.synchronize()
    S = torch.arange(n, dtype=torch.float64, device=cuda) * (800.0 / (n - 1))
    for j in range(m):
        bs = black_scholes_call(S, float(K[j]), float(v[j]), r, T)
        sel = (S > 0.6 * K[j]) & (S < 1.4 * K[j])
        assert (um[j] - bs)[sel].abs().max().item() < 2e-3
        assert (uf[j] - bs)[sel].abs().max().item() < 2e-3
    assert (um - uf).abs().max().item() < 1e-6
