"""Time stepping of batched 1D convection-diffusion (Black-Scholes) problems
on the GPU with the pentadiagonal solvers -- the application the PCR-Penta
paper targets (pentadiagonal systems from second-order upwinding of the
convection term of a Heston/Black-Scholes PDE).

Each of the m problems solves, in time-to-maturity form,

    u_t = 1/2 v S^2 u_SS + r S u_S - r u,    u(0, S) = payoff(S),

on a uniform grid S_i = i h, h = S_max/(n-1), with the operator

    L = 1/2 v S^2 (1,-2,1)/h^2 + r S (-3,4,-1)/(2h) on offsets (0,+1,+2) - r

(the second-order one-sided stencil on the upwind side of the convection term
makes L pentadiagonal), and the theta scheme

    (I - theta dt L) u^{k+1} = (I + (1-theta) dt L) u^k.

A few fully implicit start-up steps (Rannacher) damp the kink of the payoff.
The right-hand side is formed on the device with the fused FP64 residual
(r = 0 - (-B) u = B u) and every step calls the batched solver; the band
arrays of each operator are assembled once and reused by every step with the
same (theta, dt).  At S = 0 the
stencil needs no outside values (S_0 = 0 removes the diffusion and
convection terms).  At S_max the values beyond the grid are extrapolated
linearly (u_SS = 0, the far-field behaviour of a call): the ghost values
u_n = 2u_{n-1} - u_{n-2} and u_{n+1} = 3u_{n-1} - 2u_{n-2} fold into the last
two rows, which keeps the matrix pentadiagonal and diagonally dominant.
"""
from __future__ import annotations

import math

import torch

from . import CONTIGUOUS, residual_f64, solve_f64, solve_mixed


def operator_bands(v: torch.Tensor, n: int, r: float, coef: float, s_max: float = 800.0,
                   far: str = "linear"):
    """Bands (a, b, c, d, e), each (m, n), of I + coef * L for variances v (m,).
    far="linear" extrapolates linearly beyond S_max; far="drop" drops the
    missing terms (the benchmark generator's convention)."""
    m = v.shape[0]
    dev = v.device
    h = s_max / (n - 1)
    S = torch.arange(n, device=dev, dtype=torch.float64) * h
    diff = 0.5 * v[:, None] * (S * S)[None, :] / (h * h)
    conv = (r * S / (2.0 * h))[None, :].expand(m, n)
    a = torch.zeros(m, n, dtype=torch.float64, device=dev)
    b = coef * diff
    c = 1.0 + coef * (-2.0 * diff - 3.0 * conv - r)
    d = coef * (diff + 4.0 * conv)
    e = coef * (-conv)
    b[:, 0] = 0.0
    if far == "linear" and n >= 4:
        dn1, en1, en2 = d[:, -1].clone(), e[:, -1].clone(), e[:, -2].clone()
        c[:, -1] += 2.0 * dn1 + 3.0 * en1
        b[:, -1] += -dn1 - 2.0 * en1
        d[:, -2] += 2.0 * en2
        c[:, -2] += -en2
    d[:, -1] = 0.0
    e[:, -2:] = 0.0
    return [t.contiguous() for t in (a, b, c, d, e)]


def price_call(K: torch.Tensor, v: torch.Tensor, r: float, T: float, steps: int, n: int = 4096,
               s_max: float = 800.0, theta: float = 0.5, startup: int = 4, solver: str = "mixed",
               tol: float = 1e-12) -> torch.Tensor:
    """European call values u(T, S_i), shape (m, n), for strikes K (m,) and variances v (m,)."""
    m = v.shape[0]
    dev = v.device
    h = s_max / (n - 1)
    S = torch.arange(n, device=dev, dtype=torch.float64) * h
    u = torch.clamp(S[None, :] - K[:, None], min=0.0).contiguous()
    dt = T / steps
    zero = torch.zeros(m * n, dtype=torch.float64, device=dev)
    rhs = torch.empty(m * n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream

    # The operators depend only on (theta, dt): assembled once per pair and
    # reused by every step that has it (all steps after the start-up).
    ops = {}

    def operators(th: float, dtk: float):
        key = (th, dtk)
        if key not in ops:
            A = operator_bands(v, n, r, -th * dtk, s_max)
            negB = [-t for t in operator_bands(v, n, r, (1.0 - th) * dtk, s_max)] if th < 1.0 else None
            ops[key] = (A, negB)
        return ops[key]

    # two solution buffers used in turn: every other step repeats the solver's
    # arguments, so its sweeps run as a replayed graph
    bufs = [torch.empty(m * n, dtype=torch.float64, device=dev) for _ in range(2)]

    def step(th: float, dtk: float, u_flat: torch.Tensor) -> torch.Tensor:
        A, negB = operators(th, dtk)
        x = bufs[1] if u_flat.data_ptr() == bufs[0].data_ptr() else bufs[0]
        if negB is not None:
            residual_f64(*negB, zero, u_flat, rhs, m, n, CONTIGUOUS, stream=stream)   # rhs = B u
            x.copy_(rhs)
        else:
            x.copy_(u_flat)
        if solver == "mixed":
            solve_mixed(*A, x, m, n, CONTIGUOUS, tol=tol, stream=stream, report=False)
        else:
            solve_f64(*A, x, m, n, CONTIGUOUS, stream=stream)
        return x

    u_flat = u.reshape(-1).clone()
    t = 0.0
    k = 0
    # Rannacher start-up: `startup` implicit half steps replace the first startup/2 steps
    for _ in range(startup):
        u_flat = step(1.0, 0.5 * dt, u_flat)
        t += 0.5 * dt
    k = startup // 2
    while k < steps:
        u_flat = step(theta, dt, u_flat)
        k += 1
    return u_flat.reshape(m, n)


def black_scholes_call(S: torch.Tensor, K: float, v: float, r: float, T: float) -> torch.Tensor:
    """Closed-form European call (for tests)."""
    sig = math.sqrt(v)
    Sp = torch.clamp(S, min=1e-300)
    d1 = (torch.log(Sp / K) + (r + 0.5 * v) * T) / (sig * math.sqrt(T))
    d2 = d1 - sig * math.sqrt(T)
    N = lambda z: 0.5 * (1.0 + torch.erf(z / math.sqrt(2.0)))  # noqa: E731
    val = S * N(d1) - K * math.exp(-r * T) * N(d2)
    return torch.where(S > 0, val, torch.zeros_like(S))
