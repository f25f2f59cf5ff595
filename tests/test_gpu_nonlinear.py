"""GPU: nonlinear_diffusion / nonlinear_diffusion! (derivative_operator.jl:34-77)
against the oracle's restatement and against the reference's fast-diffusion
test problem (test/DerivativeOperators/Fast_Diffusion.jl)."""
import numpy as np
import pytest

import deo
import oracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _dev(x, dtype="f64"):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to("cuda", torch.float64 if dtype == "f64" else torch.float32)


def test_fast_diffusion_rhs(cuda):
    """The reference's fast-diffusion problem at t = 0: k = 1/u^2, Dirichlet
    ghosts u(0) = 1, u(1) = 2^-1/2, n = m = 1, second order: du/dt = d/dx(k du/dx)
    = -(x^2 + 1)^(-3/2) (the analytic solution's time derivative)."""
    n = 100
    h = 1.0 / (n + 1)
    x = np.arange(1, n + 1) * h
    u = 1 / np.sqrt(x ** 2 + 1)
    q = np.r_[1.0, u, 2.0 ** -0.5]
    p = q ** -2.0
    du = deo.nonlinear_diffusion(1, 1, 2, _dev(p), _dev(q), h, n).cpu().numpy()
    assert np.abs(du + (x ** 2 + 1) ** -1.5).max() < 2e-4
    ref = O.nonlinear_diffusion(1, 1, 2, p, q, h, n)
    scale = O.nonlinear_diffusion(1, 1, 2, p, q, h, n, absolute=True)
    assert (np.abs(du - ref) <= 16 * EPS * scale).all()


CASES = [(n, m, a) for n in (1, 2, 3) for m in (0, 1, 2) for a in (2, 4, 6)]


@pytest.mark.parametrize("n,m,a", CASES)
@pytest.mark.parametrize("grid", ["uniform", "nonuniform"])
def test_against_oracle(cuda, n, m, a, grid):
    N = 257
    rng = np.random.default_rng(n * 100 + m * 10 + a)
    dx = 1.0 / (N + 1) if grid == "uniform" else rng.uniform(0.5, 1.5, N + 1) / N
    p = rng.uniform(0.5, 2.0, N + 2)
    q = np.sin(np.linspace(0, 3, N + 2)) + 0.01 * rng.standard_normal(N + 2)
    got = deo.nonlinear_diffusion(n, m, a, _dev(p), _dev(q), dx, N).cpu().numpy()
    ref = O.nonlinear_diffusion(n, m, a, p, q, dx, N)
    scale = O.nonlinear_diffusion(n, m, a, p, q, dx, N, absolute=True)
    assert (np.abs(got - ref) <= 16 * EPS * scale).all(), np.max(np.abs(got - ref) / scale)


def test_float32_error_and_inplace(cuda):
    import torch
    N = 1000
    h = 1.0 / (N + 1)
    rng = np.random.default_rng(5)
    p = rng.uniform(0.5, 2.0, N + 2)
    q = np.cos(np.linspace(0, 5, N + 2))
    ref = O.nonlinear_diffusion(2, 1, 4, p, q, h, N)
    scale = O.nonlinear_diffusion(2, 1, 4, p, q, h, N, absolute=True)
    du = torch.empty(N, device="cuda", dtype=torch.float32)
    deo.nonlinear_diffusion_(du, 2, 1, 4, _dev(p, "f32"), _dev(q, "f32"), h, N)
    rel = np.abs(du.double().cpu().numpy() - ref) / scale
    assert rel.max() < 64 * 2.0 ** -24


def test_errors(cuda):
    N = 32
    p = _dev(np.ones(N + 2))
    with pytest.raises(deo.DeoArgError):
        deo.nonlinear_diffusion(5, 4, 2, p, p, 0.1, N)  # m + n > 8
    with pytest.raises(deo.DeoArgError):
        deo.nonlinear_diffusion(1, 1, 1, p, p, 0.1, N)  # approximation order must be > 1
    with pytest.raises(ValueError):
        deo.nonlinear_diffusion(1, 1, 2, _dev(np.ones(N)), p, 0.1, N)  # p not padded
