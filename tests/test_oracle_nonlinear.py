"""The oracle's nonlinear_diffusion (derivative_operator.jl:34-66) on the
reference's fast-diffusion problem (test/DerivativeOperators/Fast_Diffusion.jl,
CPU): du/dt = d/dx(u^-2 du/dx) on 100 knots with the time-dependent Dirichlet
ghosts u(0) = exp(-t), u(1) = (1 + exp(2t))^-1/2, evaluated on the analytic
solution u = (x^2 + exp(2t))^-1/2 at t in 0:0.1:1, matches its analytic time
derivative -exp(2t) (x^2 + exp(2t))^-3/2 to the second-order truncation error
(below 1e-4 of its size; the reference integrates to rtol 1e-3 with
KenCarp4).  Higher orders converge: approximation order 4 cuts the error by
more than 10x."""
import numpy as np
import pytest

import oracle as O


def _rhs_error(t, approx, nknots=100):
    h = 1.0 / (nknots + 1)
    x = np.arange(1, nknots + 1) * h
    u = 1 / np.sqrt(x ** 2 + np.exp(2 * t))
    q = np.r_[np.exp(-t), u, (1 + np.exp(2 * t)) ** -0.5]  # l = bc * u
    p = q ** -2.0                                          # k = l .^ (-2)
    du = O.nonlinear_diffusion(1, 1, approx, p, q, h, nknots)
    exact = -np.exp(2 * t) * (x ** 2 + np.exp(2 * t)) ** -1.5
    return np.abs(du - exact).max() / np.abs(exact).max()


@pytest.mark.parametrize("t", np.round(np.arange(0.0, 1.0001, 0.1), 1))
def test_fast_diffusion_rhs_along_the_solution(t):
    assert _rhs_error(t, 2) < 1e-4


def test_fast_diffusion_rhs_converges_with_order():
    assert _rhs_error(0.5, 4) < _rhs_error(0.5, 2) / 10
