"""The reference's KdV single-soliton example (test/DerivativeOperators/KdV.jl:4-70).

du/dt = A * bc(t) * u with A = UpwindDifference(1, 3, dx, 401, -1) (no offside,
offside = 1, and offside = 1 on a Vector dx), x = -10:1/20:10, and the
order-3 GeneralBC([0, 1, -6 phi(+-10, t), 0, -1], ...) rebuilt at every stage
time; the solution stays within atol 0.01 (isapprox: the 2-norm) of the
travelling profile phi(x, t) = sech((x - t)/2)^2 / 2 for t in 0:0.5:5.  The
reference integrates with Tsit5 (OrdinaryDiffEq, not vendored); here the
oracle's applies advance the restated SSP-RK3 scheme with the BC evaluated
at each stage's time.  The GPU test checks the library's right-hand side
against the oracle's on the same states.
"""
import numpy as np
import pytest

import oracle as O

N = 401
DX = 1.0 / 20  # x = -10:1/20:10 (Δx = 1/(N-1) with N = 21 in the reference)
X = -10.0 + DX * np.arange(N)


def phi(x, t):
    return 0.5 / np.cosh((x - t) / 2) ** 2


def _bc_oracle(t):
    return O.general([0.0, 1.0, -6 * phi(-10.0, t), 0.0, -1.0], [0.0, 1.0, -6 * phi(10.0, t), 0.0, -1.0], DX, 3)


def _operators():
    return {"offside0": O.upwind(1, 3, DX, N, -1.0),
            "offside1": O.upwind(1, 3, DX, N, -1.0, offside=1),
            "offside1_vector_dx": O.upwind(1, 3, DX * np.ones(N + 1), N, -1.0, offside=1)}


def _rhs(A, u, t):
    return O.apply([(A, _bc_oracle(t))], u)


@pytest.mark.parametrize("name", ["offside0", "offside1", "offside1_vector_dx"])
def test_kdv_single_soliton_accuracy(name):
    A = _operators()[name]
    # a fixed step well inside SSP-RK3's stability bound for the stiff order-3 boundary
    # closure (the reference's Tsit5 adapts its step to tolerance 1e-6)
    dt = 0.1 * DX
    u = phi(X, 0.0)
    t = 0.0
    for t_check in np.arange(0.0, 5.0 + 1e-12, 0.5):
        n = int(round((t_check - t) / dt))
        h = (t_check - t) / n if n else 0.0
        for _ in range(n):
            u1 = u + h * _rhs(A, u, t)
            u2 = 0.75 * u + 0.25 * (u1 + h * _rhs(A, u1, t + h))
            u = (1.0 / 3.0) * u + (2.0 / 3.0) * (u2 + h * _rhs(A, u2, t + 0.5 * h))
            t += h
        t = t_check
        assert np.linalg.norm(u - phi(X, t)) <= 0.01, (t, np.linalg.norm(u - phi(X, t)))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["offside0", "offside1", "offside1_vector_dx"])
def test_kdv_right_hand_side_on_gpu(cuda, name):
    import torch

    import deo
    dx = DX * np.ones(N + 1) if name == "offside1_vector_dx" else DX
    off = 0 if name == "offside0" else 1
    L = deo.UpwindDifference(1, 3, dx, N, -1.0, offside=off)
    Ao = _operators()[name]
    rng = np.random.default_rng(3)
    for t in (0.0, 1.25, 3.5):
        bc = deo.GeneralBC([0.0, 1.0, -6 * phi(-10.0, t), 0.0, -1.0], [0.0, 1.0, -6 * phi(10.0, t), 0.0, -1.0], DX, 3)
        u = phi(X, t) + 1e-3 * rng.standard_normal(N)
        got = (L * bc * torch.from_numpy(u).to("cuda")).cpu().numpy()
        terms = [(Ao, _bc_oracle(t))]
        ref = O.apply(terms, u)
        assert (np.abs(got - ref) <= 4 * np.spacing(O.abs_scale(terms, u))).all()
