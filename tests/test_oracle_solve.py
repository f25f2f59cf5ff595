"""The oracle's A \\ u restatement (CPU) against the reference's own left-division
known answers (test/DerivativeOperators/bc_coeff_compositions.jl:346-448:
CenteredDifference(2, 2, 0.01, 99) with Dirichlet RobinBCs, right-hand side
f'' = -2, whose solutions are the quadratics f exactly)."""
import numpy as np

import oracle as O

DX = 0.01
X = np.arange(1, 100) * DX  # dx:dx:(1 - dx)
N = len(X)


def test_homogeneous_dirichlet():
    f = -X ** 2 + X
    L = O.centered(2, 2, DX, N)
    Q = O.robin((1.0, 0.0, 0.0), (1.0, 0.0, 0.0), DX)
    x, cond = O.ghost_solve(L, Q, np.full(N, -2.0))
    assert np.allclose(x, f, rtol=1e-8, atol=1e-10)
    # the matrix case: each column along axis 1 (MultiDimBC{1})
    M = np.asfortranarray(np.stack([np.full(N, -2.0)] * 2, axis=1))
    xm, _ = O.ghost_solve(L, Q, M, axis=1)
    assert np.allclose(xm, np.stack([f, f], axis=1), rtol=1e-8, atol=1e-10)


def test_inhomogeneous_dirichlet():
    f = -X ** 2 + X + 4.0
    L = O.centered(2, 2, DX, N)
    Q = O.robin((1.0, 0.0, 4.0), (1.0, 0.0, 4.0), DX)
    x, _ = O.ghost_solve(L, Q, np.full(N, -2.0))
    assert np.allclose(x, f, rtol=1e-8, atol=1e-9)
    M2 = np.asfortranarray(np.stack([np.full(N, -2.0), np.full(N, -4.0), np.full(N, -20.0)], axis=1))
    xm, _ = O.ghost_solve(L, Q, M2, axis=1)
    want = np.stack([f, 2.0 * (f - 4.0) + 4.0, 10.0 * (f - 4.0) + 4.0], axis=1)
    assert np.allclose(xm, want, rtol=1e-8, atol=1e-8)


def test_fourth_order_consistency():
    """bc_coeff_compositions.jl:450-494: CenteredDifference(4, 4, 0.01, 20) with
    RobinBC((1,0,0), (1,0,sin(0.2+dx))): the solve reproduces u = A_l x + A_b."""
    x = np.arange(1, 21) * DX
    u = np.sin(x)
    L = O.centered(4, 4, DX, len(x))
    Q = O.robin((1.0, 0.0, 0.0), (1.0, 0.0, np.sin(0.2 + DX)), DX)
    sol, cond = O.ghost_solve(L, Q, u)
    Al = L.array() @ Q.array(len(x))[0]
    Ab = L.array() @ Q.array(len(x))[1]
    assert np.linalg.norm(Al @ sol + Ab - u) / np.linalg.norm(u) < cond * np.finfo(float).eps


def test_poisson_example():
    """test/DerivativeOperators/poisson.jl: (Δ * DirichletBC(-1, 2)) \\ fill(1.0, 10)
    equals u(x) = x^2/2 + (b - a - 1/2) x + a on the knots."""
    n = 10
    h = 1.0 / (n + 1)
    x = h * np.arange(1, n + 1)
    ua = 0.5 * x ** 2 + (2.0 + 1.0 - 0.5) * x - 1.0
    u, _ = O.ghost_solve(O.centered(2, 2, h, n), O.dirichlet(-1.0, 2.0), np.ones(n))
    assert np.allclose(u, ua, rtol=1e-12, atol=1e-12)
