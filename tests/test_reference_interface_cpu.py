"""Host-side interface tests transcribed from the reference's test-suite (CPU).

- Coefficients that the constructors compute from a number, a vector or a
  function (test/DerivativeOperators/coefficient_functions.jl:57-88).
- `size` of `L*Q` (ghost_derivative_operators_interface.jl:1-21).
- The periodic second-order check (2nd_order_check.jl): the oracle's `L2*Q*u`
  and `L1*Q*(L1*Q*u)` against the explicit periodic matrices, and the
  accuracy bounds the reference asserts.

The library's constructors run on the host, so none of this needs a GPU.
"""
import numpy as np
import pytest

import deo
import oracle as O

RTOL = np.sqrt(np.finfo(float).eps)


def _approx(x, y, atol=0.0):
    err = np.linalg.norm(np.ravel(x) - np.ravel(y))
    return err <= max(atol, RTOL * max(np.linalg.norm(np.ravel(x)), np.linalg.norm(np.ravel(y))))


DXV = [1.4, 1.1, 2.3, 3.6, 1.5]


@pytest.mark.parametrize("dx", [1.0, DXV], ids=["uniform", "nonuniform"])
@pytest.mark.parametrize("coeff,expect", [(1.0, np.ones(3)), ([1.0, 2.25, 3.5], [1.0, 2.25, 3.5]),
                                          (np.cos, np.ones(3))], ids=["number", "vector", "function"])
def test_constructor_coefficients(dx, coeff, expect):
    # coefficient_functions.jl:57-80: the coefficients start at zero and
    # compute_coeffs! adds a number or a vector, or maps a function over them
    L = deo.UpwindDifference(1, 1, dx, 3, np.asarray(coeff) if isinstance(coeff, list) else coeff)
    assert _approx(L.coefficients, expect)


def test_zero_coefficient():
    # coefficient_functions.jl:70-71
    assert _approx(deo.UpwindDifference(1, 1, 1.0, 3, 0.0).coefficients + np.ones(3) - np.ones(3), np.zeros(3))
    assert _approx(deo.CenteredDifference(2, 2, 1.0, 3, 0.0).coefficients + np.ones(3) - np.ones(3), np.zeros(3))


def test_ghost_operator_size():
    # ghost_derivative_operators_interface.jl:3-21
    L = deo.CenteredDifference(2, 2, 1.0, 10)
    for Q in (deo.RobinBC((-1.2, 0.3, 0.5), (0.2, 0.5, -30.5), 1.0), deo.PeriodicBC(np.float64)):
        A = L * Q
        assert A.size() == (10, 10)
        assert A.size()[0] * A.size()[1] == 100
        AL, Ab = A.array()
        assert AL.shape == (10, 10) and Ab.shape == (10,)


def test_second_order_periodic_check():
    # 2nd_order_check.jl
    h = 0.025 * np.pi
    N = int(2 * (np.pi / h))
    x = -np.pi + h * np.arange(N)
    L1, L2 = O.centered(1, 2, h, N), O.centered(2, 2, h, N)
    Q = O.periodic()
    u0 = np.cos(x)
    du_true = -np.cos(x)
    M = np.diag(-2.0 * np.ones(N)) + np.diag(np.ones(N - 1), 1) + np.diag(np.ones(N - 1), -1)
    M[-1, 0] = M[0, -1] = 1.0
    M = M / h ** 2
    assert _approx(M @ u0, O.apply([(L2, Q)], u0))
    A = np.zeros((N, N))
    for i in range(N):
        for j in range(N):
            if i == j:
                A[i, j] = -0.5
            if abs(i - j) == 2:
                A[i, j] = 0.25
    A[-2, 0] = A[-1, 1] = A[0, -2] = A[1, -1] = 0.25
    A = A / h ** 2
    du = O.apply([(L1, Q)], O.apply([(L1, Q)], u0))
    assert _approx(A @ u0, du)
    assert np.max(du_true - du) < 0.004
    assert np.max(du_true - O.apply([(L2, Q)], u0)) < 0.001
    # the library's concretisation of L*Q gives the same periodic matrices
    AL, Ab = (deo.CenteredDifference(2, 2, h, N) * deo.PeriodicBC(np.float64)).array()
    assert _approx(AL, M) and not Ab.any()


def _copy_u(c, u, p, t):
    c[:] = u  # the reference's coeff_func(du, u, p, t) = (du .= u)


def test_coefficient_functions_and_updates():
    # f * L keeps the coefficients and stores f (abstract_operator_functions.jl:174-186);
    # update_coefficients!(L, u, p, t) calls f(L.coefficients, u, p, t) (:190-194), also
    # through L*Q and sums (ghost_derivative_operator.jl:61-76); c * L keeps f
    # (derivative_operator_functions.jl:165-197).  The bc_coeff_compositions.jl:52-70 pattern.
    rng = np.random.default_rng(12)
    N = 20
    Q = deo.RobinBC((0.3, 0.6, 0.1), (0.2, 0.4, 0.7), 0.05)
    L = deo.CenteredDifference(4, 4, 0.05, N)
    L1 = deo.UpwindDifference(1, 1, 0.05, N, 1.0)
    for op in (L, L1):
        cL = _copy_u * op
        assert np.array_equal(cL.coefficients, op.coefficients) and cL.coeff_func is _copy_u
        coeffs = rng.random(N)
        v0 = cL._version
        cL.update_coefficients(coeffs, None, 0.0)
        assert np.array_equal(cL.coefficients, coeffs) and cL._version == v0 + 1
        cA = cL * Q
        coeffs = rng.random(N)
        cA.update_coefficients(coeffs, None, 0.0)
        assert np.array_equal(cA.L.coefficients, coeffs)
        assert (2.0 * cL).coeff_func is _copy_u
    A = L * Q
    c2A = _copy_u * A
    coeffs = rng.random(N)
    (c2A + L1 * Q).update_coefficients(coeffs, None, 0.0)
    assert np.array_equal(c2A.L.coefficients, coeffs)
    # an operator without a coefficient function is left as it is
    before = L.coefficients
    L.update_coefficients(coeffs, None, 0.0)
    assert np.array_equal(L.coefficients, before)


def test_coefficients_times_ghost_operator():
    # c * (L*Q) = (c*L)*Q for a number and a vector (ghost_derivative_operator.jl:66-72)
    rng = np.random.default_rng(13)
    L = deo.CenteredDifference(2, 2, 0.1, 12)
    Q = deo.Dirichlet0BC(np.float64)
    c = rng.random(12)
    for k in (2.5, c):
        A = k * (L * Q)
        assert isinstance(A, deo.GhostDerivativeOperator)
        assert np.array_equal(A.L.coefficients, (k * L).coefficients)
        assert np.array_equal(A.array()[0], ((k * L) * Q).array()[0])
    with pytest.raises(deo.DeoShapeError):
        np.ones(5) * (L * Q)
