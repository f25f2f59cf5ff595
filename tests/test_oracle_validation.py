"""The oracle against more of the reference's own tests (CPU).

- Biased upwind with the largest offside concretises as the centred operator
  of the same order, on regular and irregular grids and for both wind signs
  (test/DerivativeOperators/concretization.jl:134-361).
- `L * bc * M` equals `L * (Q_L * M + Q_b)` with `(Q_L, Q_b) = Array(bc, N)`
  for the six BC kinds (concretization.jl:362-405).
- Centred operators differentiate sin/cos to the accuracy the reference asserts
  on regular grids (regular_operator_validation.jl) and irregular grids
  (generic_operator_validation.jl).

The reference compares with Julia's `isapprox`: for vectors and matrices with
an `atol`, `norm(x - y) <= atol` (2-norm / Frobenius norm); without one,
`norm(x - y) <= sqrt(eps) * max(norm(x), norm(y))`.  The same checks are
written here.
"""
import numpy as np
import pytest

import oracle as O
from transcribe_reference import IRR_DX

RTOL = np.sqrt(np.finfo(float).eps)  # isapprox's default relative tolerance


def _approx(x, y, atol=None):
    err = np.linalg.norm(np.ravel(x) - np.ravel(y))
    if atol is not None:
        return err <= atol
    return err <= RTOL * max(np.linalg.norm(np.ravel(x)), np.linalg.norm(np.ravel(y)))


# (d, a, offside) pairs: CenteredDifference(d, a) against UpwindDifference(d, a, offside)
REGULAR_PAIRS = [(1, 2, 1), (1, 4, 2), (1, 6, 3), (2, 3, 2), (3, 4, 3)]
IRREGULAR_PAIRS = [(1, 2, 1), (1, 4, 2), (2, 3, 2)]


@pytest.mark.parametrize("wind", [1.0, -1.0])
@pytest.mark.parametrize("d,a,off", REGULAR_PAIRS)
def test_biased_upwind_is_centred_regular_grid(d, a, off, wind):
    # concretization.jl:134-268
    rng = np.random.default_rng(100 + 10 * d + a)
    n = 20
    L = O.centered(d, a, 1.0, n, coeff=None if wind > 0 else wind)
    K = O.upwind(d, a, 1.0, n, coeff=None if wind > 0 else wind, offside=off)
    M = rng.random(n + 2)
    AL, AK = L.array(), K.array()
    assert _approx(AL, AK)
    assert _approx(L.mul_generic(M), AL @ M)
    assert _approx(K.mul_generic(M), AK @ M)
    assert _approx(L.mul_generic(M), K.mul_generic(M))
    if wind > 0:
        # P = PeriodicBC(Float64) * M[2:21]: the padded path (convolutions.jl:367-730)
        u = M[1:-1]
        P = np.concatenate([[u[-1]], u, [u[0]]])
        assert _approx(L.mul_padded(u[-1], u, u[0]), AL @ P)
        assert _approx(K.mul_padded(u[-1], u, u[0]), AK @ P)
    # N-D: M = rand(22, 2, 2, 2, 2), the operator along axis 1 of every line
    M5 = np.asfortranarray(rng.random((n + 2, 2, 2, 2, 2)))
    yL, yK = O.mul_nd(L, M5), O.mul_nd(K, M5)
    lines = M5.reshape(n + 2, -1, order="F")
    assert _approx(yL.reshape(n, -1, order="F"), AL @ lines)
    assert _approx(yL, yK)


@pytest.mark.parametrize("wind", [1.0, -1.0])
@pytest.mark.parametrize("d,a,off", IRREGULAR_PAIRS)
def test_biased_upwind_is_centred_irregular_grid(d, a, off, wind):
    # concretization.jl:270-361, grid dx = [0.08, 0.02, 0.05, 0.04, 0.07, 0.03]
    rng = np.random.default_rng(200 + 10 * d + a)
    n = 5
    L = O.centered(d, a, IRR_DX, n, coeff=None if wind > 0 else wind)
    K = O.upwind(d, a, IRR_DX, n, coeff=None if wind > 0 else wind, offside=off)
    M = rng.random(n + 2)
    AL, AK = L.array(), K.array()
    assert _approx(AL, AK)
    assert _approx(L.mul_generic(M), K.mul_generic(M))
    assert _approx(K.mul_generic(M), AK @ M)
    if wind > 0:
        u = M[1:-1]
        P = np.concatenate([[u[-1]], u, [u[0]]])
        assert _approx(K.mul_padded(u[-1], u, u[0]), AL @ P)
    M4 = np.asfortranarray(rng.random((n + 2, 2, 2, 2)))
    assert _approx(O.mul_nd(L, M4), O.mul_nd(K, M4))
    assert _approx(O.mul_nd(K, M4).reshape(n, -1, order="F"), AK @ M4.reshape(n + 2, -1, order="F"))


def _bc_cases(M2):
    """The six BCs of concretization.jl:362-379, built from M2 = rand(11)."""
    L2 = O.centered(1, 2, 1.0, 9)
    dM = L2.mul_generic(M2)
    deriv_start, deriv_end = dM[0], dM[-1]
    M = M2[1:10]
    p1, p2 = 1.0, 0.5
    left = p1 * M[0] - p2 * deriv_start
    right = p1 * M[-1] + p2 * deriv_end
    return M, {
        "Dirichlet0BC": O.dirichlet0(),
        "DirichletBC": O.dirichlet(0.0, 0.0),
        "NeumannBC": O.neumann((deriv_start, deriv_end), 1.0, 1),
        "RobinBC": O.robin((p1, -p2, left), (p1, p2, right), 1.0, 1),
        "GeneralBC": O.general([-left, p1, -p2], [-right, p1, p2], 1.0, 1),
        "PeriodicBC": O.periodic(),
    }


@pytest.mark.parametrize("name", ["Dirichlet0BC", "DirichletBC", "NeumannBC", "RobinBC", "GeneralBC",
                                  "PeriodicBC"])
def test_bc_concretisation(name):
    # concretization.jl:362-405: L1 * bc * M == L1 * (Array(bc)[1] * M + Array(bc)[2])
    rng = np.random.default_rng(362)
    M, bcs = _bc_cases(rng.random(11))
    bc = bcs[name]
    L1 = O.centered(2, 2, 1.0, 9)
    QL, Qb = bc.array(len(M))
    lhs = O.apply([(L1, bc)], M)
    rhs = L1.array() @ (QL @ M + Qb)
    assert _approx(lhs, rhs)
    # the ghosts the BC fills are Q's first and last rows
    l, r = bc.ghosts(M)
    assert _approx([l, r], [(QL @ M + Qb)[0], (QL @ M + Qb)[-1]])


@pytest.mark.parametrize("dor", range(1, 7))
@pytest.mark.parametrize("aor", [2, 4, 6, 8, 10])
def test_regular_operator_validation(dor, aor):
    # regular_operator_validation.jl: sin on 200 points of [0, 2pi]
    nx = 200
    x = np.linspace(0.0, 2 * np.pi, nx)
    dx = x[1] - x[0]
    y = np.sin(x)
    dy = [np.cos(x), -np.sin(x), -np.cos(x), y, np.cos(x), -np.sin(x)]
    D1 = O.centered(dor, aor, dx, nx - 2)
    assert _approx(dy[dor - 1][1:-1], D1.mul_generic(y), atol=1.0 ** (1 - aor))


def _grid_0_pi():
    n = int(np.floor(np.pi / 0.01)) + 1  # 0.0:0.01:pi
    return np.arange(n) * 0.01


@pytest.mark.parametrize("dor", range(1, 5))
@pytest.mark.parametrize("aor", [2, 4, 6])
def test_irregular_constructor_on_regular_grid_matches_uniform(dor, aor):
    # generic_operator_validation.jl:10-19
    x = _grid_0_pi()
    dx = np.diff(x)
    Dr = O.centered(dor, aor, 0.01, len(x) - 2)
    Dir = O.centered(dor, aor, dx, len(x) - 2)
    assert _approx(Dr.array(), Dir.array())


@pytest.mark.parametrize("dor", range(1, 5))
@pytest.mark.parametrize("aor", range(2, 7))
def test_irregular_operator_on_regular_grid(dor, aor):
    # generic_operator_validation.jl:21-32: y = sin(2x) on 0.0:0.01:pi
    x = _grid_0_pi()
    dx = np.diff(x)
    y = np.sin(2 * x)
    xi = x[1:-1]
    dy = [2 * np.cos(2 * xi), -4 * np.sin(2 * xi), -8 * np.cos(2 * xi), 16 * y[1:-1]]
    D1 = O.centered(dor, aor, dx, len(x) - 2)
    assert _approx(D1.mul_generic(y), dy[dor - 1], atol=10.0 ** (1 - aor))


@pytest.mark.parametrize("dor", range(1, 5))
@pytest.mark.parametrize("aor", range(4, 11))
def test_irregular_grid_operator_validation(dor, aor):
    # generic_operator_validation.jl:34-56: x = cumsum(sin(0:0.05:pi)) scaled to [0, pi]
    s = np.sin(np.arange(int(np.floor(np.pi / 0.05)) + 1) * 0.05)
    x = np.cumsum(s)
    x = x / x[-1] * np.pi
    dx = np.diff(x)
    y = np.sin(2 * x)
    xi = x[1:-1]
    dy = [2 * np.cos(2 * xi), -4 * np.sin(2 * xi), -8 * np.cos(2 * xi), 16 * y[1:-1]]
    D1 = O.centered(dor, aor, dx, len(x) - 2)
    tol = 2 * 10.0 ** (2 - aor) * dx.max() ** (2 - dor)
    assert _approx(D1.mul_generic(y), dy[dor - 1], atol=tol)
