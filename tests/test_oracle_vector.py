"""The oracle's vector-calculus restatement (CPU) against the reference's own
tests (test/DerivativeOperators/gradient_operator.jl, divergence_operator.jl,
curl_operator.jl, vector_algebraic_operations.jl: analytic answers on the grid
-5:1.25:5 checked at atol 1e-3) and against an independent pure-Python loop
restatement of the specialised 2-D methods on a non-separable field (which
the reference's tests, all on separable functions, do not exercise)."""
import numpy as np
import pytest

import oracle as O

X = np.arange(-5.0, 5.0 + 1e-9, 1.25)  # -5:1.25:5
H = 1.25
N = len(X) - 2
XI = X[1:-1]
DX_CASES = [H, H * np.ones(len(X) - 1)]  # uniform, and the non-uniform check of each test


def _ops(nd, dx, approx=4, scale=None):
    ops = [O.centered(1, approx, dx, N, axis=a + 1) for a in range(nd)]
    if scale is not None:
        for op in ops:
            op.scale(scale)
    return ops


def _grid(nd, pts):
    return np.meshgrid(*([pts] * nd), indexing="ij")


@pytest.mark.parametrize("dx", DX_CASES, ids=["uniform", "nonuniform"])
@pytest.mark.parametrize("nd", [2, 3, 4])
def test_gradient_reference_cases(nd, dx):
    """gradient_operator.jl:3-128: grad(sum x_k^2) = 2 x_k e_k."""
    u0 = np.asfortranarray(sum(g ** 2 for g in _grid(nd, X)))
    u = O.vector_calculus(O.GRADIENT, _ops(nd, dx), u0)
    assert u.shape == (N,) * nd + (nd,)
    gi = _grid(nd, XI)
    for a in range(nd):
        assert np.abs(u[..., a] - 2 * gi[a]).max() < 1e-3
    if nd == 3 and np.ndim(dx) == 0:  # 2 * A * u0 (gradient_operator.jl:75-81)
        u1 = O.vector_calculus(O.GRADIENT, _ops(nd, dx, scale=2.0), u0)
        assert np.abs(u1 - 2 * u).max() < 1e-3


@pytest.mark.parametrize("dx", DX_CASES, ids=["uniform", "nonuniform"])
@pytest.mark.parametrize("nd", [2, 3, 4])
def test_divergence_reference_cases(nd, dx):
    """divergence_operator.jl:3-141: div of (x_k^2 + x_{k+1}^2) e_k (2-D: x_k^2 e_k)."""
    g = _grid(nd, X)
    u0 = np.zeros(g[0].shape + (nd,), order="F")
    for k in range(nd):
        u0[..., k] = g[k] ** 2 if nd == 2 else g[k] ** 2 + g[(k + 1) % nd] ** 2
    if nd == 4:  # the 4-D test's fourth component is x^2 + w^2
        u0[..., 3] = g[0] ** 2 + g[3] ** 2
    u = O.vector_calculus(O.DIVERGENCE, _ops(nd, dx), u0)
    gi = _grid(nd, XI)
    assert np.abs(u - 2 * sum(gi)).max() < 1e-3
    if nd == 3 and np.ndim(dx) == 0:
        u1 = O.vector_calculus(O.DIVERGENCE, _ops(nd, dx, scale=2.0), u0)
        assert np.abs(u1 - 2 * u).max() < 1e-3


@pytest.mark.parametrize("dx", DX_CASES, ids=["uniform", "nonuniform"])
def test_curl_reference_case(dx):
    """curl_operator.jl:3-54: curl((y^2+z^2), (x^2+z^2), (x^2+y^2)) = 2(y-z, z-x, x-y)."""
    x, y, z = _grid(3, X)
    u0 = np.zeros(x.shape + (3,), order="F")
    u0[..., 0] = y ** 2 + z ** 2
    u0[..., 1] = x ** 2 + z ** 2
    u0[..., 2] = x ** 2 + y ** 2
    u = O.vector_calculus(O.CURL, _ops(3, dx), u0)
    xi, yi, zi = _grid(3, XI)
    assert np.abs(u[..., 0] - 2 * (yi - zi)).max() < 1e-3
    assert np.abs(u[..., 1] - 2 * (zi - xi)).max() < 1e-3
    assert np.abs(u[..., 2] - 2 * (xi - yi)).max() < 1e-3
    if np.ndim(dx) == 0:
        u1 = O.vector_calculus(O.CURL, _ops(3, dx, scale=2.0), u0)
        assert np.abs(u1 - 2 * u).max() < 1e-3


def test_vector_algebra_reference_case():
    """vector_algebraic_operations.jl test: dot, cross and L2 norm on -5:1.25:5."""
    x, y, z = _grid(3, X)
    u0 = np.stack([x ** 2, y ** 2, z ** 2], axis=-1)
    u1 = np.stack([x, y, z], axis=-1)
    assert np.abs(O.dot_product(u0, u1) - (x ** 3 + y ** 3 + z ** 3)).max() < 1e-3
    c = O.cross_product(u0, u1)
    assert np.abs(c[..., 0] - y * z * (y - z)).max() < 1e-3
    assert np.abs(c[..., 1] - x * z * (z - x)).max() < 1e-3
    assert np.abs(c[..., 2] - x * y * (x - y)).max() < 1e-3
    assert np.abs(O.square_norm(u1) - np.sqrt(x ** 2 + y ** 2 + z ** 2)).max() < 1e-3


def _loops_2d(kind, ops, M):
    """vector_calculus_convolutions.jl:186-328 (gradient) / :330-466 (divergence)
    written out with 1-based loops as the reference has them."""
    s = (ops[0].len, ops[1].len)
    bpc, stl, bstl = ops[0].bpc, ops[0].stl, ops[0].bstl
    mid = stl // 2
    out = np.zeros(s + ((2,) if kind == O.GRADIENT else ()), order="F")
    tabs = [op.tables() for op in ops]
    coef = [t[3] for t in tabs]

    def x(p, q, comp):  # 1-based padded index
        return M[p - 1, q - 1] if kind == O.GRADIENT else M[p - 1, q - 1, comp]

    def add(i, j, comp, v):
        if kind == O.GRADIENT:
            out[i - 1, j - 1, comp] += v
        else:
            out[i - 1, j - 1] += v

    st = lambda a, i: tabs[a][0][0][0] if ops[a].uniform else tabs[a][0][0][i - bpc - 1]
    for j in range(1, s[1] + 1):  # BC_left, axis 1
        for i in range(1, bpc + 1):
            add(i, j, 0, sum(coef[0][i - 1] * tabs[0][1][0][i - 1][k - 1] * x(k, j, 0) for k in range(1, bstl + 1)))
    for j in range(1, bpc + 1):  # BC_left, axis 2
        for i in range(1, s[0] + 1):
            add(i, j, 1, sum(coef[1][j - 1] * tabs[1][1][0][j - 1][k - 1] * x(i, k, 1) for k in range(1, bstl + 1)))
    for j in range(1, s[1] + 1):  # interior, axis 1
        for i in range(1 + bpc, s[0] - bpc + 1):
            add(i, j, 0, sum(coef[0][i - 1] * st(0, i)[k - 1] * x(i + k - mid, j, 0) for k in range(1, stl + 1)))
    for j in range(1 + bpc, s[1] - bpc + 1):  # interior, axis 2
        for i in range(1, s[0] + 1):
            add(i, j, 1, sum(coef[1][j - 1] * st(1, j)[k - 1] * x(i, j + k - mid, 1) for k in range(1, stl + 1)))
    for j in range(1, s[1] + 1):  # BC_right, axis 1
        for i in range(s[0] - bpc + 1, s[0] + 1):
            hi = tabs[0][2][0][i - s[0] + bpc - 1]
            add(i, j, 0, sum(coef[0][i - 1] * hi[k - 1] * x(s[0] - bstl + k + 2, j, 0) for k in range(1, bstl + 1)))
    for j in range(s[1] - bpc + 1, s[1] + 1):  # BC_right, axis 2
        for i in range(1, s[0] + 1):
            hi = tabs[1][2][0][j - s[1] + bpc - 1]
            add(i, j, 1, sum(coef[1][j - 1] * hi[k - 1] * x(i, s[1] - bstl + k + 2, 1) for k in range(1, bstl + 1)))
    return out


@pytest.mark.parametrize("kind", [O.GRADIENT, O.DIVERGENCE])
@pytest.mark.parametrize("grid", ["uniform", "nonuniform"])
def test_specialised_2d_against_loops(kind, grid):
    """The C++ restatement against the loops above on a non-separable random
    field with varying coefficients: same values to rounding (the loops sum
    with Python's left-to-right order too)."""
    rng = np.random.default_rng(7 + kind)
    n1, n2 = 9, 7
    dx = [0.3, 0.2] if grid == "uniform" else [rng.uniform(0.5, 1.5, n1 + 1), rng.uniform(0.5, 1.5, n2 + 1)]
    ops = [O.centered(1, 4, dx[0], n1, axis=1), O.centered(1, 4, dx[1], n2, axis=2)]
    ops[0].set_coefficients(rng.uniform(0.5, 2.0, n1))
    ops[1].set_coefficients(rng.uniform(0.5, 2.0, n2))
    shape = (n1 + 2, n2 + 2) + (() if kind == O.GRADIENT else (2,))
    M = np.asfortranarray(rng.standard_normal(shape))
    got = O.vector_calculus(kind, ops, M)
    want = _loops_2d(kind, ops, M)
    assert np.allclose(got, want, rtol=1e-13, atol=1e-13)


def test_specialised_indexing_is_reproduced():
    """On a field that varies along y, the 2-D gradient's x-derivative at output
    (i, j) is taken along padded row j (the reference's x[i + idx - mid, j]),
    so it equals the derivative at the grid's y[j], not y[j + 1]."""
    xs = np.linspace(0.0, 1.0, 12)
    ys = np.linspace(0.0, 2.0, 10)
    M = np.asfortranarray(xs[:, None] ** 2 * ys[None, :])
    h1, h2 = xs[1] - xs[0], ys[1] - ys[0]
    ops = [O.centered(1, 4, h1, 10, axis=1), O.centered(1, 4, h2, 8, axis=2)]
    g = O.vector_calculus(O.GRADIENT, ops, M)
    # second-order exact stencils: d/dx (x^2 y) = 2 x y
    np.testing.assert_allclose(g[:, :, 0], 2 * xs[1:-1, None] * ys[None, :-2], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(g[:, :, 1], xs[:-2, None] ** 2 * np.ones((1, 8)), rtol=1e-9, atol=1e-9)


def test_errors():
    ops = _ops(2, H)
    with pytest.raises(AssertionError):
        O.vector_calculus(O.CURL, ops, np.zeros((N + 2, N + 2, 3)))  # Curl needs 3 axes
