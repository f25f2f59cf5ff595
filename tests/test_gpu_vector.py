"""GPU: Gradient / Divergence / Curl and the vector algebra against the
oracle's restatement of the reference's methods (vector_calculus_*.jl,
vector_algebraic_operations.jl), plus the reference's own analytic tests.

Tolerance (Float64): 4 ulp of sum_k |c_k u_k| per output entry (the kernels
fuse each tap's multiply-add; the oracle rounds product and sum separately,
as plain Julia code does).  Float32: within 64 * 2^-24 of that scale against
the Float64 oracle."""
import zlib

import numpy as np
import pytest

import deo
import oracle as O

pytestmark = pytest.mark.gpu


def _dev(x, dtype="f64"):
    import torch
    t = deo.julia_array(x.shape, torch.float64 if dtype == "f64" else torch.float32)
    t.copy_(torch.from_numpy(np.asarray(x, dtype=np.float64)).to(t.dtype))
    return t


def _host(t):
    return t.double().cpu().numpy()


KINDS = {"gradient": (O.GRADIENT, deo.Gradient), "divergence": (O.DIVERGENCE, deo.Divergence),
         "curl": (O.CURL, deo.Curl)}


def _pair(kind, approx, dx, lens, coeff=None):
    """The library operator and the oracle's axis operators of the same definition."""
    ctor = KINDS[kind][1]
    A = ctor(approx, tuple(dx), tuple(lens), coeff if coeff is not None else 1)
    ops = [O.centered(1, approx, dx[a], lens[a], coeff, axis=a + 1) for a in range(len(lens))]
    return A, ops


def _in_shape(kind, lens):
    p = tuple(n + 2 for n in lens)
    return p if kind == "gradient" else p + (len(lens) if kind == "divergence" else 3,)


def _check(kind, A, ops, M, got, init=None, nulp=4.0):
    k = KINDS[kind][0]
    ref = O.vector_calculus(k, ops, M, out=None if init is None else np.asfortranarray(init.copy()),
                            overwrite=init is None)
    scale = O.vector_calculus(k, ops, M, absolute=True)
    if init is not None:
        scale = scale + np.abs(init)
    err = np.abs(got - ref)
    tol = nulp * np.spacing(scale)
    assert (err <= tol).all(), f"max err/ulp {np.max(err / np.spacing(scale))}"


CASES = [
    ("gradient", (9, 7)), ("gradient", (6, 8, 5)), ("gradient", (7,)), ("gradient", (5, 4, 6, 5)),
    ("divergence", (9, 7)), ("divergence", (6, 8, 5)), ("divergence", (5, 6, 4, 5)),
    ("curl", (7, 7, 7)),
]


@pytest.mark.parametrize("kind,lens", CASES)
@pytest.mark.parametrize("approx", [2, 4, 6])
@pytest.mark.parametrize("grid", ["uniform", "nonuniform"])
def test_against_oracle(cuda, kind, lens, approx, grid):
    rng = np.random.default_rng(zlib.crc32(repr((kind, lens, approx, grid)).encode()))
    lens = tuple(max(n, approx + 2) for n in lens)  # room for the boundary rows
    dx = [0.1 * (a + 1) for a in range(len(lens))] if grid == "uniform" else \
        [rng.uniform(0.5, 1.5, n + 1) / n for n in lens]
    A, ops = _pair(kind, approx, dx, lens)
    M = np.asfortranarray(rng.standard_normal(_in_shape(kind, lens)))
    got = _host(A * _dev(M))
    _check(kind, A, ops, M, got)


@pytest.mark.parametrize("kind,lens", [("gradient", (10, 10)), ("divergence", (8, 8, 8)), ("curl", (8, 8, 8))])
def test_mul_accumulates(cuda, kind, lens):
    """mul!(x_temp, .., A, M) adds into x_temp, terms in the reference's order."""
    rng = np.random.default_rng(3)
    dx = [0.05] * len(lens)
    A, ops = _pair(kind, 4, dx, lens)
    M = np.asfortranarray(rng.standard_normal(_in_shape(kind, lens)))
    x0 = np.asfortranarray(rng.standard_normal(A.out_shape()))
    xt = _dev(x0)
    A.mul_(xt, _dev(M))
    _check(kind, A, ops, M, _host(xt), init=x0)


@pytest.mark.parametrize("kind", ["gradient", "divergence", "curl"])
def test_scaled_and_coefficient_vectors(cuda, kind):
    """2 * A, and coeff_func given as a vector (coefficients[i] on every row,
    right boundary rows included)."""
    rng = np.random.default_rng(11)
    n = 9
    lens = (n, n, n)
    c = rng.uniform(0.5, 2.0, n)
    A, ops = _pair(kind, 4, [0.1, 0.2, 0.3], lens, coeff=c)
    M = np.asfortranarray(rng.standard_normal(_in_shape(kind, lens)))
    _check(kind, A, ops, M, _host(A * _dev(M)))
    A2 = 2 * A
    for op in ops:
        op.scale(2.0)
    _check(kind, A2, ops, M, _host(A2 * _dev(M)))


@pytest.mark.parametrize("kind,lens", [("gradient", (40, 33)), ("divergence", (24, 19, 30)), ("curl", (21, 21, 21))])
def test_float32(cuda, kind, lens):
    rng = np.random.default_rng(5)
    dx = [1.0 / (n + 1) for n in lens]
    A, ops = _pair(kind, 4, dx, lens)
    M = np.asfortranarray(rng.standard_normal(_in_shape(kind, lens)))
    got = _host(A * _dev(M, "f32"))
    k = KINDS[kind][0]
    ref = O.vector_calculus(k, ops, M)
    scale = O.vector_calculus(k, ops, M, absolute=True)
    assert (np.abs(got - ref) <= 64 * 2.0 ** -24 * scale).all()


def test_reference_analytic_cases(cuda):
    """The reference's tests on -5:1.25:5 (gradient_operator.jl, divergence_operator.jl,
    curl_operator.jl), uniform and non-uniform dx."""
    X = np.arange(-5.0, 5.0 + 1e-9, 1.25)
    N = len(X) - 2
    XI = X[1:-1]
    for dx in (1.25, 1.25 * np.ones(len(X) - 1)):
        for nd in (2, 3, 4):
            g = np.meshgrid(*([X] * nd), indexing="ij")
            gi = np.meshgrid(*([XI] * nd), indexing="ij")
            G = deo.Gradient(4, (dx,) * nd, (N,) * nd)
            u = _host(G * _dev(np.asfortranarray(sum(a ** 2 for a in g))))
            for a in range(nd):
                assert np.abs(u[..., a] - 2 * gi[a]).max() < 1e-3
            M = np.zeros(g[0].shape + (nd,), order="F")
            for k in range(nd):
                M[..., k] = g[k] ** 2
            D = deo.Divergence(4, (dx,) * nd, (N,) * nd)
            assert np.abs(_host(D * _dev(M)) - 2 * sum(gi)).max() < 1e-3
        x, y, z = np.meshgrid(X, X, X, indexing="ij")
        M = np.stack([y ** 2 + z ** 2, x ** 2 + z ** 2, x ** 2 + y ** 2], axis=-1)
        C = deo.Curl(4, (dx,) * 3, (N,) * 3)
        u = _host(C * _dev(np.asfortranarray(M)))
        xi, yi, zi = np.meshgrid(XI, XI, XI, indexing="ij")
        assert np.abs(u[..., 0] - 2 * (yi - zi)).max() < 1e-3
        assert np.abs(u[..., 1] - 2 * (zi - xi)).max() < 1e-3
        assert np.abs(u[..., 2] - 2 * (xi - yi)).max() < 1e-3
        u2 = _host((2 * C) * _dev(np.asfortranarray(M)))
        assert np.abs(u2 - 2 * u).max() < 1e-3


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_vector_algebra(cuda, dtype):
    """dot / cross / square norm: bit-identical to the oracle's plain-arithmetic
    restatement in Float64 (products rounded before the sums, sqrt correctly
    rounded); Float32 against the same formulas evaluated in float32."""
    rng = np.random.default_rng(9)
    A = np.asfortranarray(rng.standard_normal((11, 6, 7, 3)))
    B = np.asfortranarray(rng.standard_normal((11, 6, 7, 3)))
    if dtype == "f32":
        A32, B32 = A.astype(np.float32), B.astype(np.float32)
        d = np.zeros(A.shape[:-1], np.float32)
        for i in range(3):
            d = d + A32[..., i] * B32[..., i]
        assert np.array_equal(deo.dot_product(_dev(A32, dtype), _dev(B32, dtype)).cpu().numpy(), d)
        return
    assert np.array_equal(_host(deo.dot_product(_dev(A), _dev(B))), O.dot_product(A, B))
    assert np.array_equal(_host(deo.cross_product(_dev(A), _dev(B))), O.cross_product(A, B))
    assert np.array_equal(_host(deo.square_norm(_dev(A))), O.square_norm(A))
    u = _dev(np.zeros((11, 6, 7)))
    deo.dot_product_(u, _dev(A), _dev(B))
    assert np.array_equal(_host(u), O.dot_product(A, B))


def test_errors(cuda):
    G = deo.Gradient(4, (0.1, 0.1), (8, 8))
    with pytest.raises(deo.DeoShapeError):
        G * _dev(np.zeros((8, 8)))  # not padded
    with pytest.raises(AssertionError):
        deo.Curl(4, (0.1,) * 3, (8, 8, 9))
    with pytest.raises(deo.DeoArgError):
        deo.dot_product(_dev(np.zeros((4, 4, 3))), _dev(np.zeros((4, 4, 2))))
    with pytest.raises(deo.DeoArgError):
        deo.dot_product_(_dev(np.zeros((4, 4, 3))), _dev(np.zeros((4, 4, 3))), _dev(np.zeros((4, 4, 3))))
    M = _dev(np.zeros((10, 10)))
    with pytest.raises(deo.DeoShapeError):
        G.mul_(M, M)  # x_temp has the wrong size
    import torch
    buf = torch.zeros(400, dtype=torch.float64, device="cuda")
    Mv = torch.as_strided(buf, (10, 10), (1, 10))
    xv = torch.as_strided(buf, (8, 8, 2), (1, 8, 64), 50)
    with pytest.raises(deo.DeoArgError):
        G.mul_(xv, Mv)  # x_temp overlaps M


@pytest.mark.parametrize("kind", ["gradient", "divergence", "curl"])
def test_full_size_against_oracle(cuda, kind):
    """The benchmark's size (256^3, 4th order, Float64) against the oracle, every
    entry within 4 ulp of its absolute-value scale, and linearity in M."""
    import torch
    n = 256
    A, ops = _pair(kind, 4, [1.0 / (n + 1)] * 3, (n, n, n))
    rng = np.random.default_rng(17)
    M = np.asfortranarray(rng.standard_normal(_in_shape(kind, (n, n, n))))
    Md = _dev(M)
    got = A * Md
    _check(kind, A, ops, M, _host(got))
    # linearity: A(2 M) = 2 A(M) exactly (scaling by 2 is exact in every tap)
    assert torch.equal(A * (2.0 * Md), 2.0 * got)


def test_nonfinite_and_plan_info(cuda):
    """Inf/NaN inputs give the oracle's non-finite pattern (0 * Inf in the
    centre tap included); the uniform 4th-order plan takes the 5-tap marching
    kernel; accumulating applies keep the reference's order."""
    n = 16
    A, ops = _pair("gradient", 4, [0.1, 0.1, 0.1], (n, n, n))
    assert A.info(0) == {"band_nk": 5} and A.info(1) == {"band_nk": 5}
    graded = [0.1 * (1.0 + 0.3 * np.sin(np.arange(n + 1) + a)) for a in range(3)]
    Anu, _ = _pair("gradient", 4, graded, (n, n, n))
    assert Anu.info(0) == {"band_nk": 0}
    rng = np.random.default_rng(3)
    M = np.asfortranarray(rng.standard_normal((n + 2,) * 3))
    M[8, 9, 10] = np.inf
    M[3, 12, 5] = np.nan
    got = _host(A * _dev(M))
    with np.errstate(invalid="ignore"):
        ref = O.vector_calculus(O.GRADIENT, ops, M)
    assert np.array_equal(np.isnan(got), np.isnan(ref)) and np.array_equal(np.isinf(got), np.isinf(ref))
    fin = np.isfinite(ref)
    Mf = np.where(np.isfinite(M), M, 0.0)
    scale = O.vector_calculus(O.GRADIENT, ops, np.asfortranarray(Mf), absolute=True)
    assert (np.abs(got[fin] - ref[fin]) <= 4 * np.spacing(scale[fin])).all()
    x0 = np.asfortranarray(rng.standard_normal(A.out_shape()))
    M2 = np.asfortranarray(rng.standard_normal((n + 2,) * 3))
    xt = _dev(x0)
    A.mul_(xt, _dev(M2))
    _check("gradient", A, ops, M2, _host(xt), init=x0)
