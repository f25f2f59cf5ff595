"""GPU: A \\ u (ghost_derivative_operator.jl:39-58) -- the banded LU of A_l
applied to every line -- against the oracle's dense restatement and the
reference's own left-division known answers.  Parity bar (the reference's own,
bc_coeff_compositions.jl:488): ||x - x_oracle|| / ||x_oracle|| < cond(A_l) * eps
(Float64); Float32 lines are solved in Float64 and rounded once."""
import zlib

import numpy as np
import pytest

import deo
import oracle as O

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _dev(x, dtype="f64"):
    import torch
    t = deo.julia_array(np.shape(x), torch.float64 if dtype == "f64" else torch.float32)
    t.copy_(torch.from_numpy(np.asarray(x, dtype=np.float64)).to(t.dtype))
    return t


def _host(t):
    return t.double().cpu().numpy()


DX = 0.01
X = np.arange(1, 100) * DX
N = len(X)


def test_reference_left_division_cases(cuda):
    """bc_coeff_compositions.jl:346-448: f'' = -2 with Dirichlet RobinBCs (0 and 4)
    gives the quadratics exactly; the matrix versions go through MultiDimBC{1}."""
    L = deo.CenteredDifference(2, 2, DX, N)
    for g in (0.0, 4.0):
        f = -X ** 2 + X + g
        Q = deo.RobinBC((1.0, 0.0, g), (1.0, 0.0, g), DX)
        x = _host(deo.ldiv(L * Q, _dev(np.full(N, -2.0))))
        assert np.allclose(x, f, rtol=1e-8, atol=1e-8)
        M = np.stack([np.full(N, -2.0), np.full(N, -4.0), np.full(N, -20.0)], axis=1)
        Qx = deo.MultiDimBC(Q, M.shape, 1)
        xm = _host(deo.ldiv(L * Qx, _dev(M)))
        want = np.stack([f, 2.0 * (f - g) + g, 10.0 * (f - g) + g], axis=1)
        assert np.allclose(xm, want, rtol=1e-8, atol=1e-8)


BCS = ["dirichlet0", "dirichlet", "robin", "general"]


def _bcs(name, dx, order):
    if name == "dirichlet0":
        return deo.Dirichlet0BC(), O.dirichlet0()
    if name == "dirichlet":
        return deo.DirichletBC(1.5, -0.5), O.dirichlet(1.5, -0.5)
    if name == "robin":
        l, r = (1.0, 0.3, 0.2), (0.7, 0.4, -0.1)
        return deo.RobinBC(l, r, dx, order), O.robin(l, r, dx, order)
    al, ar = [0.3, 1.0, 0.2], [-0.1, 0.8, 0.5]
    return deo.GeneralBC(al, ar, dx, order), O.general(al, ar, dx, order)


OPS = [("centred", d, a, 1.0) for d in (1, 2) for a in (2, 4)] + \
      [("upwind", 1, a, c) for a in (1, 2) for c in (1.0, -1.0)]
CASES = [op + (bc, grid) for op in OPS for bc in BCS for grid in ("uniform", "nonuniform")]


@pytest.mark.parametrize("kind,d,a,c,bc,grid", CASES)
def test_1d_against_oracle(cuda, kind, d, a, c, bc, grid):
    rng = np.random.default_rng(zlib.crc32(repr((kind, d, a, c, bc, grid)).encode()))
    n = 64
    dx = 1.0 / (n + 1) if grid == "uniform" else rng.uniform(0.5, 1.5, n + 1) / n
    order = a if bc != "general" else 2
    Qd, Qo = _bcs(bc, dx, order)
    if kind == "centred":
        L, Lo = deo.CenteredDifference(d, a, dx, n), O.centered(d, a, dx, n)
    else:
        L, Lo = deo.UpwindDifference(d, a, dx, n, c), O.upwind(d, a, dx, n, c)
    u = rng.standard_normal(n)
    try:
        ref, cond = O.ghost_solve(Lo, Qo, u)
    except np.linalg.LinAlgError:
        ref, cond = None, np.inf
    if not cond < 1e12:  # (near-)singular A_l: the reference's LU fails too
        pytest.skip("singular or ill-conditioned A_l")
    x = _host(deo.ldiv(L * Qd, _dev(u)))
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < max(cond, 1.0) * EPS * 16


@pytest.mark.parametrize("shape,axis", [((48, 40), 1), ((48, 40), 2), ((24, 20, 28), 1), ((24, 20, 28), 2),
                                        ((24, 20, 28), 3)])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_nd_lines_against_oracle(cuda, shape, axis, dtype):
    rng = np.random.default_rng(len(shape) * 10 + axis)
    n = shape[axis - 1]
    h = 1.0 / (n + 1)
    l, r = (1.0, 0.5, 0.3), (1.0, -0.2, 0.1)
    L = deo.CenteredDifference(2, 4, h, n, axis=axis)
    Q = deo.MultiDimBC(deo.RobinBC(l, r, h, 4), shape, axis)
    u = np.asfortranarray(rng.standard_normal(shape))
    ref, cond = O.ghost_solve(O.centered(2, 4, h, n), O.robin(l, r, h, 4), u, axis=axis)
    x = _host(deo.ldiv(L * Q, _dev(u, dtype)))
    rel = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    assert rel < (cond * EPS * 16 if dtype == "f64" else 1e-6 + cond * 2.0 ** -24 * 4)
    # A (A \ u) = u through the apply (same affine map for constant coefficients)
    if dtype == "f64":
        back = _host((L * Q) * _dev(x))
        assert np.linalg.norm(back - u) / np.linalg.norm(u) < 1e-9


def test_in_place_and_host_plan(cuda):
    n = 100
    h = 1.0 / (n + 1)
    A = deo.CenteredDifference(2, 2, h, n) * deo.Dirichlet0BC()
    rng = np.random.default_rng(2)
    u = rng.standard_normal(n)
    ref, _ = O.ghost_solve(O.centered(2, 2, h, n), O.dirichlet0(), u)
    t = _dev(u)
    A.ldiv(t, x=t)  # in place
    assert np.allclose(_host(t), ref, rtol=1e-10, atol=1e-12)
    p = deo.solve_plan_for(A, (n,), 0)
    assert p.bands() == (1, 1)


def test_singular_operators_raise(cuda):
    """An exactly singular A_l (a zero pivot, where the reference's LU throws
    SingularException): [1 -2 1] with first-order Neumann ghosts on a unit grid
    eliminates in integers down to a last pivot of 0.  (Numerically singular
    matrices without an exact zero pivot factor, as they do in the reference.)"""
    n = 32
    L = deo.CenteredDifference(2, 2, 1.0, n)
    with pytest.raises(deo.DeoArgError):
        deo.ldiv(L * deo.Neumann0BC(1.0, 1), _dev(np.ones(n)))   # constants in the null space
    with pytest.raises(deo.DeoShapeError):
        deo.ldiv(L * deo.Dirichlet0BC(), _dev(np.ones(n + 1)))


def test_full_size_residual_and_oracle(cuda):
    """256^3 along axis 2 (the benchmark's size): against the oracle's dense
    solve of every line, and A (A \\ u) = u through the apply."""
    n = 256
    h = 1.0 / (n + 1)
    shape = (n, n, n)
    l, r = (1.0, 0.5, 0.0), (1.0, 0.5, 0.0)
    L = deo.CenteredDifference(2, 2, h, n, axis=2)
    A = L * deo.MultiDimBC(deo.RobinBC(l, r, h, 2), shape, 2)
    u = np.asfortranarray(np.random.default_rng(23).standard_normal(shape))
    x = deo.ldiv(A, _dev(u))
    ref, cond = O.ghost_solve(O.centered(2, 2, h, n), O.robin(l, r, h, 2), u, axis=2)
    xh = _host(x)
    assert np.linalg.norm(xh - ref) / np.linalg.norm(ref) < 16 * cond * EPS
    back = _host(A * x)
    assert np.linalg.norm(back - u) / np.linalg.norm(u) < 1e-9


def test_poisson_example(cuda):
    """test/DerivativeOperators/poisson.jl on the GPU: (Δ * DirichletBC(-1, 2)) \\ 1."""
    n = 10
    h = 1.0 / (n + 1)
    x = h * np.arange(1, n + 1)
    ua = 0.5 * x ** 2 + (2.0 + 1.0 - 0.5) * x - 1.0
    u = _host(deo.ldiv(deo.CenteredDifference(2, 2, h, n) * deo.DirichletBC(-1.0, 2.0), _dev(np.ones(n))))
    assert np.allclose(u, ua, rtol=1e-12, atol=1e-12)
