"""The oracle against the reference's own known answers (CPU)."""
import numpy as np
import pytest

import oracle as O
from transcribe_reference import CENTRED_CASES, IRR_DX, UPWIND_CASES

FX = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "reference_fixtures.npz"))
RNG = np.random.default_rng(1234)


@pytest.mark.parametrize("d,a,dx,n,key,rows", CENTRED_CASES)
def test_centred_matrices(d, a, dx, n, key, rows):
    L = O.centered(d, a, IRR_DX if dx == "irr" else dx, n)
    ref = FX[key]
    A = L.array()
    x = RNG.random(n + 2)
    y = L.mul_generic(x)  # L*x on a padded Vector (convolutions.jl:17-22)
    if rows:
        A, y = A[rows[0]:rows[1]], y[rows[0]:rows[1]]
    np.testing.assert_allclose(A, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(y, ref @ x, rtol=1e-12, atol=1e-12 * np.abs(ref @ x).max())
    # L*Q*u on a BoundaryPaddedVector agrees with the matrix (test/.../convolutions.jl:45-81)
    yp = L.mul_padded(x[0], x[1:-1], x[-1])
    if rows:
        yp = yp[rows[0]:rows[1]]
    np.testing.assert_allclose(yp, ref @ x, rtol=1e-12, atol=1e-12 * np.abs(ref @ x).max())


@pytest.mark.parametrize("name,d,a,dx,n,c,key,mult", UPWIND_CASES)
def test_upwind_matrices(name, d, a, dx, n, c, key, mult):
    L = O.upwind(d, a, IRR_DX if dx == "irr" else dx, n, c)
    ref = mult * FX[key]
    x = RNG.random(n + 2)
    y = L.mul_generic(x)
    scale = np.abs(ref @ x).max()
    np.testing.assert_allclose(y, ref @ x, rtol=1e-12, atol=1e-12 * scale)
    u = x[:n]
    xp = np.concatenate([[u[-1]], u, [u[0]]])  # PeriodicBC(Float64) * x[1:N]
    np.testing.assert_allclose(L.mul_padded(u[-1], u, u[0]), ref @ xp, rtol=1e-12, atol=1e-12 * scale)
    np.testing.assert_allclose(L.array(), ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_scalar_multiplication():
    # derivative_operators_interface.jl:407-415
    L = O.centered(2, 2, 10.0, 3).scale(3.3)
    np.testing.assert_allclose(L.array(), FX["scalar_mult_3p3"], rtol=1e-12)


def test_robin_general_known_answer():
    # robin.jl:92-110
    u = np.arange(1.0, 11.0)
    for q in (O.robin((1.0, 6.0, 10.0), (1.0, 6.0, 10.0), 1.0, 3),
              O.general([-10.0, 1.0, 6.0], [-10.0, 1.0, 6.0], 1.0, 3),
              O.general([-10.0, 1.0, 6.0], [-10.0, 1.0, 6.0], np.ones(10), 3)):
        l, r = q.ghosts(u)
        assert l == pytest.approx(FX["robin3_u0"][0], rel=1e-12)
        assert r == pytest.approx(FX["robin3_uend"][0], rel=1e-12)


@pytest.mark.parametrize("uniform", [True, False])
def test_robin_closed_forms(uniform):
    # robin.jl:15-38 and :45-90
    rng = np.random.default_rng(7)
    for i in range(1, 6):
        al, bl, cl, dx, ar, br, cr = rng.random(7)
        q = O.robin((al, bl, cl), (ar, br, cr), dx if uniform else dx * np.ones(5 * i))
        QL, Qb = q.array(5 * i)
        np.testing.assert_allclose(QL[1:5 * i + 1, :], np.eye(5 * i))
        assert QL[0, 0] == pytest.approx(1 / (1 - al * dx / bl), rel=1e-12)
        assert QL[-1, -1] == pytest.approx(1 / (1 + ar * dx / br), rel=1e-12)
        assert Qb[0] == pytest.approx(cl / (al - bl / dx), rel=1e-12)
        assert Qb[-1] == pytest.approx(cr / (ar + br / dx), rel=1e-12)
        u = rng.random(5 * i)
        l, r = q.ghosts(u)
        assert l == pytest.approx((cl - (bl / dx) * u[0]) / (al - bl / dx), rel=1e-12)
        assert r == pytest.approx((cr + (br / dx) * u[-1]) / (ar + br / dx), rel=1e-12)


def test_complete_stencil_weights():
    # derivative_operators_interface.jl:148-151: centred weights d = 1..3, a = 2, 4
    w2 = np.concatenate([O.calculate_weights(d, 0.0, np.arange(-(s // 2), s // 2 + 1))
                         for d, s in ((1, 3), (2, 3), (3, 5))])
    w4 = np.concatenate([O.calculate_weights(d, 0.0, np.arange(-(s // 2), s // 2 + 1))
                         for d, s in ((1, 5), (2, 5), (3, 7))])
    np.testing.assert_allclose(w2, FX["ctr_weights_a2"], atol=1e-10)
    np.testing.assert_allclose(w4, FX["ctr_weights_a4"], atol=1e-10)


def test_nd_apply_is_per_line():
    # differentiation_dimension.jl: applying along axis k equals the 1-D
    # generic operator on every line along k
    rng = np.random.default_rng(3)
    u = np.asfortranarray(rng.standard_normal((6, 7, 8)))
    L = O.centered(2, 4, 0.1, 7, axis=2)
    q = O.robin((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), 0.1, 1)
    out = O.apply([(L, q)], u)
    for i in range(6):
        for k in range(8):
            line = u[i, :, k]
            l, r = q.ghosts(line)
            np.testing.assert_array_equal(out[i, :, k], L.mul_generic(np.concatenate([[l], line, [r]])))


def test_composite_sum_order():
    # (A*Q)*u = sum(op -> op*u, ops), left to right (composite_operators.jl:64-65)
    rng = np.random.default_rng(4)
    u = np.asfortranarray(rng.standard_normal((9, 10)))
    q = O.dirichlet0()
    L1, L2 = O.centered(2, 2, 0.1, 9, axis=1), O.centered(1, 4, 0.1, 10, axis=2)
    both = O.apply([(L1, q), (L2, q)], u)
    np.testing.assert_array_equal(both, O.apply([(L1, q)], u) + O.apply([(L2, q)], u))


def test_ssprk3_matches_manual_stages():
    rng = np.random.default_rng(5)
    u0 = rng.standard_normal(32)
    L = O.centered(2, 2, 1.0 / 33, 32)
    L.scale(1e-3)
    q = O.dirichlet0()
    dt = 1e-2
    f = lambda v: O.apply([(L, q)], v)
    u1 = u0 + dt * f(u0)
    u2 = 0.75 * u0 + 0.25 * (u1 + dt * f(u1))
    u3 = (1.0 / 3.0) * u0 + (2.0 / 3.0) * (u2 + dt * f(u2))
    np.testing.assert_array_equal(O.ssprk3([(L, q)], u0, dt, 1), u3)
