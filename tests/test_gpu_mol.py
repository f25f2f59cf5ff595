"""GPU: the reference's method-of-lines examples (test/DerivativeOperators/
heat_eqn.jl) advanced with the library's SSP-RK3 stages instead of
OrdinaryDiffEq's Tsit5, at the reference's own tolerances, and its statement
that an UpwindDifference with as many offside as primary wind points behaves
like a CenteredDifference."""
import numpy as np
import pytest

import deo

pytestmark = pytest.mark.gpu


def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to("cuda")


def test_heat_equation_dirichlet(cuda):
    """heat_eqn.jl:4-28: x = -pi:2pi/511:pi, u0 = -(x - 0.5)^2 + 1/12, Dirichlet
    ghosts from the analytic profile; the end points stay within rtol 0.05 of
    u0 for t in 0:0.1:1 -- with A = CenteredDifference(2, 2) and with
    UpwindDifference(2, 1; offside = 1)."""
    h = 2 * np.pi / 511
    x = -np.pi + h * np.arange(512)
    ua = lambda s: -(s - 0.5) ** 2 + 1.0 / 12
    u0 = ua(x)
    bc = deo.DirichletBC(float(ua(-np.pi - h)), float(ua(np.pi + h)))
    dt = 0.25 * h * h  # SSP-RK3 stable for the second difference (CFL 0.5 of the explicit bound)
    steps = int(round(0.1 / dt))
    dt = 0.1 / steps
    for L in (deo.CenteredDifference(2, 2, h, 512), deo.UpwindDifference(2, 1, h, 512, 1.0, offside=1)):
        A = deo.DiffEqOperatorCombination([L * bc])
        u = _dev(u0)
        for _ in range(10):
            u = deo.autodiff.ssprk3_solve(A, u, dt, steps)
            v = u.cpu().numpy()
            assert abs(v[0] - u0[0]) <= 0.05 * abs(u0[0])
            assert abs(v[-1] - u0[-1]) <= 0.05 * abs(u0[-1])


def test_upwind_with_offside_matches_centred(cuda):
    """UpwindDifference(2, 1; offside = 1) applies the centred 3-point stencil
    (heat_eqn.jl:18-19): the same result as CenteredDifference(2, 2) in the
    interior and at the boundary rows."""
    h = 2 * np.pi / 511
    rng = np.random.default_rng(4)
    u = _dev(rng.standard_normal(512))
    bc = deo.DirichletBC(0.3, -0.2)
    c = (deo.CenteredDifference(2, 2, h, 512) * bc * u).cpu().numpy()
    w = (deo.UpwindDifference(2, 1, h, 512, 1.0, offside=1) * bc * u).cpu().numpy()
    assert np.allclose(w, c, rtol=1e-12, atol=1e-9 * np.abs(c).max())


def test_heat_equation_sine_decay(cuda):
    """heat_equation.jl: du/dt = Delta*bc*u on 100 knots of (0, 1) with
    Dirichlet0BC, u0 = sin(2 pi x); at t = 0.03 the solution matches
    sin(2 pi x) exp(-t (2 pi)^2) to rtol 1e-3 (isapprox on the vectors).  The
    reference integrates with KenCarp4; here the library's SSP-RK3 stages."""
    nknots = 100
    h = 1.0 / (nknots + 1)
    knots = h * np.arange(1, nknots + 1)
    ua = lambda x, t: np.sin(2 * np.pi * x) * np.exp(-t * (2 * np.pi) ** 2)
    A = deo.DiffEqOperatorCombination([deo.CenteredDifference(2, 2, h, nknots) * deo.Dirichlet0BC(np.float64)])
    t1 = 0.03
    steps = int(np.ceil(t1 / (0.4 * h * h)))
    u = deo.autodiff.ssprk3_solve(A, _dev(ua(knots, 0.0)), t1 / steps, steps).cpu().numpy()
    ref = ua(knots, t1)
    assert np.linalg.norm(u - ref) <= 1e-3 * max(np.linalg.norm(u), np.linalg.norm(ref))


def test_ode_call_interface(cuda):
    """(A)(u, p, t) = A*u and (A)(du, u, p, t) = mul!(du, A, u) (DiffEqOperators.jl:67-76)
    for L*Q, sums of them, and a DerivativeOperator on a padded vector."""
    import torch
    rng = np.random.default_rng(8)
    h = 0.01
    L = deo.CenteredDifference(2, 4, h, 64)
    A = L * deo.RobinBC((1.0, 0.5, 0.2), (1.0, 0.5, -0.1), h, 1)
    B = A + deo.UpwindDifference(1, 2, h, 64, -0.7) * deo.Dirichlet0BC(np.float64)
    u = _dev(rng.standard_normal(64))
    for op in (A, B):
        ref = (op * u).cpu().numpy()
        assert np.array_equal(op(u, None, 0.0).cpu().numpy(), ref)
        du = torch.empty_like(u)
        op(du, u, None, 0.0)
        assert np.array_equal(du.cpu().numpy(), ref)
    M = _dev(rng.standard_normal(66))
    assert np.array_equal(L(M, None, 0.0).cpu().numpy(), (L * M).cpu().numpy())


def test_time_dependent_coefficients(cuda):
    """(A)(du, u, p, t) runs update_coefficients! before the apply
    (DiffEqOperators.jl:67-76): with coeff_func(c, u, p, t) = (c .= 1 + t) the
    applies at t = 0 and t = 1 use coefficients 1 and 2, and a cached device
    plan never serves the old values."""
    import oracle as O
    import torch
    rng = np.random.default_rng(9)
    h = 0.02
    f = lambda c, u, p, t: c.__setitem__(slice(None), 1.0 + t)
    A = (f * deo.UpwindDifference(1, 2, h, 48, 1.0)) * deo.RobinBC((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), h, 1)
    u_np = rng.standard_normal(48)
    u = _dev(u_np)
    du = torch.empty_like(u)
    q = O.robin((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), h, 1)
    for t in (0.0, 1.0, 0.0):
        A(du, u, None, t)
        Lo = O.upwind(1, 2, h, 48, np.full(48, 1.0 + t))
        ref = O.apply([(Lo, q)], u_np)
        tol = 4 * np.spacing(O.abs_scale([(Lo, q)], u_np))
        assert (np.abs(du.cpu().numpy() - ref) <= tol).all(), t
