"""Seeded random properties of the oracle (CPU), over operators the reference
builds (centred / upwind with offside, uniform / non-uniform grids, scalar or
vector coefficients) and every BC kind:

- with a constant coefficient, the generic method on a padded vector equals
  the concretisation, L*[l; u; r] == Array(L) * [l; u; r]
  (concretization.jl:8-52, 556-671), and so does L*Q*u on a 1-D array,
  == Array(L) * (Q_L u + Q_b).  With a coefficient vector the reference's
  methods read other entries than Array(L) does -- the generic method's right
  boundary rows read coeff[1:bpc] (convolutions.jl:109), the padded-vector
  methods coeff[i-bpc] (:384) -- and the oracle keeps those reads;
- linearity in u of the homogeneous part: (L*Q)(a u + b v) - (L*Q)(0)
  == a ((L*Q) u - (L*Q) 0) + b ((L*Q) v - (L*Q) 0), to rounding;
- the N-D per-line apply equals the 1-D generic apply on every line.
"""
import numpy as np
import pytest

import oracle as O


def _case(seed):
    rng = np.random.default_rng(5000 + seed)
    upwind = rng.random() < 0.5
    if upwind:
        d, a = int(rng.integers(1, 3)), int(rng.integers(1, 4))
        off = int(rng.integers(0, (d + a - 1) // 2 + 1))
    else:
        d, a = int(rng.integers(1, 5)), int(rng.choice([2, 4, 6]))
        off = 0
    n = int(rng.integers(2 * (d + a) + 2, 60))
    dx = 1.0 / (n + 1) if rng.random() < 0.5 else rng.uniform(0.5, 1.5, n + 1) / n
    const = rng.random() < 0.5
    coeff = float(rng.uniform(-2, 2)) if const else rng.uniform(-1, 1, n)
    if not upwind and not const:
        coeff = np.abs(coeff) + 0.5
    op = O.upwind(d, a, dx, n, coeff, offside=off) if upwind else O.centered(d, a, dx, n, coeff)
    k = rng.random()
    al = (float(rng.uniform(0.5, 1.5)), float(rng.uniform(0.1, 1.0)), float(rng.uniform(-1, 1)))
    ar = (float(rng.uniform(0.5, 1.5)), float(rng.uniform(0.1, 1.0)), float(rng.uniform(-1, 1)))
    if k < 0.2:
        q = O.dirichlet0()
    elif k < 0.35:
        q = O.dirichlet(al[2], ar[2])
    elif k < 0.5:
        q = O.neumann((al[2], ar[2]), dx, int(rng.integers(1, 4)))
    elif k < 0.75:
        q = O.robin(al, ar, dx, int(rng.integers(1, 4)))
    elif k < 0.9:
        q = O.general((float(rng.uniform(-1, 1)), 1.0, float(rng.uniform(0.1, 1.0))),
                      (float(rng.uniform(-1, 1)), 1.0, float(rng.uniform(0.1, 1.0))), dx, 2)
    else:
        q = O.periodic()
    return rng, op, q, n, const


@pytest.mark.parametrize("seed", range(120))
def test_apply_matches_concretisation(seed):
    rng, op, q, n, const = _case(seed)
    A = op.array()
    x = rng.standard_normal(n + 2)
    y = op.mul_generic(x)
    scale = np.abs(A) @ np.abs(x)
    # with a coefficient vector only the generic method's right boundary rows read other entries
    keep = slice(None) if const else slice(0, n - op.n_high)
    assert (np.abs(y - A @ x)[keep] <= 64 * np.finfo(float).eps * scale[keep] + 1e-300).all()
    if not const:
        return
    u = rng.standard_normal(n)
    QL, Qb = q.array(n)
    got = O.apply([(op, q)], u)
    ref = A @ (QL @ u + Qb)
    sc = np.abs(A) @ (np.abs(QL) @ np.abs(u) + np.abs(Qb))
    assert (np.abs(got - ref) <= 64 * np.finfo(float).eps * sc + 1e-300).all()


@pytest.mark.parametrize("seed", range(120))
def test_homogeneous_part_is_linear(seed):
    rng, op, q, n, _ = _case(seed)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    a, b = rng.uniform(-2, 2, 2)
    f = lambda w: O.apply([(op, q)], w)
    z = f(np.zeros(n))
    lhs = f(a * u + b * v) - z
    rhs = a * (f(u) - z) + b * (f(v) - z)
    sc = O.abs_scale([(op, q)], np.abs(a * u) + np.abs(b * v)) + np.abs(z)
    assert (np.abs(lhs - rhs) <= 256 * np.finfo(float).eps * (sc + np.abs(a) * np.abs(f(u)) +
                                                              np.abs(b) * np.abs(f(v))) + 1e-300).all()


@pytest.mark.parametrize("seed", range(30))
def test_nd_apply_is_the_generic_apply_per_line(seed):
    rng, op1, q, n, _ = _case(seed)
    other = int(rng.integers(3, 7))
    for axis in (1, 2):
        shape = (n, other) if axis == 1 else (other, n)
        op1.axis = axis  # the axis a term acts on is the apply's argument, not the operator's
        u = np.asfortranarray(rng.standard_normal(shape))
        out = O.apply([(op1, q)], u)
        for j in range(other):
            line = u[:, j] if axis == 1 else u[j, :]
            if q.kind == 1:  # N-D PeriodicBC pads with the edge planes (multi_dim_bc_operators.jl:221-228)
                l, r = line[0], line[-1]
            else:
                l, r = q.ghosts(line)
            ref = op1.mul_generic(np.concatenate([[l], line, [r]]))
            got = out[:, j] if axis == 1 else out[j, :]
            np.testing.assert_array_equal(got, ref)
