"""CPU: boundary conditions that differ per line (MultiDimBC{dim}(BCs::Array),
multi_dim_bc_operators.jl:91-93) in the oracle and the Python front-end.

The reference pads every line with its own BC: Q*u gives, for line (I, J),
the ghosts of BCs[I, J] * u[I, :, J] (slice_rmul, :28-52), the 1-D ghost fill
-- its own test checks Ax[:, j] == Array(BCx[j] * A[:, j]) for an array mixing
RobinBC and PeriodicBC (test/DerivativeOperators/multi_dim_bc_test.jl:17-34).
So the N-D apply with per-line BCs must equal, line by line, the 1-D apply of
the operator with that line's BC."""
import numpy as np
import pytest

import deo
import oracle as O


def _mixed(n_lines, seed):
    """The reference test's mix: RobinBC((1,2,3),(0,-1,2),0.1,4) and PeriodicBC, plus
    Dirichlet and a GeneralBC, in a seeded order."""
    rng = np.random.default_rng(seed)
    pool = [O.robin((1.0, 2.0, 3.0), (0.0, -1.0, 2.0), 0.1, 4), O.periodic(), O.dirichlet(0.5, -0.25),
            O.general([0.3, 1.0, 0.2], [-0.1, 0.7, 0.4], 0.1, 2)]
    return [pool[k] for k in rng.integers(0, len(pool), n_lines)]


@pytest.mark.parametrize("shape,axis", [((9, 7), 1), ((9, 7), 2), ((8, 6, 5), 1), ((8, 6, 5), 2), ((8, 6, 5), 3)])
@pytest.mark.parametrize("d,a", [(2, 2), (1, 4), (3, 2)])
def test_per_line_bcs_equal_the_1d_apply_of_each_line(shape, axis, d, a):
    rng = np.random.default_rng(1)
    u = np.asfortranarray(rng.standard_normal(shape))
    n = shape[axis - 1]
    nlines = int(np.prod(shape)) // n
    lines = _mixed(nlines, 2)
    op = O.centered(d, a, 0.1, n, axis=axis)
    got = O.apply([(op, lines[0], None, lines)], u)
    # line (I, J) in the column-major order of the other axes
    um = np.moveaxis(u, axis - 1, 0).reshape(n, -1, order="F")
    gm = np.moveaxis(got, axis - 1, 0).reshape(n, -1, order="F")
    op1 = O.centered(d, a, 0.1, n, axis=1)
    for j in range(nlines):
        # N-D arrays take the generic per-line methods: the operator on the line padded by its own BC
        l, r = lines[j].ghosts(um[:, j])
        x = np.concatenate([[l], um[:, j], [r]])
        assert np.array_equal(gm[:, j], op1.mul_generic(x)), j


def test_all_periodic_array_pads_with_the_edge_planes():
    """An array of PeriodicBCs dispatches to the periodic padding
    (multi_dim_bc_operators.jl:221-228), as PeriodicBC(T, s) does."""
    rng = np.random.default_rng(3)
    u = np.asfortranarray(rng.standard_normal((7, 6)))
    op = O.centered(2, 2, 0.1, 7, axis=1)
    a = O.apply([(op, O.periodic(), None, [O.periodic()] * 6)], u)
    b = O.apply([(op, O.periodic())], u)
    assert np.array_equal(a, b)


def test_front_end_shapes_and_uniform_arrays():
    Q = deo.RobinBC((1.0, 2.0, 3.0), (0.0, -1.0, 2.0), 0.1, 4)
    P = deo.PeriodicBC()
    arr = np.empty((5,), dtype=object)
    for k in range(5):
        arr[k] = Q if k % 2 else P
    Qx = deo.MultiDimBC(arr, dim=1)
    assert Qx.line_bcs(1)[1] is Q and Qx.line_bcs(1)[0] is P
    Qx.check_size((9, 5))
    with pytest.raises(deo.DeoShapeError):
        Qx.check_size((9, 6))  # the reference asserts perpsize(u, D) == size(Q.BCs)
    with pytest.raises(deo.DeoArgError):
        deo.MultiDimBC(arr)  # an array needs dim
    Qy = deo.MultiDimBC(np.array([[Q, Q], [Q, P]], dtype=object), dim=2)
    with pytest.raises(deo.DeoShapeError):
        Qy.check_size((3, 4, 2))  # perpsize along 2 is (3, 2), the array is (2, 2)
    Qy.check_size((2, 4, 2))
    Qc = deo.compose(Qx, deo.MultiDimBC(Q, (9, 5), 2))
    assert Qc.line_bcs(1) is not None and Qc.line_bcs(2) is None
