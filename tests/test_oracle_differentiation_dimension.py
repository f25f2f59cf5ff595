"""The oracle's N-D `mul!(x_temp, L, M)` on already padded arrays against the
reference's differentiation-dimension tests
(test/DerivativeOperators/differentiation_dimension.jl): every line along the
operator's axis equals the analytic operator matrix times that line, for
axes 1-3 of 2-D and 3-D arrays, axis 6 of a 7-D array, the non-symmetric
interior stencil of CenteredDifference(3, 4) and a scaled operator.  The GPU
kernel for the same call is checked against the oracle in test_gpu_padded.py.
"""
import numpy as np
import pytest

import oracle as O
from transcribe_reference import fourth_deriv_approx_stencil, second_derivative_stencil

RTOL = np.sqrt(np.finfo(float).eps)


def _approx(x, y):
    return np.linalg.norm(np.ravel(x) - np.ravel(y)) <= RTOL * max(np.linalg.norm(np.ravel(x)),
                                                                    np.linalg.norm(np.ravel(y)))


def _field(shape, axis, f):
    """M[idx] = f(idx[axis] * 0.1) with Julia's 1-based index."""
    idx = np.arange(1, shape[axis - 1] + 1)
    sh = [1] * len(shape)
    sh[axis - 1] = shape[axis - 1]
    return np.asfortranarray(np.broadcast_to(f(0.1 * idx).reshape(sh), shape))


def _lines(a, axis):
    return np.moveaxis(a, axis - 1, 0).reshape(a.shape[axis - 1], -1)


@pytest.mark.parametrize("axis", [1, 2])
def test_2d_fourth_derivative(axis):
    # differentiation_dimension.jl:25-63
    M = _field((22, 22), axis, np.sin)
    L = O.centered(4, 4, 0.1, 20, axis=axis)
    out = O.mul_nd(L, M)
    line = _lines(M, axis)[:, 0]
    correct = 10000.0 * fourth_deriv_approx_stencil(20) @ line
    for col in _lines(out, axis).T:
        assert _approx(col, correct)


@pytest.mark.parametrize("axis", [1, 2, 3])
@pytest.mark.parametrize("d", [2, 4])
def test_3d_second_and_fourth_derivative(d, axis):
    # :65-123 (L2 = CenteredDifference(2, 2)) and :125-185 (L4 = CenteredDifference(4, 4))
    M = _field((22, 22, 22), axis, np.sin)
    L = O.centered(d, d, 0.1, 20, axis=axis)
    out = O.mul_nd(L, M)
    line = _lines(M, axis)[:, 0]
    correct = (100.0 * second_derivative_stencil(20) if d == 2 else
               10000.0 * fourth_deriv_approx_stencil(20)) @ line
    for col in _lines(out, axis).T:
        assert _approx(col, correct)


def test_arbitrary_higher_dimension():
    # :186-208: CenteredDifference{6}(4, 4, 0.1, 30) on a 5x5x5x5x5x32x5 array
    shape = (5, 5, 5, 5, 5, 32, 5)
    M = _field(shape, 6, np.cos)
    L = O.centered(4, 4, 0.1, 30, axis=6)
    out = O.mul_nd(L, M)
    assert out.shape == (5, 5, 5, 5, 5, 30, 5)
    correct = 1e4 * fourth_deriv_approx_stencil(30) @ _lines(M, 6)[:, 0]
    for col in _lines(out, 6).T:
        assert _approx(col, correct)


def test_non_symmetric_interior_stencil():
    # :209-283: CenteredDifference(3, 4) -- M_temp = Array(L) * M along axis 1,
    # transpose(Array(L) * transpose(M)) along axis 2, and 3-D slices
    L1 = O.centered(3, 4, 0.1, 30, axis=1)
    L2 = O.centered(3, 4, 0.1, 30, axis=2)
    A = L1.array()
    M = _field((32, 32), 1, np.cos)
    assert _approx(O.mul_nd(L1, M), A @ M)
    M = _field((32, 32), 2, np.cos)
    assert _approx(O.mul_nd(L2, M), (A @ M.T).T)
    M3 = _field((32, 32, 32), 1, np.cos)
    out = O.mul_nd(L1, M3)
    for i in range(32):
        assert _approx(out[:, :, i], A @ M3[:, :, i])
    correct = L1.mul_generic(M3[:, 0, 0])
    for axis in (2, 3):
        L = O.centered(3, 4, 0.1, 30, axis=axis)
        Ma = _field((32, 32, 32), axis, np.cos)
        for col in _lines(O.mul_nd(L, Ma), axis).T:
            assert _approx(col, correct)


@pytest.mark.parametrize("axis", [1, 2, 3])
def test_scaled_operator(axis):
    # :292-370: mul!(M_temp, 5.5 * CenteredDifference{N}(3, 4, 0.1, 30), M)
    L = O.centered(3, 4, 0.1, 30, axis=axis)
    M = _field((32, 32, 32), axis, np.cos)
    correct = 5.5 * L.mul_generic(_lines(M, axis)[:, 0])
    L.scale(5.5)
    for col in _lines(O.mul_nd(L, M), axis).T:
        assert _approx(col, correct)
