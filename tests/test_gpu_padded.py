"""GPU: a DerivativeOperator on an already padded array -- L*M and
mul!(x_temp, L, M; overwrite) (derivative_operator_functions.jl:17-69, 150-163;
convolutions.jl:17-22 for vectors) -- against the oracle's restatement, at the
4-ulp-of-sum|c_k u_k| bar."""
import zlib

import numpy as np
import pytest

import deo
import oracle as O
from cases import nonuniform_dx, to_device, to_host

pytestmark = pytest.mark.gpu


def _ops(kind, d, a, n, grid, coeff, axis, rng):
    dx = 1.0 / (n + 1) if grid == "uniform" else nonuniform_dx(n)
    c = rng.uniform(0.5, 1.5, n) if coeff == "vector" else (rng.uniform(-1, 1, n) if coeff == "signed" else None)
    if kind == "centered":
        return (deo.CenteredDifference(d, a, dx, n, 1 if c is None else c, axis=axis),
                O.centered(d, a, dx, n, c, axis=axis))
    return (deo.UpwindDifference(d, a, dx, n, 1.0 if c is None else c, axis=axis),
            O.upwind(d, a, dx, n, 1.0 if c is None else c, axis=axis))


def _check(got, ref, scale):
    assert (np.abs(got - ref) <= 4 * np.spacing(scale)).all(), np.max(np.abs(got - ref) / np.spacing(scale))


CASES = [("centered", 2, 2, "uniform", None), ("centered", 1, 4, "nonuniform", "vector"),
         ("centered", 3, 4, "uniform", "vector"), ("upwind", 1, 2, "uniform", "signed"),
         ("upwind", 2, 3, "nonuniform", "signed"), ("centered", 4, 6, "nonuniform", None)]


@pytest.mark.parametrize("kind,d,a,grid,coeff", CASES)
@pytest.mark.parametrize("shape,axis,strip", [((60,), 1, False), ((40, 30), 1, False), ((40, 30), 2, True),
                                              ((14, 12, 16), 3, False), ((14, 12, 16), 2, True)])
def test_against_oracle(cuda, kind, d, a, grid, coeff, shape, axis, strip):
    rng = np.random.default_rng(zlib.crc32(repr((kind, d, a, grid, coeff, shape, axis, strip)).encode()))
    n = shape[axis - 1]
    L, Lo = _ops(kind, d, a, n, grid, coeff, axis, rng)
    # M padded along the axis; with strip, padded on every axis (x_temp keeps the unpadded sizes)
    in_shape = tuple(s + 2 if (b == axis - 1 or strip) else s for b, s in enumerate(shape))
    M = np.asfortranarray(rng.standard_normal(in_shape))
    if strip:
        x0 = np.asfortranarray(rng.standard_normal(shape))
        xt = to_device(x0)
        deo.mul_(xt, L, to_device(M), overwrite=False)
        ref = O.mul_nd(Lo, M, out=x0.copy(order="F"), overwrite=False)
        scale = O.mul_nd(Lo, M, out_shape=shape, absolute=True) + np.abs(x0)
        _check(to_host(xt), ref, scale)
    else:
        got = to_host(L * to_device(M))
        ref = O.mul_nd(Lo, M)
        scale = O.mul_nd(Lo, M, absolute=True)
        _check(got, ref, scale)


def test_size_errors(cuda):
    L = deo.CenteredDifference(2, 2, 0.1, 10, axis=2)
    with pytest.raises(deo.DeoShapeError):
        L * to_device(np.zeros((5, 10)))  # axis 2 not padded
    with pytest.raises(deo.DeoShapeError):
        deo.mul_(to_device(np.zeros((5, 10))), L, to_device(np.zeros((8, 12))))  # axis 1: 8 is neither 5 nor 7
    with pytest.raises(deo.DeoShapeError):
        L * to_device(np.zeros(12))  # axis 2 of a vector
