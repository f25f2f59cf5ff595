"""Gradient / Divergence / Curl and the pointwise vector algebra on the GPU.

    Gradient(approx_order, dx, len; coeff_func)    A * M : (len+2 ...)    -> (len..., N)
    Divergence(approx_order, dx, len; coeff_func)  A * M : (len+2 ..., N) -> (len...)
    Curl(approx_order, dx, len; coeff_func)        A * M : (len+2 ..., 3) -> (len..., 3)

(vector_calculus_operators.jl:1-88, vector_calculus_convolutions.jl).  Each
operator holds the reference's `ops`: CenteredDifference{n}(1, approx_order,
dx[n], len[n], coeff_func) per axis; `c * A` scales each op's coefficients.
`A * M` starts from zeros; `mul_(x_temp, A, M)` adds into x_temp, as the
reference's mul! does.  For 2-D and 3-D arrays the reference's specialised
methods are followed exactly, including their reading of the axes other
than the differentiated one at the padded index equal to the output index.

dot_product, cross_product and square_norm (vector_algebraic_operations.jl)
act on (s..., ncomp) arrays.  Arrays are column-major CUDA tensors (Julia
layout, see julia_array); Float64 and Float32.
"""
from __future__ import annotations

import ctypes as C
import numbers
from typing import Sequence

from . import _lib as L
from ._lib import DeoArgError, check
from .operators import (CenteredDifference, DerivativeOperator, DimensionMismatch, _check_layout, _dtype_code,
                        _stream_ptr, julia_array)

GRADIENT, DIVERGENCE, CURL = 0, 1, 2


class _VectorCalculusOperator:
    kind = -1

    def __init__(self, ops: Sequence[DerivativeOperator]):
        self.ops = list(ops)
        self._plans: dict = {}

    @property
    def ndims(self) -> int:
        return len(self.ops)

    @property
    def lens(self) -> tuple:
        return tuple(op.len for op in self.ops)

    def _plan(self, dtype_code: int):
        h = self._plans.get(dtype_code)
        if h is None:
            arr = (C.c_void_p * self.ndims)(*[op._h.value for op in self.ops])
            out = C.c_void_p()
            check(L.lib().deo_vector_calculus_plan(self.kind, self.ndims, arr, int(dtype_code), C.byref(out)))
            h = self._plans[dtype_code] = out
        return h

    def info(self, dtype_code: int = 0) -> dict:
        """Execution choice of the plan for a dtype: the interior band width
        of the unrolled marching kernel (0 = row tables everywhere)."""
        nk = C.c_int()
        check(L.lib().deo_vector_calculus_info(self._plan(dtype_code), C.byref(nk)))
        return {"band_nk": nk.value}

    def __del__(self):
        try:
            for h in self._plans.values():
                L.lib().deo_vector_calculus_destroy(h)
            self._plans = {}
        except Exception:
            pass

    def __rmul__(self, c):
        """c * A: every axis operator's coefficients scaled by c
        (vector_calculus_operators.jl:75-88)."""
        if isinstance(c, numbers.Number):
            return type(self)([c * op for op in self.ops])
        return NotImplemented

    # shapes ---------------------------------------------------------------
    def in_shape(self) -> tuple:
        padded = tuple(n + 2 for n in self.lens)
        return padded if self.kind == GRADIENT else padded + (self.ndims,)

    def out_shape(self) -> tuple:
        if self.kind == DIVERGENCE:
            return self.lens
        return self.lens + (self.ndims,)

    def _check(self, M, out=None):
        if not getattr(M, "is_cuda", False):
            raise DeoArgError(2, "M must be a CUDA tensor")
        _check_layout(M, "M")
        if tuple(M.shape) != self.in_shape():
            raise DimensionMismatch(f"M has size {tuple(M.shape)}; this operator needs {self.in_shape()}")
        if out is not None:
            _check_layout(out, "x_temp")
            if tuple(out.shape) != self.out_shape() or out.dtype != M.dtype or out.device != M.device:
                raise DimensionMismatch(f"x_temp has size {tuple(out.shape)}; this operator writes "
                                        f"{self.out_shape()} of M's dtype")

    def _apply(self, out, M, overwrite: bool):
        h = self._plan(_dtype_code(M))
        check(L.lib().deo_vector_calculus_apply(h, C.c_void_p(M.data_ptr()), C.c_void_p(out.data_ptr()),
                                                1 if overwrite else 0, _stream_ptr()))
        return out

    def __mul__(self, M):
        """A * M (vector_calculus_operators.jl:49-73): a new array from zeros."""
        if isinstance(M, numbers.Number):
            return NotImplemented
        self._check(M)
        out = julia_array(self.out_shape(), M.dtype, M.device)
        return self._apply(out, M, True)

    def mul_(self, x_temp, M, overwrite: bool = False):
        """mul!(x_temp, .., A, M): adds A*M into x_temp (the reference's
        vector-calculus mul! always accumulates); overwrite=True replaces."""
        self._check(M, x_temp)
        return self._apply(x_temp, M, overwrite)


class GradientOperator(_VectorCalculusOperator):
    kind = GRADIENT


class DivergenceOperator(_VectorCalculusOperator):
    kind = DIVERGENCE


class CurlOperator(_VectorCalculusOperator):
    kind = CURL


def _axis_ops(approximation_order: int, dx, lens, coeff_func):
    lens = tuple(int(n) for n in lens)
    if isinstance(dx, (numbers.Number,)) or len(dx) != len(lens):
        raise DeoArgError(2, "dx must hold one grid spacing (a number or a vector) per axis")
    return [CenteredDifference(1, approximation_order, dx[n], lens[n], coeff_func, axis=n + 1)
            for n in range(len(lens))]


def Gradient(approximation_order: int, dx, len, coeff_func=1) -> GradientOperator:
    """Gradient(approximation_order, dx::NTuple{N}, len::NTuple{N}; coeff_func)
    (vector_calculus_operators.jl:9-16)."""
    return GradientOperator(_axis_ops(approximation_order, dx, len, coeff_func))


def Divergence(approximation_order: int, dx, len, coeff_func=1) -> DivergenceOperator:
    """Divergence(approximation_order, dx, len; coeff_func) (vector_calculus_operators.jl:38-45)."""
    return DivergenceOperator(_axis_ops(approximation_order, dx, len, coeff_func))


def Curl(approximation_order: int, dx, len, coeff_func=1) -> CurlOperator:
    """Curl(approximation_order, dx::NTuple{3}, len::NTuple{3}; coeff_func)
    (vector_calculus_operators.jl:24-32)."""
    lens = tuple(len)
    if not (lens[0] == lens[1] == lens[2]):
        raise AssertionError("All dimensions must have equal no. of grid points")
    return CurlOperator(_axis_ops(approximation_order, dx, lens, coeff_func))


def mul_(x_temp, A: _VectorCalculusOperator, M, overwrite: bool = False):
    return A.mul_(x_temp, M, overwrite)


# ---------------------------------------------------------------------------
# vector algebra (vector_algebraic_operations.jl)
# ---------------------------------------------------------------------------
def _vec_check(*xs):
    for x in xs:
        if not getattr(x, "is_cuda", False):
            raise DeoArgError(2, "arrays must be CUDA tensors")
        _check_layout(x, "array")


def dot_product_(u, A, B):
    """dot_product!(u, A, B) (vector_algebraic_operations.jl:11-28)."""
    _vec_check(u, A, B)
    if tuple(A.shape) != tuple(B.shape) or A.dtype != B.dtype:
        raise DeoArgError(2, "Vectors must have the same shape")
    if u.dim() != A.dim() - 1 or tuple(u.shape) != tuple(A.shape[:-1]) or u.dtype != A.dtype:
        raise DeoArgError(2, "Output should be scalar matrix, one dimension less than input")
    npts = u.numel()
    check(L.lib().deo_dot_product(_dtype_code(A), npts, int(A.shape[-1]), C.c_void_p(A.data_ptr()),
                                  C.c_void_p(B.data_ptr()), C.c_void_p(u.data_ptr()), _stream_ptr()))
    return u


def dot_product(A, B):
    """dot_product(A, B) (vector_algebraic_operations.jl:3-9)."""
    if tuple(A.shape) != tuple(B.shape):
        raise DeoArgError(2, "Vectors must have the same shape")
    return dot_product_(julia_array(tuple(A.shape[:-1]), A.dtype, A.device), A, B)


def cross_product_(u, A, B):
    """cross_product!(u, A, B) (vector_algebraic_operations.jl:39-52) for (s1, s2, s3, 3) arrays."""
    _vec_check(u, A, B)
    if not (tuple(A.shape) == tuple(B.shape) == tuple(u.shape)) or A.dtype != B.dtype or u.dtype != A.dtype:
        raise DeoArgError(2, "Vectors must have the same shape")
    if A.dim() != 4 or A.shape[-1] != 3:
        raise DeoArgError(2, "cross_product acts on (s1, s2, s3, 3) arrays")
    npts = u.numel() // 3
    check(L.lib().deo_cross_product(_dtype_code(A), npts, C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()),
                                    C.c_void_p(u.data_ptr()), _stream_ptr()))
    return u


def cross_product(A, B):
    """cross_product(A, B) (vector_algebraic_operations.jl:30-37)."""
    if tuple(A.shape) != tuple(B.shape):
        raise DeoArgError(2, "Vectors must have the same shape")
    return cross_product_(julia_array(tuple(A.shape), A.dtype, A.device), A, B)


def square_norm_(u, A):
    """square_norm!(u, A) (vector_algebraic_operations.jl:54-62): sqrt of dot_product(A, A)."""
    _vec_check(u, A)
    if u.dim() != A.dim() - 1 or tuple(u.shape) != tuple(A.shape[:-1]) or u.dtype != A.dtype:
        raise DeoArgError(2, "Output should be scalar matrix, one dimension less than input")
    check(L.lib().deo_square_norm(_dtype_code(A), u.numel(), int(A.shape[-1]), C.c_void_p(A.data_ptr()),
                                  C.c_void_p(u.data_ptr()), _stream_ptr()))
    return u


def square_norm(A):
    """square_norm(A) (vector_algebraic_operations.jl:54-58)."""
    return square_norm_(julia_array(tuple(A.shape[:-1]), A.dtype, A.device), A)
