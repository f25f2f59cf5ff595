"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates DiffEqOperators.jl's stencil-apply path in C++
(``deo_oracle.cpp``).  Only the test-suite, the smoke check and the bench's
CPU-baseline leg import this module; the product package never does.

Arrays follow Julia's layout: N-D arrays are column-major (axis 1 contiguous),
so numpy arrays passed here are Fortran-ordered.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libdeo_oracle.so")
_lib = None

_dp = C.POINTER(C.c_double)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, a few seconds)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "deo_oracle.cpp"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_julia_powi.restype = C.c_double
        L.orc_julia_powi.argtypes = [C.c_double, C.c_long]
        L.orc_calculate_weights.argtypes = [C.c_int, C.c_double, _dp, C.c_int, _dp]
        L.orc_centered.restype = C.c_void_p
        L.orc_centered.argtypes = [C.c_int, C.c_int, _dp, C.c_int, C.c_int]
        L.orc_upwind.restype = C.c_void_p
        L.orc_upwind.argtypes = [C.c_int, C.c_int, _dp, C.c_int, C.c_int, C.c_int]
        L.orc_op_free.argtypes = [C.c_void_p]
        L.orc_op_abs.restype = C.c_void_p
        L.orc_op_abs.argtypes = [C.c_void_p]
        L.orc_op_info.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.orc_op_tables.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.orc_op_set_coeff.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int]
        L.orc_op_scale_coeff.argtypes = [C.c_void_p, _dp, C.c_int]
        L.orc_robin.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_void_p]
        L.orc_general.argtypes = [_dp, C.c_int, _dp, C.c_int, _dp, C.c_int, C.c_int, C.c_void_p]
        L.orc_bc_size.restype = C.c_int
        L.orc_bc_ghosts.argtypes = [C.c_void_p, _dp, C.c_long, _dp, _dp]
        L.orc_mul_generic.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
        L.orc_mul_padded.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp, _dp, C.c_int]
        L.orc_apply_nd.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.c_void_p,
                                   C.POINTER(_dp), C.c_int, C.POINTER(C.c_long), _dp, _dp, C.c_int, C.c_int]
        L.orc_abs_scale_nd.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.c_void_p,
                                       C.POINTER(_dp), C.c_int, C.POINTER(C.c_long), _dp, _dp]
        L.orc_apply_nd_lines.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.c_void_p,
                                         C.POINTER(_dp), C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_long), _dp,
                                         _dp, C.c_int, C.c_int]
        L.orc_abs_scale_nd_lines.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.c_void_p,
                                             C.POINTER(_dp), C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_long),
                                             _dp, _dp]
        L.orc_array_op.argtypes = [C.c_void_p, _dp]
        L.orc_array_bc.argtypes = [C.c_void_p, C.c_long, _dp, _dp]
        L.orc_ssprk3.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.c_void_p,
                                 C.POINTER(_dp), C.c_int, C.POINTER(C.c_long), _dp, C.c_double, C.c_int, C.c_int]
        L.orc_vector_calculus.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_void_p), _dp, _dp, C.c_int, C.c_int]
        L.orc_mul_nd.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_long), C.POINTER(C.c_long), _dp, _dp,
                                 C.c_int, C.c_int]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64
    return a.ctypes.data_as(_dp)


def _f64(x) -> np.ndarray:
    return np.ascontiguousarray(np.atleast_1d(np.asarray(x, dtype=np.float64)).ravel())


def julia_powi(x: float, n: int) -> float:
    return lib().orc_julia_powi(float(x), int(n))


def calculate_weights(order: int, x0: float, x: Sequence[float]) -> np.ndarray:
    xv = _f64(x)
    out = np.zeros_like(xv)
    if lib().orc_calculate_weights(order, float(x0), _ptr(xv), len(xv), _ptr(out)) != 0:
        raise AssertionError("Not enough points for the requested order.")
    return out


class Op:
    """A DerivativeOperator built by the oracle's restated constructors."""

    def __init__(self, handle, axis: int):
        if not handle:
            raise AssertionError("invalid operator arguments")
        self.h = C.c_void_p(handle)
        self.axis = axis
        info = (C.c_int * 13)()
        lib().orc_op_info(self.h, info)
        (self.d, self.a, self.len, self.stl, self.bstl, self.bpc, self.off, wind, uniform,
         self.n_st, self.n_low, self.n_high, self.coeff_func_sign) = list(info)
        self.wind, self.uniform = bool(wind), bool(uniform)

    def __del__(self):
        try:
            lib().orc_op_free(self.h)
        except Exception:
            pass

    def tables(self):
        halves = 2 if (self.wind and not self.uniform) else 1
        st = np.zeros(halves * self.n_st * self.stl)
        lo = np.zeros(max(1, halves * self.n_low * self.bstl))
        hi = np.zeros(max(1, halves * self.n_high * self.bstl))
        co = np.zeros(self.len)
        lib().orc_op_tables(self.h, _ptr(st), _ptr(lo), _ptr(hi), _ptr(co))
        return (st.reshape(halves, self.n_st, self.stl),
                lo[: halves * self.n_low * self.bstl].reshape(halves, self.n_low, self.bstl),
                hi[: halves * self.n_high * self.bstl].reshape(halves, self.n_high, self.bstl),
                co)

    def set_coefficients(self, c, coeff_func_sign: int = 0):
        cv = _f64(c)
        lib().orc_op_set_coeff(self.h, _ptr(cv), len(cv), int(coeff_func_sign))
        self.coeff_func_sign = int(coeff_func_sign)
        return self

    def scale(self, c):
        cv = _f64(c)
        lib().orc_op_scale_coeff(self.h, _ptr(cv), len(cv))
        return self

    def abs(self) -> "Op":
        """|tables| and |coefficients| (for the sum|c_k u_k| tolerance).  Sign
        decisions of upwind rows follow |coefficients| >= 0, so use this only
        with the upwind direction frozen (see abs_terms)."""
        return Op(lib().orc_op_abs(self.h), self.axis)

    def array(self) -> np.ndarray:
        M = np.zeros((self.len, self.len + 2), order="F")
        lib().orc_array_op(self.h, M.ctypes.data_as(_dp))
        return M

    def mul_generic(self, x, out=None, overwrite=True) -> np.ndarray:
        xv = _f64(x)
        assert len(xv) == self.len + 2
        o = np.zeros(self.len) if out is None else out
        lib().orc_mul_generic(self.h, _ptr(xv), _ptr(o), int(overwrite))
        return o

    def mul_padded(self, l, u, r, out=None, overwrite=True) -> np.ndarray:
        uv = _f64(u)
        o = np.zeros(self.len) if out is None else out
        lib().orc_mul_padded(self.h, float(l), float(r), _ptr(uv), _ptr(o), int(overwrite))
        return o


def _dx_arg(dx):
    dxv = _f64(dx)
    return dxv, len(dxv)


def centered(d: int, a: int, dx, length: int, coeff=None, axis: int = 1) -> Op:
    dxv, n = _dx_arg(dx)
    op = Op(lib().orc_centered(d, a, _ptr(dxv), n, length), axis)
    if coeff is not None:
        op.set_coefficients(coeff, 1 if np.ndim(coeff) == 0 and coeff >= 0 else (-1 if np.ndim(coeff) == 0 else 0))
    return op


def upwind(d: int, a: int, dx, length: int, coeff=None, offside: int = 0, axis: int = 1) -> Op:
    dxv, n = _dx_arg(dx)
    op = Op(lib().orc_upwind(d, a, _ptr(dxv), n, length, offside), axis)
    if coeff is not None:
        sign = 0
        if np.ndim(coeff) == 0:
            sign = 1 if coeff >= 0 else -1
        op.set_coefficients(coeff, sign)
    return op


class BC(C.Structure):
    _fields_ = [("kind", C.c_int), ("ml", C.c_int), ("mr", C.c_int),
                ("al", C.c_double * 32), ("ar", C.c_double * 32),
                ("bl", C.c_double), ("br", C.c_double)]

    @property
    def a_l(self):
        return np.array(self.al[: self.ml])

    @property
    def a_r(self):
        return np.array(self.ar[: self.mr])

    def ghosts(self, u):
        uv = _f64(u)
        l, r = C.c_double(), C.c_double()
        lib().orc_bc_ghosts(C.byref(self), _ptr(uv), len(uv), C.byref(l), C.byref(r))
        return l.value, r.value

    def array(self, N: int):
        QL = np.zeros((N + 2, N), order="F")
        Qb = np.zeros(N + 2)
        lib().orc_array_bc(C.byref(self), N, QL.ctypes.data_as(_dp), _ptr(Qb))
        return QL, Qb


def robin(l, r, dx, order: int = 1) -> BC:
    q = BC()
    lv, rv = _f64(l), _f64(r)
    dxv, n = _dx_arg(dx)
    if lib().orc_robin(_ptr(lv), _ptr(rv), _ptr(dxv), n, order, C.byref(q)) != 0:
        raise ValueError("order too large or dx too short")
    return q


def general(al, ar, dx, order: int = 1) -> BC:
    q = BC()
    alv, arv = _f64(al), _f64(ar)
    dxv, n = _dx_arg(dx)
    if lib().orc_general(_ptr(alv), len(alv), _ptr(arv), len(arv), _ptr(dxv), n, order, C.byref(q)) != 0:
        raise ValueError("order too large or dx too short")
    return q


def dirichlet(l: float, r: float) -> BC:
    """DirichletBC(αl, αr) = RobinBC((1,0,αl), (1,0,αr), 1.0, 2) (bc_operators.jl:175-177)."""
    return robin((1.0, 0.0, l), (1.0, 0.0, r), 1.0, 2)


def dirichlet0() -> BC:
    return dirichlet(0.0, 0.0)


def neumann(a, dx, order: int = 1) -> BC:
    return robin((0.0, 1.0, a[0]), (0.0, 1.0, a[1]), dx, order)


def neumann0(dx, order: int = 1) -> BC:
    return neumann((0.0, 0.0), dx, order)


def periodic() -> BC:
    q = BC()
    q.kind = 1
    return q


class _Args:
    """ctypes argument block shared by apply / abs_scale / ssprk3."""

    def __init__(self, terms, u: np.ndarray):
        """terms: (Op, BC[, field[, line_bcs]]); line_bcs (may be None) is a
        sequence of one BC per line of the term, in the column-major order of
        the other axes (MultiDimBC{dim}(BCs::Array))."""
        self.u = np.asfortranarray(u, dtype=np.float64)
        self.sizes = (C.c_long * self.u.ndim)(*self.u.shape)
        n = self.n = len(terms)
        self.ops = (C.c_void_p * n)(*[t[0].h.value for t in terms])
        self.axes = (C.c_int * n)(*[t[0].axis for t in terms])
        self.bcs = (BC * n)(*[t[1] for t in terms])
        self.keep, self.fptrs = [], (_dp * n)()
        for i, t in enumerate(terms):
            f = t[2] if len(t) > 2 else None
            if f is not None:
                f = np.asfortranarray(f, dtype=np.float64)
                self.keep.append(f)
                self.fptrs[i] = f.ctypes.data_as(_dp)
            else:
                self.fptrs[i] = _dp()
        self.lines = (C.c_void_p * n)()
        self.has_lines = False
        for i, t in enumerate(terms):
            lb = t[3] if len(t) > 3 else None
            if lb is not None:
                arr = (BC * len(lb))(*lb)
                self.keep.append(arr)
                self.lines[i] = C.cast(arr, C.c_void_p)
                self.has_lines = True

    def head(self):
        return (self.n, self.ops, self.axes, C.cast(self.bcs, C.c_void_p), self.fptrs, self.u.ndim, self.sizes)


def apply(terms, u: np.ndarray, out: np.ndarray | None = None, overwrite: bool = True,
          nthreads: int = 1) -> np.ndarray:
    """sum_t (L_t*Q_t)*u.  terms: list of (Op, BC[, field]); u Fortran-ordered."""
    a = _Args(terms, u)
    o = np.zeros(a.u.shape, order="F") if out is None else out
    if a.has_lines:
        h = a.head()
        rc = lib().orc_apply_nd_lines(*h[:5], a.lines, *h[5:], a.u.ctypes.data_as(_dp), o.ctypes.data_as(_dp),
                                      int(overwrite), int(nthreads))
    else:
        rc = lib().orc_apply_nd(*a.head(), a.u.ctypes.data_as(_dp), o.ctypes.data_as(_dp), int(overwrite),
                                int(nthreads))
    if rc != 0:
        raise AssertionError("size mismatch between operator and array")
    return o


def abs_scale(terms, u: np.ndarray) -> np.ndarray:
    """sum_k |c_k * u_k| per point, ghost terms expanded (parity tolerance scale)."""
    a = _Args(terms, u)
    o = np.zeros(a.u.shape, order="F")
    if a.has_lines:
        h = a.head()
        rc = lib().orc_abs_scale_nd_lines(*h[:5], a.lines, *h[5:], a.u.ctypes.data_as(_dp), o.ctypes.data_as(_dp))
    else:
        rc = lib().orc_abs_scale_nd(*a.head(), a.u.ctypes.data_as(_dp), o.ctypes.data_as(_dp))
    if rc != 0:
        raise AssertionError("size mismatch between operator and array")
    return o


def nonlinear_diffusion(n: int, m: int, approx: int, p, q, dx, nknots: int, absolute: bool = False) -> np.ndarray:
    """nonlinear_diffusion!{N}(du, n, m, approx, p, q, dx, nknots) as the reference
    computes it (derivative_operator.jl:34-66): the operators by the generic
    method on the padded vectors (orc_mul_generic), the broadcasts in numpy in
    the reference's operation order (no contraction).  absolute=True gives the
    same sum over |weights| and |values| (the error scale)."""
    p = _f64(p)
    q = _f64(q)

    def D(k, x):
        op = centered(k, approx, dx, nknots)
        if absolute:
            return op.abs().mul_generic(np.abs(x))
        return op.mul_generic(x)
    pp, qq = (np.abs(p), np.abs(q)) if absolute else (p, q)
    du = (D(m, q) if m > 0 else qq[1:nknots + 1]) * D(n, p)
    b = 1
    for ell in range(1, n):
        b = b * (n - ell + 1) // ell
        du = du + (float(b) * D(ell + m, q)) * D(n - ell, p)
    return du + D(m + n, q) * pp[1:nknots + 1]


def mul_nd(op: Op, M, out_shape=None, out=None, overwrite: bool = True, absolute: bool = False) -> np.ndarray:
    """L*M / mul!(x_temp, L, M; overwrite) on an already padded array M
    (derivative_operator_functions.jl:17-69, 150-163), restated in
    deo_oracle.cpp (orc_mul_nd); the operator acts on axis op.axis.  out_shape
    defaults to M's shape with that axis 2 shorter (L*M).  absolute=True gives
    sum_k |c_k u_k| per point with the same rows (the tolerance scale)."""
    M = np.asfortranarray(M, dtype=np.float64)
    a = op.axis - 1
    if out_shape is None:
        out_shape = tuple(n - 2 if b == a else n for b, n in enumerate(M.shape))
    o = np.zeros(out_shape, order="F") if out is None else out
    nd = M.ndim
    osz = (C.c_long * nd)(*o.shape)
    isz = (C.c_long * nd)(*M.shape)
    if lib().orc_mul_nd(op.h, op.axis, nd, osz, isz, M.ctypes.data_as(_dp), o.ctypes.data_as(_dp),
                        int(overwrite or absolute), int(absolute)) != 0:
        raise AssertionError("size mismatch between the operator, x_temp and M")
    return o


def mul_combination(ops, M, x_temp, absolute: bool = False) -> np.ndarray:
    """mul!(x_temp, L1 + L2 + ..., M) for DerivativeOperators on an already
    padded M, restated from the reference: vectors through the cache loop of
    composite_operators.jl:76-83; 2-D and 3-D arrays through the fallback
    branch of derivative_operator_functions.jl:380-463 (2-D) and 771-800 (3-D),
    which every operator with Vector coefficients takes: operator k reads
    view(M, 1:x_temp_1, ..., 1:(x_temp_axis + 2), ...), i.e. the block of M
    that begins at index 1 on every axis, except that in 2-D an operator whose
    other axis no operator of the sum acts on reads M whole.  The first
    operator overwrites x_temp, the others add into it (mul!(...; overwrite =
    false)).  absolute=True gives sum_k |c_k u_k| over all operators' rows (the
    tolerance scale)."""
    M = np.asfortranarray(M, dtype=np.float64)
    nd = M.ndim
    if nd not in (1, 2, 3):
        raise AssertionError("mul! of a sum of operators is defined for vectors and 2-D / 3-D arrays")
    operated = {op.axis for op in ops}
    for k, op in enumerate(ops):
        V = M
        others = {b for b in range(1, nd + 1) if b != op.axis}
        if nd == 3 or (nd == 2 and others & operated):
            V = np.asfortranarray(M[tuple(slice(0, x_temp.shape[b - 1] + (2 if b == op.axis else 0))
                                          for b in range(1, nd + 1))])
        if not absolute:
            mul_nd(op, V, out_shape=x_temp.shape, out=x_temp, overwrite=(k == 0))
            continue
        a = mul_nd(op, V, out_shape=x_temp.shape, absolute=True)
        if k == 0:
            x_temp[...] = a
        else:
            x_temp += a
    return x_temp


GRADIENT, DIVERGENCE, CURL = 0, 1, 2


def vector_calculus(kind: int, ops, M, out=None, overwrite: bool = True, absolute: bool = False) -> np.ndarray:
    """Gradient (kind 0), Divergence (1) or Curl (2) of the padded array M as
    the reference computes `A * M` (overwrite) or `mul!(out, .., A, M)`
    (vector_calculus_operators.jl:47-73, vector_calculus_convolutions.jl),
    restated in deo_oracle.cpp (orc_vector_calculus).  ops[a] is the operator
    of axis a+1.  M and the result are Fortran-ordered: Gradient M has size
    len + 2 on every axis and the result (len..., N); Divergence M has
    (len + 2..., N) and the result (len...); Curl M has (len + 2 ...,3) and the
    result (len..., 3).  absolute=True gives sum_k |c_k u_k| per entry."""
    nd = len(ops)
    lens = [op.len for op in ops]
    shape = tuple(lens) + ((nd,) if kind == GRADIENT else ((3,) if kind == CURL else ()))
    x = np.asfortranarray(np.abs(M) if absolute else M, dtype=np.float64)
    use = [op.abs() for op in ops] if absolute else list(ops)
    o = np.zeros(shape, order="F") if out is None else out
    assert o.flags.f_contiguous and o.dtype == np.float64 and o.shape == shape
    handles = (C.c_void_p * nd)(*[op.h.value for op in use])
    rc = lib().orc_vector_calculus(kind, nd, handles, x.ctypes.data_as(_dp), o.ctypes.data_as(_dp),
                                   int(overwrite or absolute), int(absolute))
    if rc != 0:
        raise AssertionError("invalid vector-calculus arguments")
    return o


def dot_product(A, B) -> np.ndarray:
    """dot_product(A, B) (vector_algebraic_operations.jl:3-28): sum over the
    last axis of A .* B, components added in order from zero, each product
    rounded (plain Julia arithmetic)."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    u = np.zeros(A.shape[:-1])
    for i in range(A.shape[-1]):
        u = u + A[..., i] * B[..., i]
    return u


def cross_product(A, B) -> np.ndarray:
    """cross_product(A, B) (vector_algebraic_operations.jl:30-52) of two
    (s1, s2, s3, 3) arrays, each product rounded before the difference."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    u = np.empty(A.shape, order="F")
    u[..., 0] = A[..., 1] * B[..., 2] - A[..., 2] * B[..., 1]
    u[..., 1] = A[..., 2] * B[..., 0] - A[..., 0] * B[..., 2]
    u[..., 2] = A[..., 0] * B[..., 1] - A[..., 1] * B[..., 0]
    return u


def square_norm(A) -> np.ndarray:
    """square_norm(A) (vector_algebraic_operations.jl:54-62): dot_product(A, A)
    then `u .^ 0.5`, taken here as the correctly rounded square root (Julia's
    Float64 power is within one ulp of it)."""
    return np.sqrt(dot_product(A, A))


def ghost_solve(op: Op, bc: BC, u: np.ndarray, axis: int = 1):
    """A \\ u for A = L*Q (ghost_derivative_operator.jl:39-58): (A_l, A_b) =
    Array(L) * Array(Q) (concretization.jl:914-918; Array(PeriodicBC) wraps
    around), then A_l x = u - A_b by a dense LU (numpy), line by line along
    `axis` (1-based) of a Fortran-ordered array.  Returns (x, cond(A_l))."""
    Lm = op.array()
    QL, Qb = bc.array(op.len)
    Al = Lm @ QL
    Ab = Lm @ Qb
    x = np.moveaxis(np.asarray(u, dtype=np.float64), axis - 1, 0)
    shp = x.shape
    rhs = x.reshape(shp[0], -1) - Ab[:, None]
    sol = np.linalg.solve(Al, rhs)
    out = np.moveaxis(sol.reshape(shp), 0, axis - 1)
    return np.asfortranarray(out), float(np.linalg.cond(Al))


def ulp_tolerance(terms, u: np.ndarray, n_ulp: float = 4.0) -> np.ndarray:
    """Per-point tolerance: n_ulp units in the last place of sum_k |c_k u_k|."""
    return n_ulp * np.spacing(abs_scale(terms, u))


def ssprk3(terms, u0: np.ndarray, dt: float, nsteps: int, nthreads: int = 1) -> np.ndarray:
    """SSP-RK3 (Shu-Osher) steps of du/dt = sum_t L_t Q_t u."""
    a = _Args(terms, np.array(u0, dtype=np.float64, order="F", copy=True))
    rc = lib().orc_ssprk3(*a.head(), a.u.ctypes.data_as(_dp), float(dt), int(nsteps), int(nthreads))
    if rc != 0:
        raise AssertionError("size mismatch")
    return a.u


def concretize_probe(terms, shape) -> tuple[np.ndarray, np.ndarray]:
    """(A_l, A_b) of the affine map u -> sum_t L_t Q_t u, by unit-vector probes
    (the reference's own convert_by_multiplication test helper,
    test/DerivativeOperators/derivative_operators_interface.jl:102-117)."""
    n = int(np.prod(shape))
    zero = np.zeros(shape, order="F")
    Ab = apply(terms, zero).ravel(order="F")
    Al = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        col = apply(terms, e.reshape(shape, order="F")).ravel(order="F")
        Al[:, j] = col - Ab
    return Al, Ab
