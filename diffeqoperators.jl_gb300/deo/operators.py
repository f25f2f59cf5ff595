"""Host-side mirror of DiffEqOperators.jl's operator API over libdeo.

Names, argument meaning and errors follow the reference:

    L  = CenteredDifference(2, 2, h, N)              # CenteredDifference{1}
    Q  = Dirichlet0BC(np.float64)
    du = L * Q * u                                    # (L*Q)*u, u a CUDA tensor
    mul_(du, L * Q, u)                                # mul!(du, L*Q, u)

    Dxx = CenteredDifference(2, 4, h, n, axis=1)      # CenteredDifference{1}
    Dyy = CenteredDifference(2, 4, h, n, axis=2)      # CenteredDifference{2}
    Qc  = compose(*RobinBC((1., .5, 0.), (1., .5, 0.), (h, h, h), 1, (n, n, n)))
    du  = (Dxx + Dyy + Dzz) * Qc * u

Arrays use Julia's layout: an N-D array of size (s1, s2, ...) is a
column-major (Fortran-ordered) tensor whose axis 1 is contiguous; build one
with `julia_array(...)` or pass `x.permute(...)` views of that layout.
Device tensors run on the current torch stream; numpy arrays go through the
library's host-buffer entry point (copies included).
"""
from __future__ import annotations

import ctypes as C
import numbers
from typing import Iterable, Sequence

import numpy as np

from . import _lib as L
from ._lib import BCStruct, DeoArgError, DeoShapeError, Term, check

_dp = C.POINTER(C.c_double)


def _f64(x) -> np.ndarray:
    return np.ascontiguousarray(np.atleast_1d(np.asarray(x, dtype=np.float64)).ravel())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def calculate_weights(order: int, x0: float, x: Sequence[float]) -> np.ndarray:
    """Fornberg weights (fornberg.jl:7-62)."""
    xv = _f64(x)
    out = np.zeros_like(xv)
    if order >= len(xv):
        raise AssertionError("Not enough points for the requested order.")
    check(L.lib().deo_calculate_weights(int(order), float(x0), _ptr(xv), len(xv), _ptr(out)))
    return out


# ---------------------------------------------------------------------------
# torch / layout helpers
# ---------------------------------------------------------------------------
def _torch():
    import torch
    return torch


def fortran_strides(shape: Sequence[int]) -> tuple:
    s, out = 1, []
    for n in shape:
        out.append(s)
        s *= n
    return tuple(out)


def julia_array(shape: Sequence[int], dtype=None, device="cuda", fill=None):
    """A column-major torch tensor of Julia size `shape` (axis 1 contiguous)."""
    torch = _torch()
    dtype = dtype or torch.float64
    t = torch.empty(tuple(reversed(tuple(shape))), dtype=dtype, device=device).permute(
        *reversed(range(len(shape))))
    if fill is not None:
        t.fill_(fill)
    return t


def to_julia_layout(x):
    """Copy a tensor/ndarray into Julia (column-major) layout, same Julia size."""
    torch = _torch()
    if isinstance(x, np.ndarray):
        return np.asfortranarray(x)
    out = julia_array(tuple(x.shape), x.dtype, x.device)
    out.copy_(x)
    return out


def _check_layout(x, what="u"):
    if tuple(x.stride()) != fortran_strides(x.shape):
        raise DeoArgError(2, f"{what} must be column-major (Julia layout, axis 1 contiguous); "
                             f"got strides {tuple(x.stride())} for size {tuple(x.shape)}")


def _dtype_code(x) -> int:
    torch = _torch()
    if x.dtype == torch.float64:
        return L.DEO_F64
    if x.dtype == torch.float32:
        return L.DEO_F32
    raise DeoArgError(2, f"unsupported dtype {x.dtype} (Float64 and Float32 only)")


def _stream_ptr():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


# ---------------------------------------------------------------------------
# Derivative operators
# ---------------------------------------------------------------------------
class DerivativeOperator:
    """DerivativeOperator (derivative_operator.jl:14-29) backed by a deo_operator."""

    __array_ufunc__ = None  # `c * L` with a numpy vector c goes to __rmul__

    def __init__(self, handle: int, axis: int = 1):
        self._h = C.c_void_p(handle)
        self.axis = int(axis)
        self._desc = L.OperatorDesc()
        self.coeff_func = None  # a 4-argument function (coefficients, u, p, t) set by `f * L`
        self._version = 0       # bumped when update_coefficients rewrites the coefficients
        self._refresh()

    def _refresh(self):
        check(L.lib().deo_operator_describe(self._h, C.byref(self._desc)))

    def __del__(self):
        try:
            if self._h:
                L.lib().deo_operator_destroy(self._h)
                self._h = None
        except Exception:
            pass

    # fields -------------------------------------------------------------
    derivative_order = property(lambda s: s._desc.derivative_order)
    approximation_order = property(lambda s: s._desc.approximation_order)
    len = property(lambda s: s._desc.len)
    stencil_length = property(lambda s: s._desc.stencil_length)
    boundary_stencil_length = property(lambda s: s._desc.boundary_stencil_length)
    boundary_point_count = property(lambda s: s._desc.boundary_point_count)
    offside = property(lambda s: s._desc.offside)
    winding = property(lambda s: bool(s._desc.winding))
    uniform = property(lambda s: bool(s._desc.uniform))
    coeff_func_sign = property(lambda s: s._desc.coeff_func_sign)

    def _halves(self):
        return 2 if (self.winding and not self.uniform) else 1

    def _table(self, ptr, rows, width):
        n = self._halves() * rows * width
        if n == 0:
            return np.zeros((self._halves(), rows, width))
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy().reshape(self._halves(), rows, width)

    @property
    def stencil_coefs(self):
        d = self._desc
        return self._table(d.stencil_coefs, d.n_stencil_rows, d.stencil_length)

    @property
    def low_boundary_coefs(self):
        d = self._desc
        return self._table(d.low_boundary_coefs, d.n_low_rows, d.boundary_stencil_length)

    @property
    def high_boundary_coefs(self):
        d = self._desc
        return self._table(d.high_boundary_coefs, d.n_high_rows, d.boundary_stencil_length)

    @property
    def coefficients(self):
        return np.ctypeslib.as_array(self._desc.coefficients, shape=(self.len,)).copy()

    @property
    def size(self):
        return (self.len, self.len + 2)

    def copy(self) -> "DerivativeOperator":
        h = C.c_void_p()
        check(L.lib().deo_operator_clone(self._h, C.byref(h)))
        out = DerivativeOperator(h.value, self.axis)
        out.coeff_func = self.coeff_func  # c * L keeps A.coeff_func (derivative_operator_functions.jl:165-197)
        return out

    # algebra ------------------------------------------------------------
    def __rmul__(self, c):
        """c * L scales the coefficients (derivative_operator_functions.jl:165-197);
        f * L for a function f keeps them and stores f as the coefficient function
        that update_coefficients calls (abstract_operator_functions.jl:174-194)."""
        if callable(c) and not isinstance(c, (numbers.Number, np.ndarray)):
            out = self.copy()
            cv = self.coefficients
            check(L.lib().deo_operator_set_coefficients(out._h, _ptr(cv), cv.size, 0))
            out._refresh()
            out.coeff_func = c
            return out
        if isinstance(c, numbers.Number) or (isinstance(c, np.ndarray) and c.ndim <= 1):
            cv = _f64(c)
            if cv.size not in (1, self.len):
                raise DimensionMismatch(f"length of c ({cv.size}) must match length of A ({self.len})")
            out = self.copy()
            check(L.lib().deo_operator_scale_coefficients(out._h, _ptr(cv), cv.size))
            out._refresh()
            return out
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, (AtomicBC, MultiDimensionalBC)):
            return GhostDerivativeOperator(self, other)
        if isinstance(other, DerivativeOperator) or isinstance(other, numbers.Number):
            return NotImplemented
        return _mul_padded(self, other)

    def __add__(self, other):
        return DiffEqOperatorCombination([self]) + other

    def __neg__(self):
        return (-1.0) * self

    def __call__(self, *args):
        return _ode_call(self, args, update=False)

    def update_coefficients(self, u, p, t):
        """update_coefficients!(L, u, p, t) (abstract_operator_functions.jl:190-194):
        coeff_func(coefficients, u, p, t) rewrites the coefficient vector in place."""
        if self.coeff_func is None:
            return
        cv = self.coefficients
        self.coeff_func(cv, u, p, t)
        cv = _f64(cv)
        if cv.size != self.len:
            raise DimensionMismatch(f"the coefficient function left {cv.size} coefficients, len is {self.len}")
        check(L.lib().deo_operator_set_coefficients(self._h, _ptr(cv), cv.size, 0))
        self._refresh()
        self._version += 1

    def array(self, N: int | None = None) -> np.ndarray:
        """Array(L): len x (len+2) (concretization.jl:8-52, :556-671)."""
        M = np.zeros((self.len, self.len + 2), order="F")
        check(L.lib().deo_operator_array(self._h, M.ctypes.data_as(_dp)))
        return M

    def banded(self):
        """BandedMatrix(L) (concretization.jl:123-128 centred, :794-890 upwind):
        (data, (lower, upper)) with the reference's bandwidths and data the
        (lower+upper+1) x (len+2) band storage (entry (i, j) at row upper+i-j
        of column j, 0-based here), BandedMatrices.jl's `bandeddata` layout."""
        lo, up = C.c_int(), C.c_int()
        check(L.lib().deo_operator_banded(self._h, C.byref(lo), C.byref(up), None))
        data = np.zeros((lo.value + up.value + 1, self.len + 2), order="F")
        check(L.lib().deo_operator_banded(self._h, C.byref(lo), C.byref(up), data.ctypes.data_as(_dp)))
        return data, (lo.value, up.value)


def _ode_call(A, args, update: bool):
    """(A)(u, p, t) = A*u and (A)(du, u, p, t) = mul!(du, A, u), the (u,p,t)
    interface: L*Q terms and their sums first run update_coefficients
    (DiffEqOperators.jl:67-76), a bare DerivativeOperator does not
    (abstract_operator_functions.jl:197-198)."""
    if update and len(args) in (3, 4):
        A.update_coefficients(*args[-3:])
    if len(args) == 3:
        return A * args[0]
    if len(args) == 4:
        return mul_(args[0], A, args[1])
    raise TypeError("call as A(u, p, t) or A(du, u, p, t)")


class DimensionMismatch(DeoShapeError):
    def __init__(self, msg):
        super().__init__(1, msg)


def _apply_coeff(op: DerivativeOperator, coeff_func):
    """compute_coeffs! on a fresh operator (coefficient_functions.jl:7-46)."""
    if coeff_func is None:
        return op
    if isinstance(coeff_func, numbers.Number):
        cv = _f64(coeff_func)
        sign = 1 if coeff_func >= 0 else -1
    elif callable(coeff_func):
        cur = op.coefficients * 0.0
        try:
            vals = np.asarray(coeff_func(cur), dtype=np.float64)
            if vals.shape != cur.shape:
                raise TypeError
        except TypeError:
            vals = np.array([coeff_func(c) for c in cur], dtype=np.float64)
        cv, sign = _f64(vals), 0
    else:
        cv, sign = _f64(coeff_func), 0
        if cv.size != op.len:
            raise DimensionMismatch(f"coefficient vector has {cv.size} entries, operator len {op.len}")
    check(L.lib().deo_operator_set_coefficients(op._h, _ptr(cv), cv.size, sign))
    op._refresh()
    return op


def _dx_args(dx):
    dxv = _f64(dx)
    return dxv, dxv.size


def CenteredDifference(derivative_order: int, approximation_order: int, dx, len: int, coeff_func=1,
                       axis: int = 1) -> DerivativeOperator:
    """CenteredDifference{axis}(d, a, dx, len, coeff_func) (derivative_operator.jl:81-205)."""
    if approximation_order <= 1:
        raise AssertionError("approximation_order must be greater than 1.")
    dxv, n = _dx_args(dx)
    h = C.c_void_p()
    check(L.lib().deo_centered_difference(int(derivative_order), int(approximation_order), _ptr(dxv), n,
                                          int(len), C.byref(h)))
    return _apply_coeff(DerivativeOperator(h.value, axis), coeff_func)


def UpwindDifference(derivative_order: int, approximation_order: int, dx, len: int, coeff_func=1,
                     offside: int = 0, axis: int = 1) -> DerivativeOperator:
    """UpwindDifference{axis}(d, a, dx, len, coeff_func; offside) (derivative_operator.jl:454-639)."""
    if offside < 0:
        raise AssertionError("Number of offside points should be non-negative")
    if offside > (derivative_order + approximation_order - 1) // 2:
        raise AssertionError("Number of offside points should not exceed the primary wind points")
    dxv, n = _dx_args(dx)
    h = C.c_void_p()
    check(L.lib().deo_upwind_difference(int(derivative_order), int(approximation_order), _ptr(dxv), n, int(len),
                                        int(offside), C.byref(h)))
    return _apply_coeff(DerivativeOperator(h.value, axis), coeff_func)


def operator_from_tables(desc: dict, axis: int = 1) -> DerivativeOperator:
    """Build from a DerivativeOperator's own fields (what the Julia shim passes)."""
    keep = {}
    d = L.OperatorDesc()
    for k in ("derivative_order", "approximation_order", "len", "stencil_length", "boundary_stencil_length",
              "boundary_point_count", "offside", "winding", "uniform", "coeff_func_sign", "n_stencil_rows",
              "n_low_rows", "n_high_rows"):
        setattr(d, k, int(desc[k]))
    for k in ("stencil_coefs", "low_boundary_coefs", "high_boundary_coefs", "coefficients"):
        a = _f64(desc[k])
        keep[k] = a
        setattr(d, k, _ptr(a))
    h = C.c_void_p()
    check(L.lib().deo_operator_from_tables(C.byref(d), C.byref(h)))
    return DerivativeOperator(h.value, axis)


# ---------------------------------------------------------------------------
# Boundary conditions
# ---------------------------------------------------------------------------
class AtomicBC:
    """An affine ghost map (RobinBC, GeneralBC, Dirichlet/Neumann) or PeriodicBC."""

    def __init__(self, s: BCStruct, name: str):
        self._s = s
        self.name = name

    @property
    def a_l(self):
        return np.array(self._s.a_l[: self._s.m_l])

    @property
    def a_r(self):
        return np.array(self._s.a_r[: self._s.m_r])

    @property
    def b_l(self):
        return self._s.b_l

    @property
    def b_r(self):
        return self._s.b_r

    @property
    def periodic(self):
        return self._s.kind == L.DEO_BC_PERIODIC

    def array(self, N: int):
        """Array(Q, N) -> (Q_L, Q_b) (concretization.jl:187-192, :227-230)."""
        QL = np.zeros((N + 2, N), order="F")
        Qb = np.zeros(N + 2)
        check(L.lib().deo_bc_array(C.byref(self._s), int(N), QL.ctypes.data_as(_dp), _ptr(Qb)))
        return QL, Qb

    def __mul__(self, u):
        """Q*u -> the padded vector [ghost_l; u; ghost_r] as a numpy array (bc_operators.jl:188-192)."""
        uv = np.asarray(u, dtype=np.float64)
        if uv.ndim != 1:
            raise DeoArgError(2, "Q*u materialises a padded Vector only; apply N-D BCs through L*Q*u")
        if self.periodic:
            return np.concatenate([[uv[-1]], uv, [uv[0]]])
        l = float(np.dot(self.a_l, uv[: self._s.m_l])) + self.b_l
        r = float(np.dot(self.a_r, uv[len(uv) - self._s.m_r:])) + self.b_r
        return np.concatenate([[l], uv, [r]])

    def __repr__(self):
        return f"{self.name}(a_l={self.a_l}, b_l={self.b_l}, a_r={self.a_r}, b_r={self.b_r})"


def _bc_call(fn, *args, name=""):
    s = BCStruct()
    check(fn(*args, C.byref(s)))
    return AtomicBC(s, name)


def _robin_atomic(l, r, dx, order=1):
    lv, rv = _f64(l), _f64(r)
    dxv, n = _dx_args(dx)
    return _bc_call(L.lib().deo_robin_bc, _ptr(lv), _ptr(rv), _ptr(dxv), n, int(order), name="RobinBC")


def _general_atomic(al, ar, dx, order=1):
    alv, arv = _f64(al), _f64(ar)
    dxv, n = _dx_args(dx)
    return _bc_call(L.lib().deo_general_bc, _ptr(alv), alv.size, _ptr(arv), arv.size, _ptr(dxv), n, int(order),
                    name="GeneralBC")


def RobinBC(l, r, dx, order=1, s=None, dim=None):
    """RobinBC(l, r, dx, order) (bc_operators.jl:26-60); with `s` (domain size)
    the multi-dimensional form: one MultiDimDirectionalBC per axis with
    dx = dxyz[axis] (multi_dim_bc_operators.jl:138-149)."""
    if s is None:
        return _robin_atomic(l, r, dx, order)
    if dim is not None:
        return MultiDimDirectionalBC(_robin_atomic(l, r, dx, order), dim, s)
    return tuple(MultiDimDirectionalBC(_robin_atomic(l, r, dx[k], order), k + 1, s) for k in range(len(s)))


def GeneralBC(al, ar, dx, order=1, s=None, dim=None):
    """GeneralBC(αl, αr, dx, order) (bc_operators.jl:90-169) / multi-D (multi_dim_bc_operators.jl:151-163)."""
    if s is None:
        return _general_atomic(al, ar, dx, order)
    if dim is not None:
        return MultiDimDirectionalBC(_general_atomic(al, ar, dx, order), dim, s)
    return tuple(MultiDimDirectionalBC(_general_atomic(al, ar, dx[k], order), k + 1, s) for k in range(len(s)))


def DirichletBC(l: float, r: float, s=None, dim=None):
    """DirichletBC(αl, αr) = RobinBC((1,0,αl),(1,0,αr),1,2) (bc_operators.jl:175-177)."""
    q = _bc_call(L.lib().deo_dirichlet_bc, float(l), float(r), name="DirichletBC")
    if s is None:
        return q
    if dim is not None:
        return MultiDimDirectionalBC(q, dim, s)
    return tuple(MultiDimDirectionalBC(q, k + 1, s) for k in range(len(s)))


def Dirichlet0BC(T=np.float64, s=None, dim=None):
    return DirichletBC(0.0, 0.0, s, dim)


def NeumannBC(alpha, dx, order=1, s=None, dim=None):
    """NeumannBC((αl, αr), dx, order) = RobinBC((0,1,αl),(0,1,αr),dx,order) (bc_operators.jl:173-174)."""
    if s is None:
        dxv, n = _dx_args(dx)
        return _bc_call(L.lib().deo_neumann_bc, float(alpha[0]), float(alpha[1]), _ptr(dxv), n, int(order),
                        name="NeumannBC")
    return RobinBC((0.0, 1.0, alpha[0]), (0.0, 1.0, alpha[1]), dx, order, s, dim)


def Neumann0BC(dx, order=1, s=None, dim=None):
    return NeumannBC((0.0, 0.0), dx, order, s, dim)


def PeriodicBC(T=np.float64, s=None, dim=None):
    """PeriodicBC(T) (bc_operators.jl:17-19); with `s`, the N-D form, which pads
    with the edge planes themselves (multi_dim_bc_operators.jl:221-228)."""
    q = _bc_call(L.lib().deo_periodic_bc, name="PeriodicBC")
    if s is None:
        return q
    if dim is not None:
        return MultiDimDirectionalBC(q, dim, s)
    return tuple(MultiDimDirectionalBC(q, k + 1, s) for k in range(len(s)))


class MultiDimensionalBC:
    pass


class MultiDimDirectionalBC(MultiDimensionalBC):
    """BCs extending dimension `axis` (multi_dim_bc_operators.jl:54-57): one
    atomic BC for every line (`s` = the array's size, :97-101), or an array of
    atomic BCs with one per line, shaped like the array without that axis
    (MultiDimBC{dim}(BCs::Array), :91-93; its lines get BCs[I, J] * u[I, :, J])."""

    def __init__(self, bc, axis: int, s: Sequence[int] | None = None):
        self.axis = int(axis)
        if isinstance(bc, AtomicBC):
            if s is None:
                raise DeoArgError(2, "an atomic BC needs the array size s")
            self.bc, self.lines, self.shape = bc, None, tuple(int(n) for n in s)
            self.ndims = len(self.shape)
        else:
            arr = np.asarray(bc, dtype=object)
            if arr.size == 0 or not all(isinstance(b, AtomicBC) for b in arr.ravel()):
                raise DeoArgError(2, "MultiDimBC{dim}(BCs): an array of atomic BCs is needed")
            self.bc, self.lines, self.shape = arr.ravel()[0], arr, None
            self.ndims = arr.ndim + 1

    def __add__(self, other):
        return compose(self, other)

    def check_size(self, shape) -> None:
        """The reference's assertion at Q*u (multi_dim_bc_operators.jl:211, 237)."""
        if self.lines is None:
            if tuple(self.shape) != tuple(shape):
                raise DeoShapeError(1, f"BC built for size {self.shape}, array has size {tuple(shape)}")
            return
        perp = tuple(n for k, n in enumerate(shape) if k != self.axis - 1)
        if tuple(self.lines.shape) != perp:
            raise DeoShapeError(1, f"Size of the BCs array in the MultiDimBC is incorrect, needs to be {perp} to "
                                   f"extend dimension {self.axis}, got {tuple(self.lines.shape)}")

    def line_bcs(self, axis: int):
        """The per-line BCs in the column-major order of the other axes, or None."""
        if axis != self.axis:
            raise DeoShapeError(1, f"operator differentiates along {axis} but the BC extends dimension {self.axis}")
        return None if self.lines is None else list(self.lines.ravel(order="F"))

    def bc_for(self, axis: int, ndims: int) -> AtomicBC:
        if axis != self.axis:
            raise DeoShapeError(1, f"operator differentiates along {axis} but the BC extends dimension {self.axis}")
        return self.bc


class ComposedMultiDimBC(MultiDimensionalBC):
    """compose(Qx, Qy, ...) (multi_dim_bc_operators.jl:178-192)."""

    def __init__(self, bcs: Sequence[MultiDimDirectionalBC]):
        self.parts = {b.axis: b for b in bcs}
        self.bcs = {b.axis: b.bc for b in bcs}
        self.shape = next((b.shape for b in bcs if b.shape is not None), None)
        self.ndims = bcs[0].ndims

    def check_size(self, shape) -> None:
        for b in self.parts.values():
            b.check_size(shape)

    def line_bcs(self, axis: int):
        return self.parts[axis].line_bcs(axis)

    def bc_for(self, axis: int, ndims: int) -> AtomicBC:
        return self.bcs[axis]


def compose(*bcs):
    if not bcs:
        raise DeoArgError(2, "compose needs at least one BC")
    n = bcs[0].ndims
    if len(bcs) != n:
        raise DeoArgError(2, "There must be enough BCs to cover every dimension - check that the number of "
                             "MultiDimBCs == N")
    axes = [b.axis for b in bcs]
    if len(set(axes)) != len(axes):
        raise DeoArgError(2, "There are multiple boundary conditions that extend along the same dimension - make "
                             "sure every dimension has a unique extension")
    return ComposedMultiDimBC(sorted(bcs, key=lambda b: b.axis))


def MultiDimBC(bc, s=None, dim: int | None = None):
    """MultiDimBC{dim}(BC, s) / MultiDimBC(BC, s) (multi_dim_bc_operators.jl:93-110);
    MultiDimBC(BCs, dim=dim) with an array of atomic BCs, one per line along
    `dim` (MultiDimBC{dim}(BCs::Array), :91-93)."""
    if not isinstance(bc, AtomicBC):
        if dim is None:
            raise DeoArgError(2, "MultiDimBC with an array of BCs needs dim")
        return MultiDimDirectionalBC(bc, dim)
    if dim is not None:
        return MultiDimDirectionalBC(bc, dim, s)
    return tuple(MultiDimDirectionalBC(bc, k + 1, s) for k in range(len(s)))


# ---------------------------------------------------------------------------
# L*Q and combinations
# ---------------------------------------------------------------------------
class FieldCoefficient:
    """An operator whose coefficient is a full field: it acts on each line
    with coefficients = the field along that line (the reference builds one
    operator per line for this)."""

    def __init__(self, op: DerivativeOperator, field):
        self.op, self.field = op, field

    def __mul__(self, Q):
        return GhostDerivativeOperator(self.op, Q, field=self.field)

    def __add__(self, other):
        return DiffEqOperatorCombination([self]) + other


def with_field(op: DerivativeOperator, field) -> FieldCoefficient:
    return FieldCoefficient(op, field)


class GhostDerivativeOperator:
    """L*Q (ghost_derivative_operator.jl:1-37)."""

    __array_ufunc__ = None  # `c * (L*Q)` with a numpy vector c goes to __rmul__

    def __init__(self, Lop: DerivativeOperator, Q, field=None):
        self.L, self.Q, self.field = Lop, Q, field

    def terms(self):
        return [self]

    def __add__(self, other):
        return DiffEqOperatorCombination([self]) + other

    def __mul__(self, u):
        return _apply_terms(self.terms(), u)

    def __call__(self, *args):
        return _ode_call(self, args, update=True)

    def update_coefficients(self, u, p, t):
        """update_coefficients!(A::GhostDerivativeOperator, u, p, t) (ghost_derivative_operator.jl:61-63)."""
        self.L.update_coefficients(u, p, t)

    def __rmul__(self, c):
        """c * (L*Q) = (c*L)*Q for a number, a vector or a function (ghost_derivative_operator.jl:66-76)."""
        out = c * self.L
        if out is NotImplemented:
            return NotImplemented
        return GhostDerivativeOperator(out, self.Q, self.field)

    def size(self):
        return (self.L.len, self.L.len)

    def ldiv(self, u, x=None):
        """A \\ u (ghost_derivative_operator.jl:39-58): x with A_l x + A_b = u, every
        line of u along the operator's axis solved with one banded LU of A_l.
        x (optional) receives the result; it may be u itself."""
        return ldiv_(x, self, u) if x is not None else ldiv(self, u)

    def array(self, N: int | None = None):
        """Array(L*Q) = (Array(L)*Q_L, Array(L)*Q_b) (concretization.jl:914-918), 1-D."""
        if not isinstance(self.Q, AtomicBC):
            raise DeoArgError(2, "Array(L*Q) is defined here for atomic BCs; use concretize() for N-D")
        A = self.L.array()
        QL, Qb = self.Q.array(self.L.len)
        return A @ QL, A @ Qb


class SolvePlan:
    """A compiled deo_solve: A = L*Q factored for (Julia size, dtype)."""

    def __init__(self, A: "GhostDerivativeOperator", shape, dtype_code: int):
        self.shape = tuple(int(n) for n in shape)
        nd = len(self.shape)
        ax = A.L.axis
        if isinstance(A.Q, AtomicBC):
            if nd > 1 and ax != 1:
                raise DeoShapeError(1, "an atomic BC on an N-D array extends dimension 1; use MultiDimBC")
            bc = A.Q
        else:
            A.Q.check_size(self.shape)
            if A.Q.line_bcs(ax) is not None:
                raise DeoArgError(2, "A \\ u is built here for one BC per axis, not an array of per-line BCs")
            bc = A.Q.bc_for(ax, nd)
        if ax > nd:
            raise DeoShapeError(1, f"operator axis {ax} but u has {nd} dimensions")
        sizes = (C.c_int64 * nd)(*self.shape)
        h = C.c_void_p()
        check(L.lib().deo_solve_plan(A.L._h, C.byref(bc._s), nd, sizes, ax, dtype_code, C.byref(h)))
        self._h = h

    def bands(self):
        kl, ku = C.c_int(), C.c_int()
        check(L.lib().deo_solve_bands(self._h, C.byref(kl), C.byref(ku)))
        return kl.value, ku.value

    def __del__(self):
        try:
            if self._h:
                L.lib().deo_solve_destroy(self._h)
                self._h = None
        except Exception:
            pass


_solve_cache: dict = {}


def solve_plan_for(A: "GhostDerivativeOperator", shape, dtype_code: int) -> SolvePlan:
    key = (id(A), tuple(shape), dtype_code)
    hit = _solve_cache.get(key)
    if hit is not None and hit[0] is A and hit[2] == A.L._version:
        return hit[1]
    p = SolvePlan(A, shape, dtype_code)
    _solve_cache[key] = (A, p, A.L._version)
    return p


def ldiv_(x, A: "GhostDerivativeOperator", u):
    """x = A \\ u on CUDA tensors in Julia layout (x may be u)."""
    if not isinstance(A, GhostDerivativeOperator):
        raise DeoArgError(2, "A \\ u is defined for a single L*Q (GhostDerivativeOperator)")
    _check_layout(u, "u")
    _check_layout(x, "x")
    if tuple(x.shape) != tuple(u.shape) or x.dtype != u.dtype or not u.is_cuda or x.device != u.device:
        raise DimensionMismatch("x must be a CUDA tensor of u's size and dtype")
    p = solve_plan_for(A, tuple(u.shape), _dtype_code(u))
    check(L.lib().deo_solve_apply(p._h, C.c_void_p(u.data_ptr()), C.c_void_p(x.data_ptr()), _stream_ptr()))
    return x


def ldiv(A: "GhostDerivativeOperator", u):
    """A \\ u (ghost_derivative_operator.jl:39-58): a new array."""
    return ldiv_(julia_array(tuple(u.shape), u.dtype, u.device), A, u)


class DiffEqOperatorCombination:
    """L1 + L2 + ... (composite_operators.jl:15-83)."""

    def __init__(self, ops: list):
        self.ops = list(ops)

    def __add__(self, other):
        if isinstance(other, DiffEqOperatorCombination):
            return DiffEqOperatorCombination(self.ops + other.ops)
        if isinstance(other, (DerivativeOperator, GhostDerivativeOperator, FieldCoefficient)):
            return DiffEqOperatorCombination(self.ops + [other])
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, (AtomicBC, MultiDimensionalBC)):
            # L*Q for a combination: sum(op -> op*Q, ops) (ghost_derivative_operator.jl:11-13)
            return DiffEqOperatorCombination([op * other for op in self.ops])
        if all(isinstance(o, GhostDerivativeOperator) for o in self.ops):
            return _apply_terms(self.ops, other)
        if self.ops and all(isinstance(o, DerivativeOperator) for o in self.ops):
            return _combination_times_padded(self.ops, other)
        raise DeoArgError(2, "apply a boundary condition first: (A*Q)*u")

    def terms(self):
        return self.ops

    def __call__(self, *args):
        return _ode_call(self, args, update=True)

    def update_coefficients(self, u, p, t):
        for op in self.ops:
            upd = getattr(op, "update_coefficients", None)
            if upd is not None:
                upd(u, p, t)


# ---------------------------------------------------------------------------
# plans and application
# ---------------------------------------------------------------------------
class Plan:
    """A compiled deo_plan for (terms, Julia size, dtype)."""

    def __init__(self, ghosts: Sequence[GhostDerivativeOperator], shape: Sequence[int], dtype_code: int,
                 path: int = L.DEO_PATH_AUTO, merge_terms: bool = False, star: bool = False,
                 factor_field: bool = False):
        nd = len(shape)
        terms = (Term * len(ghosts))()
        self._keep = []
        self.shape = tuple(int(n) for n in shape)
        self.dtype_code = dtype_code
        self.fields = []
        for i, g in enumerate(ghosts):
            ax = g.L.axis
            if isinstance(g.Q, AtomicBC):
                if nd > 1 and ax != 1:
                    raise DeoShapeError(1, "an atomic BC on an N-D array extends dimension 1 "
                                           "(multi_dim_bc_operators.jl:210); use MultiDimBC for other axes")
                bc = g.Q
            else:
                g.Q.check_size(self.shape)
                bc = g.Q.bc_for(ax, nd)
            self._keep.append(bc)
            terms[i].op = g.L._h
            terms[i].axis = ax
            terms[i].bc = C.pointer(bc._s)
            terms[i].path = path
            lines = None if isinstance(g.Q, AtomicBC) else g.Q.line_bcs(ax)
            if lines is not None:
                arr = (L.BCStruct * len(lines))(*[b._s for b in lines])
                self._keep.append(arr)
                terms[i].line_bcs = C.cast(arr, C.POINTER(L.BCStruct))
            else:
                terms[i].line_bcs = None
            if g.field is not None:
                f = g.field
                _check_layout(f, "coefficient field")
                if tuple(f.shape) != self.shape:
                    raise DeoShapeError(1, "coefficient field must have the array's size")
                self.fields.append(f)
                terms[i].coeff_field = C.c_void_p(f.data_ptr())
            else:
                terms[i].coeff_field = None
        sizes = (C.c_int64 * nd)(*self.shape)
        h = C.c_void_p()
        flags = ((L.DEO_PLAN_MERGE_TERMS if merge_terms else 0) | (L.DEO_PLAN_STAR if star else 0) |
                 (L.DEO_PLAN_FACTOR_FIELD if factor_field else 0))
        check(L.lib().deo_plan_create_opts(nd, sizes, dtype_code, len(ghosts), terms, flags, C.byref(h)))
        self._h = h
        self._ops = [g.L for g in ghosts]  # keep operators alive

    def __del__(self):
        try:
            if self._h:
                L.lib().deo_plan_destroy(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def star_taps(self) -> int:
        """Taps of the merged star (DEO_PLAN_STAR), 0 without one."""
        return int(L.lib().deo_plan_star_taps(self._h))

    @property
    def evaluated_terms(self) -> int:
        """Terms evaluated per point (after DEO_PLAN_MERGE_TERMS)."""
        return int(L.lib().deo_plan_terms(self._h))

    def table_bytes(self) -> int:
        return int(L.lib().deo_plan_table_bytes(self._h))

    def set_option(self, option: int, value):
        check(L.lib().deo_plan_set_option(self._h, int(option), int(value)))
        return self

    def get_option(self, option: int) -> int:
        """1 / 0 whether a switch is on and applies to this plan; the row count
        for DEO_OPT_FX_FP64_ROWS (0 when the fixed-point kernel does not apply)."""
        v = L.lib().deo_plan_get_option(self._h, int(option))
        if v < 0:
            raise DeoArgError(2, f"unknown plan option {option}")
        return v

    def set_fast_path(self, enable: bool):
        return self.set_option(L.DEO_OPT_FAST_PATH, enable)

    @property
    def uses_fast_path(self) -> bool:
        return self.get_option(L.DEO_OPT_FAST_PATH) == 1

    @property
    def uses_exact_sums(self) -> bool:
        return self.get_option(L.DEO_OPT_EXACT_SUMS) == 1

    @property
    def kernels(self) -> tuple:
        """Names of the kernels the last forward apply launched."""
        lib = L.lib()
        return tuple(k.decode() for k in (lib.deo_plan_kernels(self._h, 0), lib.deo_plan_kernels(self._h, 1)) if k)

    def autotune(self, u, du, cache_path: str | None = None) -> dict:
        """deo_plan_autotune: time the bit-identical execution choices of a
        Laplacian-type TMA plan on u -> du (du is overwritten) and keep the
        fastest; returns the chosen options."""
        self._check(u, du)
        check(L.lib().deo_plan_autotune(self._h, C.c_void_p(u.data_ptr()), C.c_void_p(du.data_ptr()),
                                        cache_path.encode() if cache_path else None, _stream_ptr()))
        return {"f32_vector": self.get_option(L.DEO_OPT_F32_VECTOR), "f32_tile": self.get_option(L.DEO_OPT_F32_TILE),
                "shell_kernel": self.get_option(L.DEO_OPT_SHELL_KERNEL),
                "concurrent_shell": self.get_option(L.DEO_OPT_CONCURRENT_SHELL)}

    def autotune_times(self) -> list:
        """[((f32_vector, f32_tile, shell_kernel, concurrent_shell), us per apply), ...] of the last
        autotune (empty when it came from the cache)."""
        n = C.c_int()
        check(L.lib().deo_plan_autotune_times(self._h, None, None, 0, C.byref(n)))
        cands = (C.c_int * (4 * n.value))()
        ms = (C.c_float * n.value)()
        check(L.lib().deo_plan_autotune_times(self._h, cands, ms, n.value, C.byref(n)))
        return [(tuple(cands[4 * i:4 * i + 4]), round(ms[i] * 1e3, 2)) for i in range(n.value)]

    def launch_times(self) -> list:
        """Device ms of each launch of the last forward apply (needs
        set_option(DEO_OPT_LAUNCH_TIMING, 1) before that apply)."""
        ms = (C.c_float * 2)()
        n = C.c_int()
        check(L.lib().deo_plan_launch_times(self._h, ms, C.byref(n)))
        return [float(ms[i]) for i in range(n.value)]

    def _check(self, u, du):
        if tuple(u.shape) != self.shape or tuple(du.shape) != self.shape:
            raise DeoShapeError(1, f"plan is for size {self.shape}; got {tuple(u.shape)} -> {tuple(du.shape)}")
        _check_layout(u, "u")
        _check_layout(du, "du")
        if _dtype_code(u) != self.dtype_code or _dtype_code(du) != self.dtype_code:
            raise DeoArgError(2, "dtype does not match the plan")
        if not (u.is_cuda and du.is_cuda):
            raise DeoArgError(2, "device tensors required (use apply_host for host arrays)")
        if u.device != du.device:
            raise DeoArgError(2, "u and du must be on one device")

    def apply(self, u, du, overwrite: bool = True):
        self._check(u, du)
        check(L.lib().deo_apply(self._h, C.c_void_p(u.data_ptr()), C.c_void_p(du.data_ptr()), int(bool(overwrite)),
                                _stream_ptr()))
        return du

    def adjoint(self, dbar, ubar, overwrite: bool = True):
        self._check(dbar, ubar)
        check(L.lib().deo_apply_adjoint(self._h, C.c_void_p(dbar.data_ptr()), C.c_void_p(ubar.data_ptr()),
                                        int(bool(overwrite)), _stream_ptr()))
        return ubar

    def apply_host(self, u: np.ndarray, du: np.ndarray, stream=None):
        assert u.flags.f_contiguous and du.flags.f_contiguous
        check(L.lib().deo_apply_host(self._h, C.c_void_p(u.ctypes.data), C.c_void_p(du.ctypes.data),
                                     stream if stream is not None else _stream_ptr()))
        return du

    def apply_host_async(self, u, du, stream=None):
        """Pipelined host apply (deo_apply_host_async): u, du are host buffers
        (numpy Fortran arrays or pinned CPU tensors, in the plan's layout) that
        must stay alive, and du unread, until host_sync()."""
        up = u.ctypes.data if isinstance(u, np.ndarray) else u.data_ptr()
        dp = du.ctypes.data if isinstance(du, np.ndarray) else du.data_ptr()
        check(L.lib().deo_apply_host_async(self._h, C.c_void_p(up), C.c_void_p(dp),
                                           stream if stream is not None else _stream_ptr()))
        return du

    def host_sync(self):
        check(L.lib().deo_plan_host_sync(self._h))

    def concretize(self):
        """(A_l, A_b) of du = A_l u + A_b, dense, built on the device from the plan's tables."""
        n = int(np.prod(self.shape))
        Al = np.zeros((n, n), order="F")
        Ab = np.zeros(n)
        check(L.lib().deo_plan_concretize(self._h, Al.ctypes.data_as(_dp), _ptr(Ab)))
        return Al, Ab

    def bandwidths(self) -> tuple:
        lo, up = C.c_int64(), C.c_int64()
        check(L.lib().deo_plan_bandwidths(self._h, C.byref(lo), C.byref(up), _stream_ptr()))
        return lo.value, up.value

    def concretize_banded(self):
        """BandedMatrix(L*Q) on the device: (l, u, data, A_b) with data the (l+u+1) x n band storage
        (entry (i, j) at row u+i-j of column j) and A_b, both device tensors."""
        torch = _torch()
        lo, up = self.bandwidths()
        n = int(np.prod(self.shape))
        data = torch.empty((n, lo + up + 1), dtype=torch.float64, device="cuda").t()  # column-major
        ab = torch.empty(n, dtype=torch.float64, device="cuda")
        check(L.lib().deo_plan_concretize_banded(self._h, lo, up, C.c_void_p(data.data_ptr()),
                                                 C.c_void_p(ab.data_ptr()), _stream_ptr()))
        return lo, up, data, ab


_plan_cache: dict = {}


def plan_for(ghosts, shape, dtype_code, path=L.DEO_PATH_AUTO, merge_terms: bool = False,
             factor_field: bool = False) -> Plan:
    key = (tuple(id(g) for g in ghosts), tuple(shape), dtype_code, path,
           tuple(g.field.data_ptr() if g.field is not None else 0 for g in ghosts), merge_terms, factor_field)
    versions = tuple(g.L._version for g in ghosts)
    p = _plan_cache.get(key)
    if p is None or p._versions != versions:  # a plan of earlier coefficient values is replaced
        p = Plan(ghosts, shape, dtype_code, path, merge_terms, factor_field=factor_field)
        p._versions = versions
        # keep the ghosts alive with the plan so ids stay unique
        p._ghosts = list(ghosts)
        _plan_cache[key] = p
    return p


def clear_plan_cache():
    _plan_cache.clear()


def _apply_terms(ghosts, u, du=None, overwrite=True):
    if isinstance(u, np.ndarray):
        uf = np.asfortranarray(u, dtype=np.float64 if u.dtype != np.float32 else np.float32)
        code = L.DEO_F64 if uf.dtype == np.float64 else L.DEO_F32
        p = plan_for(ghosts, uf.shape, code)
        out = np.zeros(uf.shape, dtype=uf.dtype, order="F") if du is None else du
        if not overwrite:
            raise DeoArgError(2, "host arrays support overwrite=True only")
        return p.apply_host(uf, out)
    p = plan_for(ghosts, tuple(u.shape), _dtype_code(u))
    if du is None:
        du = julia_array(tuple(u.shape), u.dtype, u.device)
    return p.apply(u, du, overwrite)


def mul_(du, A, u, overwrite: bool = True):
    """mul!(du, A, u) for A = L*Q or a combination of L*Q terms
    (ghost_derivative_operator.jl:15-24, composite_operators.jl:76-83), or for
    a DerivativeOperator on an already padded array
    (derivative_operator_functions.jl:17-25)."""
    if isinstance(A, DerivativeOperator):
        return _mul_padded(A, u, du, overwrite)
    if isinstance(A, DiffEqOperatorCombination) and A.ops and all(isinstance(o, DerivativeOperator) for o in A.ops):
        return _combination_mul_padded(du, A.ops, u)
    return _apply_terms(A.terms(), u, du, overwrite)


class PaddedPlan:
    """A compiled deo_padded: L on an already padded array for (sizes, dtype)."""

    def __init__(self, op: DerivativeOperator, out_shape, in_shape, dtype_code: int, starts=None):
        nd = len(in_shape)
        osz = (C.c_int64 * nd)(*out_shape)
        isz = (C.c_int64 * nd)(*in_shape)
        h = C.c_void_p()
        if starts is None:
            check(L.lib().deo_padded_plan(op._h, int(op.axis), nd, osz, isz, int(dtype_code), C.byref(h)))
        else:
            st = (C.c_int64 * nd)(*starts)
            check(L.lib().deo_padded_plan_view(op._h, int(op.axis), nd, osz, isz, st, int(dtype_code), C.byref(h)))
        self._h = h

    def __del__(self):
        try:
            if self._h:
                L.lib().deo_padded_destroy(self._h)
                self._h = None
        except Exception:
            pass


_padded_cache: dict = {}


def _mul_padded(op: DerivativeOperator, M, out=None, overwrite: bool = True):
    """L*M and mul!(x_temp, L, M; overwrite) for an already padded array M
    (derivative_operator_functions.jl:17-69, 150-163; convolutions.jl:17-22 for
    vectors): M is padded along the operator's axis; along other axes it has
    x_temp's size or 2 more (then its edge planes are skipped)."""
    if isinstance(M, np.ndarray) or not getattr(M, "is_cuda", False):
        raise DeoArgError(2, "L*M takes a CUDA tensor (Julia layout)")
    _check_layout(M, "M")
    nd = M.dim()
    if op.axis > nd:
        raise DeoShapeError(1, f"the operator acts on axis {op.axis} but M has {nd} dimensions")
    if out is None:
        oshape = tuple(n - 2 if b == op.axis - 1 else n for b, n in enumerate(M.shape))
        if min(oshape) < 1:
            raise DeoShapeError(1, f"M of size {tuple(M.shape)} is too small")
        out = julia_array(oshape, M.dtype, M.device)
        overwrite = True
    else:
        _check_layout(out, "x_temp")
        if getattr(out, "device", None) != M.device:
            raise DeoArgError(2, "x_temp must be a CUDA tensor on M's device")
        if out.dim() != nd or out.dtype != M.dtype:
            raise DeoShapeError(1, "x_temp must have M's number of dimensions and dtype")
    key = (id(op), tuple(out.shape), tuple(M.shape), _dtype_code(M))
    hit = _padded_cache.get(key)
    if hit is None or hit[0] is not op or hit[2] != op._version:
        hit = _padded_cache[key] = (op, PaddedPlan(op, tuple(out.shape), tuple(M.shape), _dtype_code(M)),
                                    op._version)
    check(L.lib().deo_padded_apply(hit[1]._h, C.c_void_p(M.data_ptr()), C.c_void_p(out.data_ptr()),
                                   1 if overwrite else 0, _stream_ptr()))
    return out


def _padded_view_apply(op: DerivativeOperator, M, out, starts, overwrite: bool):
    """mul!(out, op, view(M, ...)) with the view beginning at the 0-based
    `starts` (0 along op's axis) and out's size along the other axes."""
    key = ("view", id(op), tuple(out.shape), tuple(M.shape), tuple(starts), _dtype_code(M))
    hit = _padded_cache.get(key)
    if hit is None or hit[0] is not op or hit[2] != op._version:
        hit = _padded_cache[key] = (op, PaddedPlan(op, tuple(out.shape), tuple(M.shape), _dtype_code(M), starts),
                                    op._version)
    check(L.lib().deo_padded_apply(hit[1]._h, C.c_void_p(M.data_ptr()), C.c_void_p(out.data_ptr()),
                                   1 if overwrite else 0, _stream_ptr()))
    return out


def _combination_times_padded(ops, M):
    """(L1 + L2 + ...) * M = sum(op -> op * M, ops) (composite_operators.jl:64-65)
    for DerivativeOperators on an already padded M: the first product written,
    the others added in order (every product must have the first one's size)."""
    out = _mul_padded(ops[0], M)
    for op in ops[1:]:
        oshape = tuple(n - 2 if b == op.axis - 1 else n for b, n in enumerate(M.shape))
        if oshape != tuple(out.shape):
            raise DimensionMismatch(f"dimensions must match: a has dims {tuple(out.shape)}, b has dims {oshape}")
        _mul_padded(op, M, out, overwrite=False)
    return out


def _combination_mul_padded(x_temp, ops, M):
    """mul!(x_temp, L1 + L2 + ..., M) for DerivativeOperators on an already
    padded M.  Vectors: the first operator written, the others added through a
    cache (composite_operators.jl:76-83).  2-D and 3-D arrays: the reference's
    composite method (derivative_operator_functions.jl:203-463, 466-802) with
    its fallback branch, the one publicly constructed operators reach (their
    coefficients are Vectors): each operator reads view(M, 1:x_temp_1, ...,
    1:(x_temp_k + 2), ...) -- starting at index 1 along the other axes even
    where M is padded there -- except, in 2-D, along an axis no operator of
    the sum acts on, where it reads M whole (and _mul! strips M's edge planes
    if it is padded there).  The first operator overwrites, the others add."""
    if x_temp is None:
        raise DeoArgError(2, "mul!(x_temp, A, M) needs x_temp")
    if not getattr(M, "is_cuda", False) or getattr(x_temp, "device", None) != M.device:
        raise DeoArgError(2, "M and x_temp must be CUDA tensors on one device")
    _check_layout(M, "M")
    _check_layout(x_temp, "x_temp")
    nd = M.dim()
    if x_temp.dim() != nd or x_temp.dtype != M.dtype:
        raise DeoShapeError(1, "x_temp must have M's number of dimensions and dtype")
    if nd == 1:
        for k, op in enumerate(ops):
            _mul_padded(op, M, x_temp, overwrite=(k == 0))
        return x_temp
    if nd not in (2, 3):
        raise DeoArgError(2, f"no mul! method for a sum of operators on a {nd}-D array (2-D and 3-D only)")
    operated = {op.axis for op in ops}
    for k, op in enumerate(ops):
        if op.axis > nd:
            raise DeoShapeError(1, f"the operator acts on axis {op.axis} but M has {nd} dimensions")
        others = [b for b in range(1, nd + 1) if b != op.axis]
        if nd == 2 and not (set(others) & operated):
            _mul_padded(op, M, x_temp, overwrite=(k == 0))
            continue
        _padded_view_apply(op, M, x_temp, [0] * nd, overwrite=(k == 0))
    return x_temp


def concretize(A, shape, dtype=np.float64):
    """(A_l, A_b) of u -> A*u on the device by unit-vector probes (checking only)."""
    ghosts = A.terms()
    p = Plan(ghosts, shape, L.DEO_F64)
    return p.concretize()
