"""libdeo host side on the CPU: the library loads, exports every symbol of
include/deo.h, and its constructors give the oracle's tables bit for bit
(no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

import deo
import oracle as O
from deo import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "deo.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(deo_[a-z0-9_]+)\s*\(", src)))


def test_header_constants_match_the_binding():
    """Every DEO_PLAN_* and DEO_OPT_* value the header defines is the one the
    Python binding passes."""
    src = open(os.path.join(ROOT, "include", "deo.h")).read()
    defs = dict(re.findall(r"#define\s+(DEO_(?:PLAN|OPT)_[A-Z0-9_]+)\s+(-?\d+)", src))
    assert "DEO_PLAN_FACTOR_FIELD" in defs and "DEO_OPT_F32_VECTOR" in defs
    for name, value in defs.items():
        assert hasattr(_lib, name), name
        assert getattr(_lib, name) == int(value), name


def test_header_symbols_exported():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.EXPORTED) | {n for n in names if n not in _lib.EXPORTED and hasattr(lib, n)}


def test_abi_version():
    assert deo.lib().deo_abi_version() == 2


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), np.abs(a - b).max()


CENTRED = [(d, a) for d in (1, 2, 3, 4) for a in (2, 3, 4, 6, 8)]


@pytest.mark.parametrize("d,a", CENTRED)
@pytest.mark.parametrize("grid", ["uniform", "nonuniform"])
def test_centred_tables_bitwise(d, a, grid):
    n = 40
    dx = 1.0 / 41 if grid == "uniform" else np.random.default_rng(d * 10 + a).uniform(0.5, 1.5, n + 1) / n
    P = deo.CenteredDifference(d, a, dx, n)
    Q = O.centered(d, a, dx, n)
    st, lo, hi, co = Q.tables()
    _same(P.stencil_coefs, st)
    _same(P.low_boundary_coefs, lo)
    _same(P.high_boundary_coefs, hi)
    _same(P.coefficients, co)
    _same(P.array(), Q.array())


UPWIND = [(d, a, off) for d in (1, 2, 3) for a in (1, 2, 3, 4) for off in (0, 1, 2) if off <= (d + a - 1) // 2]


@pytest.mark.parametrize("d,a,off", UPWIND)
@pytest.mark.parametrize("grid", ["uniform", "nonuniform"])
def test_upwind_tables_bitwise(d, a, off, grid):
    n = 30
    dx = 0.1 if grid == "uniform" else np.random.default_rng(d + 7 * a + off).uniform(0.5, 1.5, n + 1) / n
    c = np.random.default_rng(11).uniform(-1, 1, n)
    P = deo.UpwindDifference(d, a, dx, n, c, offside=off)
    Q = O.upwind(d, a, dx, n, c, offside=off)
    st, lo, hi, co = Q.tables()
    _same(P.stencil_coefs, st)
    _same(P.low_boundary_coefs, lo)
    _same(P.high_boundary_coefs, hi)
    _same(P.coefficients, co)
    _same(P.array(), Q.array())


@pytest.mark.parametrize("kind", ["centered", "upwind"])
def test_longer_dx_as_the_reference_reads_it(kind):
    # The reference takes a dx longer than len+1: its upwind constructor reads
    # x = [0; cumsum(dx)] at x[1:len+2] only, its centred constructor reads
    # dx[1:len+1] for the interior and the last d+a entries for the high
    # boundary rows (derivative_operator.jl:150-170, 515-639); the
    # coefficient tests build UpwindDifference(1, 1, dxv, 3, ...) with five
    # entries (coefficient_functions.jl:57-67).
    rng = np.random.default_rng(5)
    for d, a, off in ((1, 1, 0), (1, 2, 1), (2, 2, 0), (2, 3, 2)):
        if kind == "centered":
            a = max(a, 2)
        n = 12
        dx = rng.uniform(0.5, 1.5, n + 4) / n
        P = (deo.CenteredDifference(d, a, dx, n) if kind == "centered"
             else deo.UpwindDifference(d, a, dx, n, offside=off))
        Q = O.centered(d, a, dx, n) if kind == "centered" else O.upwind(d, a, dx, n, offside=off)
        st, lo, hi, co = Q.tables()
        _same(P.stencil_coefs, st)
        _same(P.low_boundary_coefs, lo)
        _same(P.high_boundary_coefs, hi)
        _same(P.array(), Q.array())
        if kind == "upwind":  # only dx[1:len+1] matters
            _same(P.array(), deo.UpwindDifference(d, a, dx[:n + 1], n, offside=off).array())


@pytest.mark.parametrize("d,a,off,n,ndx", [
    (2, 4, 0, 3, 4),     # centred: the high boundary needs the last d+a = 6 spacings
    (1, 4, 0, 4, 4),     # too few spacings for len+1
    (1, 4, 2, 2, 3),     # upwind, offside 2: the high downwind rows leave the grid
    (1, 4, 2, 3, 4),
])
def test_grids_too_short_for_the_stencil_are_rejected(d, a, off, n, ndx):
    # where the reference indexes outside x or dx (BoundsError), both the
    # library and the oracle refuse the operator instead of reading past dx
    dx = np.full(ndx, 0.1)
    kind = "centered" if (d, a, off, n) in ((2, 4, 0, 3), (1, 4, 0, 4)) else "upwind"
    with pytest.raises(deo.DeoShapeError):
        if kind == "centered":
            deo.CenteredDifference(d, a, dx, n)
        else:
            deo.UpwindDifference(d, a, dx, n, offside=off)
    with pytest.raises(AssertionError):
        O.centered(d, a, dx, n) if kind == "centered" else O.upwind(d, a, dx, n, offside=off)


def test_bcs_bitwise():
    rng = np.random.default_rng(2)
    for order in (1, 2, 3):
        l, r = rng.random(3), rng.random(3)
        for dx in (0.37, rng.uniform(0.5, 1.5, 12)):
            a = deo.RobinBC(l, r, dx, order)
            b = O.robin(l, r, dx, order)
            _same(a.a_l, b.a_l); _same(a.a_r, b.a_r)
            assert a.b_l == b.bl and a.b_r == b.br
            al, ar = rng.random(3 + order % 2), rng.random(3)
            g, h = deo.GeneralBC(al, ar, dx, order), O.general(al, ar, dx, order)
            _same(g.a_l, h.a_l); _same(g.a_r, h.a_r)
            assert g.b_l == h.bl and g.b_r == h.br
    d = deo.Dirichlet0BC()
    assert list(d.a_l) == [0.0, 0.0] and d.b_l == 0.0
    QL, Qb = deo.RobinBC(l, r, 0.3, 2).array(7)
    QL2, Qb2 = O.robin(l, r, 0.3, 2).array(7)
    _same(QL, QL2); _same(Qb, Qb2)


def test_weights_and_errors():
    _same(deo.calculate_weights(2, 0.0, [-2, -1, 0, 1, 2]), O.calculate_weights(2, 0.0, [-2, -1, 0, 1, 2]))
    with pytest.raises(AssertionError):
        deo.calculate_weights(3, 0.0, [0, 1, 2])
    with pytest.raises(AssertionError):
        deo.CenteredDifference(2, 1, 1.0, 10)
    with pytest.raises(AssertionError):
        deo.UpwindDifference(1, 1, 1.0, 10, offside=3)
    L = deo.CenteredDifference(2, 2, 1.0, 3)
    with pytest.raises(AssertionError):   # DimensionMismatch (derivative_operator_functions.jl:182-184)
        np.ones(10) * L


def test_coefficient_scaling_matches_reference_rules():
    # derivative_operators_interface.jl:418-438
    A = deo.CenteredDifference(2, 2, 1.0, 3)
    C = deo.UpwindDifference(1, 1, 1.0, 3, np.array([2.0, 3.0, 4.0]))
    c = np.array([1.0, 1.0, 3.0])
    assert list((c * A).coefficients) == list(c)
    assert list((c * C).coefficients) == [2.0, 3.0, 12.0]


def test_operator_from_tables_roundtrip():
    P = deo.UpwindDifference(2, 3, np.random.default_rng(0).uniform(0.5, 1, 21) / 20, 20, -1.0, offside=1)
    desc = dict(derivative_order=P.derivative_order, approximation_order=P.approximation_order, len=P.len,
                stencil_length=P.stencil_length, boundary_stencil_length=P.boundary_stencil_length,
                boundary_point_count=P.boundary_point_count, offside=P.offside, winding=1, uniform=0,
                coeff_func_sign=P.coeff_func_sign, n_stencil_rows=P.stencil_coefs.shape[1],
                n_low_rows=P.low_boundary_coefs.shape[1], n_high_rows=P.high_boundary_coefs.shape[1],
                stencil_coefs=P.stencil_coefs, low_boundary_coefs=P.low_boundary_coefs,
                high_boundary_coefs=P.high_boundary_coefs, coefficients=P.coefficients)
    R = deo.operator_from_tables(desc)
    _same(R.array(), P.array())


def test_fast_division_constants():
    # the kernels derive row indices with (umulhi(n, mul) + n) >> shr for 31-bit n
    lib = ctypes.CDLL(_lib.LIB_PATH)
    lib.deo_fastdiv_probe.restype = ctypes.c_int
    lib.deo_fastdiv_probe.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    rng = np.random.default_rng(0)
    ds = [1, 2, 3, 5, 7, 256, 257, 1023, 1025, 65535, 65537, (1 << 20) + 1, 1 << 30, (1 << 31) - 1]
    ds += [int(d) for d in rng.integers(1, 1 << 31, 300)]
    for d in ds:
        ns = [0, 1, d - 1, d, d + 1, 2 * d - 1, (1 << 31) - 1] + [int(n) for n in rng.integers(0, 1 << 31, 64)]
        for n in ns:
            if 0 <= n < (1 << 31):
                assert lib.deo_fastdiv_probe(n, d) == n // d, (n, d)


def _from_band(data, lo, up, n):
    M = np.zeros((n, n + 2))
    for j in range(n + 2):
        for b in range(lo + up + 1):
            i = b - up + j
            if 0 <= i < n:
                M[i, j] = data[b, j]
    return M


@pytest.mark.parametrize("kind,d,a", [("c", d, a) for d in (1, 2, 3, 4) for a in (2, 4, 6)] +
                         [("u", d, a) for d in (1, 2, 3) for a in (1, 2, 3)])
@pytest.mark.parametrize("grid", ["uniform", "nonuniform"])
def test_banded_matrix_export(kind, d, a, grid):
    """BandedMatrix(L): the reference's bandwidths ((bstl-3, bstl-1) centred,
    concretization.jl:126; (stl-2, stl) upwind, :802) and the entries of
    Array(L) in band storage, bit for bit the oracle's Array(L)."""
    n = 32
    dx = 1.0 / 33 if grid == "uniform" else np.random.default_rng(d * 7 + a).uniform(0.5, 1.5, n + 1) / n
    if kind == "c":
        P, Q = deo.CenteredDifference(d, a, dx, n), O.centered(d, a, dx, n)
        want = (P.boundary_stencil_length - 3, P.boundary_stencil_length - 1)
    else:
        c = np.random.default_rng(3).uniform(-1, 1, n)
        P, Q = deo.UpwindDifference(d, a, dx, n, c), O.upwind(d, a, dx, n, c)
        want = (P.stencil_length - 2, P.stencil_length)
    data, (lo, up) = P.banded()
    assert (lo, up) == want
    assert data.shape == (lo + up + 1, n + 2)
    _same(_from_band(data, lo, up, n), Q.array())


def test_padded_view_plan_rejects_bad_views():
    # deo_padded_plan_view validates the view before it touches the device:
    # starts[axis-1] must be 0 with len+2 entries there, and the block must fit in M
    import ctypes as C
    lib = deo.lib()
    L = deo.CenteredDifference(2, 2, 1.0, 10, axis=1)
    h = C.c_void_p()
    I64 = C.c_int64 * 2

    def plan(out, inn, starts):
        return lib.deo_padded_plan_view(L._h, 1, 2, I64(*out), I64(*inn), None if starts is None else I64(*starts),
                                        0, C.byref(h))
    assert plan((10, 8), (12, 10), None) == 2                         # null starts: DEO_ERR_BAD_ARG
    assert plan((10, 8), (12, 10), (1, 0)) == 1                       # the differentiated axis starts at 0
    assert b"differentiated" in lib.deo_last_error()
    assert plan((10, 8), (11, 10), (0, 0)) == 1                       # len + 2 entries along it
    assert plan((10, 8), (12, 10), (0, 3)) == 1                       # 3 + 8 > 10 along axis 2
    assert plan((10, 8), (12, 10), (0, -1)) == 1
    assert not h.value
