"""mul!(x_temp, L1 + L2 + ..., M) and (L1 + L2 + ...) * M for DerivativeOperators
on an already padded M (test/DerivativeOperators/2D_3D_fast_multiplication.jl).

The reference's 2-D / 3-D method (derivative_operator_functions.jl:203-802)
takes its fallback branch for every publicly constructed operator (their
coefficients are Vectors, not Numbers): operator k reads
view(M, 1:x_temp_1, ..., 1:(x_temp_k + 2), ...), which begins at index 1 on
the other axes even where M is padded there.  The reference's own tests use
separable fields, on which that makes no difference; the CPU tests below check
the oracle's restatement against those identities and show on a non-separable
field that the restatement keeps the index-1 views.  The GPU tests compare the
library with the oracle at the 4-ulp-of-sum|c_k u_k| bar.
"""
import zlib

import numpy as np
import pytest

import oracle as O

RTOL = np.sqrt(np.finfo(float).eps)


def _approx(x, y):
    return np.linalg.norm(np.ravel(x) - np.ravel(y)) <= RTOL * max(np.linalg.norm(np.ravel(x)),
                                                                    np.linalg.norm(np.ravel(y)))


def _field2(N, dx, dy):
    i = np.arange(1, N + 3)[:, None]
    j = np.arange(1, N + 3)[None, :]
    return np.asfortranarray(np.cos(dx * i) + np.sin(dy * j))


def _field3(N):
    i = np.arange(1, N + 3)[:, None, None]
    j = np.arange(1, N + 3)[None, :, None]
    k = np.arange(1, N + 3)[None, None, :]
    return np.asfortranarray(np.cos(0.1 * i) + np.sin(0.1 * j) + np.exp(0.01 * k))


def _op(d, a, h, N, axis, scale=None):
    L = O.centered(d, a, h, N, axis=axis)
    if scale is not None:
        L.scale(scale)
    return L


def _comb(ops, M, shape):
    return O.mul_combination(ops, M, np.zeros(shape, order="F"))


# 2-D testsets of 2D_3D_fast_multiplication.jl: (d, a) of the x and y operators, dx, dy, scales
CASES_2D = [
    ("no boundary points, dx = 1", [(2, 2)], 1.0, 1.0, None),                    # :5-52
    ("identical bpc, dx = 1", [(4, 4)], 1.0, 1.0, None),                          # :54-107
    ("differing bpc, dx = 1", [(2, 2), (3, 3), (4, 4)], 1.0, 1.0, None),          # :109-162
    ("identical bpc, dx = dy = 0.1", [(4, 4)], 0.1, 0.1, None),                   # :164-217
    ("differing bpc, dx = 0.1, dy = 0.25", [(2, 2), (3, 3), (4, 4)], 0.1, 0.25, None),  # :333-389
    ("coefficients", [(2, 2), (3, 3), (4, 4)], 0.1, 0.25, ((5.5, 1.45, 0.5), (8.14, 2.0, 4.567))),  # :394-451
]


@pytest.mark.parametrize("name,orders,dx,dy,scales", CASES_2D, ids=[c[0] for c in CASES_2D])
def test_oracle_2d_reference_identities(name, orders, dx, dy, scales):
    N = 100
    M = _field2(N, dx, dy)
    xs = [_op(d, a, dx, N, 1, scales[0][k] if scales else None) for k, (d, a) in enumerate(orders)]
    ys = [_op(d, a, dy, N, 2, scales[1][k] if scales else None) for k, (d, a) in enumerate(orders)]
    # a single axis, several operators: x_temp keeps the other axis padded
    assert _approx(_comb(xs, M, (N, N + 2)), sum(O.mul_nd(L, M) for L in xs))
    assert _approx(_comb(ys, M, (N + 2, N)), sum(O.mul_nd(L, M) for L in ys))
    # both axes: (Lx*M)[1:N, 2:N+1] + (Ly*M)[2:N+1, 1:N] summed in the sum's order
    both = [L for pair in zip(xs, ys) for L in pair]
    expect = sum(O.mul_nd(L, M)[:, 1:N + 1] if L.axis == 1 else O.mul_nd(L, M)[1:N + 1, :] for L in both)
    assert _approx(_comb(both, M, (N, N)), expect)


def test_oracle_3d_reference_identities():
    # 2D_3D_fast_multiplication.jl:644-730 (N = 100 there; the identities hold for any N)
    N = 30
    M = _field3(N)
    Lxx, Lyy, Lzz = (_op(2, 2, 1.0, N, k) for k in (1, 2, 3))
    Lx, Ly, Lz = (_op(1, 2, 1.0, N, k) for k in (1, 2, 3))
    got = _comb([Lxx, Lyy, Lzz], M, (N, N, N))
    expect = (O.mul_nd(Lxx, M)[:, 1:N + 1, 1:N + 1] + O.mul_nd(Lyy, M)[1:N + 1, :, 1:N + 1] +
              O.mul_nd(Lzz, M)[1:N + 1, 1:N + 1, :])
    assert _approx(got, expect)
    assert _approx(_comb([Lx, Lxx], M, (N, N + 2, N + 2)), O.mul_nd(Lx, M) + O.mul_nd(Lxx, M))
    assert _approx(_comb([Ly, Lyy], M, (N + 2, N, N + 2)), O.mul_nd(Ly, M) + O.mul_nd(Lyy, M))
    assert _approx(_comb([Lz, Lzz], M, (N + 2, N + 2, N)), O.mul_nd(Lz, M) + O.mul_nd(Lzz, M))
    got = _comb([Lx, Ly, Lxx, Lyy], M, (N, N, N + 2))
    expect = (O.mul_nd(Lx, M)[:, 1:N + 1, :] + O.mul_nd(Ly, M)[1:N + 1, :, :] +
              O.mul_nd(Lxx, M)[:, 1:N + 1, :] + O.mul_nd(Lyy, M)[1:N + 1, :, :])
    assert _approx(got, expect)


def test_oracle_keeps_the_index_one_views():
    # On a field that is not separable the reference's views (index 1 on the
    # other axes) and the centred slices of its own tests differ.
    N = 24
    rng = np.random.default_rng(5)
    M = np.asfortranarray(rng.standard_normal((N + 2, N + 2)))
    Lxx, Lyy = _op(2, 2, 1.0, N, 1), _op(2, 2, 1.0, N, 2)
    got = _comb([Lxx, Lyy], M, (N, N))
    views = O.mul_nd(Lxx, np.asfortranarray(M[:, :N]), out_shape=(N, N)) + \
        O.mul_nd(Lyy, np.asfortranarray(M[:N, :]), out_shape=(N, N))
    np.testing.assert_array_equal(got, views)
    centred = O.mul_nd(Lxx, M)[:, 1:N + 1] + O.mul_nd(Lyy, M)[1:N + 1, :]
    assert not np.allclose(got, centred)


def test_oracle_vector_combination():
    # composite_operators.jl:76-83: y = ops[1]*b, then y .+= op*b
    rng = np.random.default_rng(6)
    b = rng.standard_normal(42)
    L1, L2 = O.centered(2, 4, 0.1, 40), O.upwind(1, 2, 0.1, 40, rng.uniform(-1, 1, 40))
    y = O.mul_combination([L1, L2], b, np.zeros(40))
    np.testing.assert_array_equal(y, L1.mul_generic(b) + L2.mul_generic(b))


# ---- the library on the GPU against the oracle ---------------------------------------
def _gpu_cases():
    rng = np.random.default_rng(11)
    irr = lambda n: np.cumsum(rng.random(n + 2)) * 0.01  # dx = cumsum(rand(N + 2)) (:453-498)
    cases = []
    N = 60
    cases.append(("2d xx+yy", (N, N), (N + 2, N + 2), [("c", 2, 2, 1.0, 1, None), ("c", 2, 2, 1.0, 2, None)]))
    cases.append(("2d x+xx", (N, N + 2), (N + 2, N + 2), [("c", 1, 2, 0.1, 1, None), ("c", 2, 2, 0.1, 1, None)]))
    cases.append(("2d y+yy", (N + 2, N), (N + 2, N + 2), [("c", 1, 2, 0.1, 2, None), ("c", 2, 2, 0.1, 2, None)]))
    cases.append(("2d mixed bpc scaled", (N, N), (N + 2, N + 2),
                  [("c", 2, 2, 0.1, 1, 5.5), ("c", 2, 2, 0.25, 2, 8.14), ("c", 3, 3, 0.1, 1, 1.45),
                   ("c", 3, 3, 0.25, 2, 2.0), ("c", 4, 4, 0.1, 1, 0.5), ("c", 4, 4, 0.25, 2, 4.567)]))
    cases.append(("2d irregular both", (N, N), (N + 2, N + 2),
                  [("c", 2, 4, irr(N), 1, None), ("c", 1, 4, irr(N), 2, None), ("c", 4, 4, irr(N), 2, None)]))
    cases.append(("2d upwind + centred, coefficient vectors", (N, N), (N + 2, N + 2),
                  [("u", 1, 2, 0.1, 1, rng.uniform(-1, 1, N)), ("c", 2, 4, 0.1, 2, rng.uniform(0.5, 1.5, N))]))
    n = 20
    cases.append(("3d xx+yy+zz", (n, n, n), (n + 2, n + 2, n + 2),
                  [("c", 2, 2, 1.0, 1, None), ("c", 2, 2, 1.0, 2, None), ("c", 2, 2, 1.0, 3, None)]))
    cases.append(("3d x+xx", (n, n + 2, n + 2), (n + 2, n + 2, n + 2),
                  [("c", 1, 2, 1.0, 1, None), ("c", 2, 2, 1.0, 1, None)]))
    cases.append(("3d x+y+xx+yy", (n, n, n + 2), (n + 2, n + 2, n + 2),
                  [("c", 1, 2, 0.5, 1, None), ("c", 1, 2, 0.25, 2, None), ("c", 2, 4, 0.5, 1, None),
                   ("c", 2, 4, 0.25, 2, None)]))
    cases.append(("3d irregular, differing bpc", (n, n, n), (n + 2, n + 2, n + 2),
                  [("c", 2, 2, irr(n), 1, None), ("c", 3, 4, 0.25, 2, 2.0), ("c", 4, 4, irr(n), 3, None)]))
    cases.append(("1d", (40,), (42,), [("c", 2, 4, 0.1, 1, None), ("u", 1, 2, 0.1, 1, rng.uniform(-1, 1, 40))]))
    return cases


GPU_CASES = _gpu_cases()


def _pair(spec, out_shape):
    import deo
    kind, d, a, h, axis, coeff = spec
    n = out_shape[axis - 1]
    if kind == "c":
        P = deo.CenteredDifference(d, a, h, n, axis=axis)
        Q = O.centered(d, a, h, n, axis=axis)
    else:
        P = deo.UpwindDifference(d, a, h, n, axis=axis)
        Q = O.upwind(d, a, h, n, axis=axis)
    if coeff is not None:
        P = coeff * P
        Q.scale(coeff)
    return P, Q


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("case", GPU_CASES, ids=[c[0] for c in GPU_CASES])
def test_combination_on_padded_array(cuda, case, dtype):
    import torch

    import deo
    name, out_shape, in_shape, specs = case
    pairs = [_pair(s, out_shape) for s in specs]
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    M = np.asfortranarray(rng.standard_normal(in_shape))
    ref = O.mul_combination([q for _, q in pairs], M, np.zeros(out_shape, order="F"))
    scale = O.mul_combination([q for _, q in pairs], np.abs(M), np.zeros(out_shape, order="F"), absolute=True)
    tdt = torch.float64 if dtype == "f64" else torch.float32
    Md = deo.julia_array(in_shape, tdt)
    Md.copy_(torch.from_numpy(M).to(tdt))
    out = deo.julia_array(out_shape, tdt, fill=np.nan)
    A = pairs[0][0]
    for P, _ in pairs[1:]:
        A = A + P
    deo.mul_(out, A, Md)
    got = out.to(torch.float64).cpu().numpy()
    if dtype == "f64":
        assert (np.abs(got - ref) <= 4 * np.spacing(scale)).all(), np.abs(got - ref).max()
    else:
        assert (np.abs(got - ref) <= 64 * 2.0 ** -24 * scale + 1e-30).all()
    # (L1 + L2 + ...) * M = sum(op -> op * M) where every product has one size
    if len({s[4] for s in specs}) == 1:
        prod = (A * Md).to(torch.float64).cpu().numpy()
        ref2 = sum(O.mul_nd(q, M) for _, q in pairs)
        if dtype == "f64":
            assert (np.abs(prod - ref2) <= 4 * np.spacing(scale)).all()
    assert deo.device_status() == 0


@pytest.mark.gpu
def test_combination_product_sizes_must_match(cuda):
    import deo
    N = 16
    A = deo.CenteredDifference(2, 2, 1.0, N, axis=1) + deo.CenteredDifference(2, 2, 1.0, N, axis=2)
    Md = deo.julia_array((N + 2, N + 2), fill=1.0)
    with pytest.raises(deo.DeoShapeError):
        A * Md  # (N, N+2) + (N+2, N): DimensionMismatch in the reference too


@pytest.mark.parametrize("axes,nd", [((1, 2), 2), ((1, 1), 2), ((2, 2), 2), ((2, 1, 2), 2), ((1,), 2),
                                     ((1, 2, 3), 3), ((1, 1), 3), ((3,), 3), ((2, 3), 3), ((1, 1, 1), 1)])
def test_library_dispatch_matches_the_oracle(monkeypatch, axes, nd):
    """The library's choice per operator (M whole, or the view from index 1
    along the other axes; the first operator overwriting) is the oracle's:
    both are recorded on the CPU with the applies replaced by recorders."""
    import deo
    from deo import operators as ops
    calls = []
    monkeypatch.setattr(ops, "_check_layout", lambda x, what="u": None)
    monkeypatch.setattr(ops, "_mul_padded", lambda op, M, out=None, overwrite=True:
                        calls.append(("whole", op.axis, overwrite)))
    monkeypatch.setattr(ops, "_padded_view_apply", lambda op, M, out, starts, overwrite:
                        calls.append(("view", op.axis, overwrite)))

    class Dev:
        is_cuda = True
        device = "cuda:0"
        dtype = "f64"

        def __init__(self, nd):
            self.nd = nd

        def dim(self):
            return self.nd

    lib_ops = [deo.CenteredDifference(2, 2, 0.1, 6, axis=a) for a in axes]
    ops._combination_mul_padded(Dev(nd), lib_ops, Dev(nd))
    # the oracle's decision (oracle.mul_combination): a view unless 1-D, or 2-D with the other axis unoperated
    operated = set(axes)
    expect = []
    for k, a in enumerate(axes):
        others = {b for b in range(1, nd + 1) if b != a}
        view = nd == 3 or (nd == 2 and bool(others & operated))
        expect.append(("view" if view else "whole", a, k == 0))
    assert calls == expect
