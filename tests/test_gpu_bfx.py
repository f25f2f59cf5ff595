"""GPU: the block fixed-point Float64 interior kernel (k_lap_bfx) against its
integer model (tests/fx_model.py, bit for bit), against the exact rational
value of the stencil (error bound), and its fallback points against the
reference's tap order (the generic row-table kernel, bit for bit)."""
from fractions import Fraction

import numpy as np
import pytest

import deo
import fx_model as FX
import oracle as O
from cases import build, to_device, to_host
from test_gpu_parity import T

pytestmark = pytest.mark.gpu

ROBIN = ("robin", (1.0, 0.5, 0.0), (1.0, 0.5, 0.0), 1)
BFX_CASES = {
    # d2 a4 (the benchmark's band, not symmetric in Float64); two tiles along x, partial tiles everywhere
    "a4-robin": dict(shape=(70, 40, 20), terms=[T("centered", 2, 4, axis=k, h=1 / 71, bc=ROBIN) for k in (1, 2, 3)],
                     seed=21),
    # d2 a2: H = 1
    "a2-dirichlet0": dict(shape=(40, 36, 16), terms=[T("centered", 2, 2, axis=k, h=1 / 41, bc=("dirichlet0",))
                                                      for k in (1, 2, 3)], seed=22),
    # d4 a2: positive centre, large weights
    "d4a2-neumann": dict(shape=(36, 34, 18), terms=[T("centered", 4, 2, axis=k, h=0.05,
                                                       bc=("neumann", 0.5, -0.25, 1)) for k in (1, 2, 3)], seed=23),
}


def _field(kind, shape, u):
    rng = np.random.default_rng(7)
    if kind == "normal":
        return u
    if kind == "smooth":  # zero crossings: centre-test fallbacks, planes with different scales
        x, y, z = np.meshgrid(*[np.linspace(0, 1, n) for n in shape], indexing="ij")
        return np.asfortranarray(np.sin(7 * x + 1) + np.cos(5 * y) * 0.5 + np.sin(3 * z) + 1e-3 *
                                 rng.standard_normal(shape))
    if kind == "wide":  # +-2^40 range with zeros: inexact planes, many fallbacks
        v = rng.standard_normal(shape) * np.exp2(rng.integers(-40, 41, size=shape).astype(np.float64))
        v[rng.random(shape) < 0.05] = 0.0
        return np.asfortranarray(v)
    if kind == "special":
        v = u.copy()
        v[3, 4, 5] = np.inf
        v[shape[0] // 2, 6, 7] = np.nan
        return v
    if kind == "zero":  # every value exact: no centre test, no fallback
        return np.zeros(shape, order="F")
    if kind == "steps":  # small integers: exact planes of equal scale
        return np.asfortranarray(rng.integers(-8, 9, size=shape).astype(np.float64))
    raise ValueError(kind)


@pytest.mark.parametrize("field", ["normal", "smooth", "wide", "special", "zero", "steps"])
@pytest.mark.parametrize("name", list(BFX_CASES))
def test_block_fixed_point_against_integer_model(cuda, name, field):
    case = BFX_CASES[name]
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    u = _field(field, shape, u)
    p = deo.Plan(A.terms(), shape, 0)
    ud = to_device(u)
    got_t, gen_t = deo.julia_array(shape), deo.julia_array(shape)
    p.set_option(deo.DEO_OPT_EXACT_SUMS, 5)
    p.apply(ud, got_t)
    assert p.kernels[0] == "k_lap_bfx"
    p.set_option(deo.DEO_OPT_FAST_PATH, 0)
    p.apply(ud, gen_t)
    assert p.kernels == ("k_apply",)
    assert deo.device_status() == 0
    got, gen = to_host(got_t), to_host(gen_t)
    Lo = oterms[0][0]
    w = Lo.tables()[0][0, 0, :]
    H = len(w) // 2
    lo = max(Lo.bpc, H)
    interior = np.zeros(shape, bool)
    interior[tuple(slice(lo, n - lo) for n in shape)] = True
    # shell points: the reference's order, bit for bit
    assert np.array_equal(got[~interior], gen[~interior], equal_nan=True)
    model, use = FX.bfx_apply(u, w, H, [lo + 1] * 3, [n - lo for n in shape])
    assert not use[~interior].any()
    # points the kernel evaluates in fixed point: the model bit for bit
    sel = use & interior
    assert np.array_equal(got[sel], model[sel])
    assert np.array_equal(np.signbit(got[sel]), np.signbit(model[sel]))
    # fallback points: the reference's order bit for bit
    fb = interior & ~use
    assert np.array_equal(got[fb], gen[fb], equal_nan=True)
    if field in ("zero", "steps"):
        assert not fb.any()
    if field == "special":
        assert fb.any()
    # error against the exact rational value (a sample of the fixed-point points)
    if field != "special":
        idx = np.argwhere(sel)
        rng = np.random.default_rng(3)
        worst = 0.0
        for i in idx[rng.permutation(len(idx))[:400]]:
            val, scale = FX.exact_point(u, tuple(i), w, H, 3)
            if scale:
                err = abs(Fraction(float(got[tuple(i)])) - val)
                worst = max(worst, float(err / Fraction(float(np.spacing(float(scale))))))
        assert worst <= 2.5, worst
    # and the oracle at the parity bar
    ref = O.apply(oterms, u)
    tol = 4 * np.spacing(O.abs_scale(oterms, u))
    with np.errstate(invalid="ignore"):
        ok = np.abs(got - ref) <= tol
    if field == "special":
        ok |= ~np.isfinite(ref)
    assert ok.all()


def test_block_fixed_point_accumulate_and_streams(cuda):
    """overwrite = 0 adds to du; two applies of one plan in flight on two streams."""
    import torch
    case = BFX_CASES["a4-robin"]
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0)
    p.set_option(deo.DEO_OPT_EXACT_SUMS, 5)
    ud = to_device(u)
    base = np.asfortranarray(np.random.default_rng(1).standard_normal(shape))
    acc = to_device(base)
    p.apply(ud, acc, overwrite=False)
    assert p.kernels[0] == "k_lap_bfx"
    one = deo.julia_array(shape)
    p.apply(ud, one)
    Lo = oterms[0][0]
    lo = max(Lo.bpc, len(Lo.tables()[0][0, 0, :]) // 2)
    inner = tuple(slice(lo, n - lo) for n in shape)
    # interior points: du + the overwrite result, rounded once (fallback points included)
    assert np.array_equal(to_host(acc)[inner], (to_host(one) + base)[inner])
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    o1, o2 = deo.julia_array(shape), deo.julia_array(shape)
    torch.cuda.synchronize()
    with torch.cuda.stream(s1):
        p.apply(ud, o1)
    with torch.cuda.stream(s2):
        p.apply(ud, o2)
    torch.cuda.synchronize()
    assert torch.equal(o1, one) and torch.equal(o2, one)
    assert deo.device_status() == 0


def test_block_fixed_point_not_used_for_first_derivatives(cuda):
    """A band whose centre weight is (nearly) zero cannot bound the error
    through the centre: the plan keeps the other exact-sum kernels."""
    case = dict(shape=(20, 18, 16), terms=[T("centered", 1, 4, axis=k, h=0.05, bc=("dirichlet0",))
                                           for k in (1, 2, 3)], seed=5)
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0)
    p.set_option(deo.DEO_OPT_EXACT_SUMS, 5)
    out = deo.julia_array(shape)
    p.apply(to_device(u), out)
    assert p.kernels[0] != "k_lap_bfx"
    tol = 4 * np.spacing(O.abs_scale(oterms, u))
    assert (np.abs(to_host(out) - O.apply(oterms, u)) <= tol).all()
