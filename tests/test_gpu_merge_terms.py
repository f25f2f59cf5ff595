"""GPU: plans built with DEO_PLAN_MERGE_TERMS, where terms on one axis with
the same boundary condition are evaluated as one term (per padded position
the sum of their weights, rounded once), against the oracle's term-by-term
sums at the same 4-ulp-of-sum|c_k u_k| bar as every other path: 1-D and
2-D, uniform and non-uniform grids, centred and upwind operators,
coefficient vectors, forward, accumulate, the adjoint (dot-product identity
with the merged forward operator) and the batched kernel.  Terms that
differ in boundary condition or carry a coefficient field stay separate."""
import numpy as np
import pytest

import deo
import oracle as O
from cases import build, to_device, to_host
from test_gpu_parity import T

pytestmark = pytest.mark.gpu

ROBIN = ("robin", (1.0, 0.5, 0.2), (0.7, 0.3, -0.1), 1)
GEN = ("general", (-1.0, 1.0, 0.5), (0.5, 1.0, 0.25), 2)

CASES = [
    (dict(shape=(300,), terms=[T("centered", 1, 4, bc=ROBIN), T("centered", 2, 4, bc=ROBIN)], seed=1), 1),
    (dict(shape=(257,), terms=[T("centered", 1, 6, grid="nonuniform", bc=GEN),
                               T("centered", 2, 6, grid="nonuniform", bc=GEN)], seed=2), 1),
    (dict(shape=(200,), terms=[T("centered", 1, 2, bc=ROBIN), T("centered", 2, 4, bc=ROBIN),
                               T("centered", 3, 2, bc=ROBIN)], seed=3), 1),
    (dict(shape=(190,), terms=[T("upwind", 1, 2, coeff=0.7, bc=("dirichlet", 0.3, -1.2)),
                               T("centered", 2, 2, bc=("dirichlet", 0.3, -1.2))], seed=4), 1),
    (dict(shape=(180,), terms=[T("upwind", 1, 3, coeff=-0.4, grid="nonuniform", bc=GEN),
                               T("centered", 2, 4, grid="nonuniform", bc=GEN, coeff="vector")], seed=5), 1),
    (dict(shape=(96, 80), terms=[T("centered", 1, 2, axis=1, bc=("dirichlet0",)),
                                 T("centered", 2, 2, axis=1, bc=("dirichlet0",)),
                                 T("centered", 2, 2, axis=2, bc=("dirichlet0",))], seed=6), 2),
    (dict(shape=(90, 70), terms=[T("centered", 1, 6, axis=1, grid="nonuniform", bc=GEN),
                                 T("centered", 1, 6, axis=2, grid="nonuniform", bc=GEN),
                                 T("centered", 2, 6, axis=1, grid="nonuniform", bc=GEN),
                                 T("centered", 2, 6, axis=2, grid="nonuniform", bc=GEN)], seed=7), 2),
    (dict(shape=(64, 50), terms=[T("centered", 2, 2, axis=1, bc=("periodic",)),
                                 T("centered", 1, 4, axis=1, bc=("periodic",)),
                                 T("centered", 2, 2, axis=2, bc=("periodic",))], seed=8), 2),
    # not merged: another boundary condition on the same axis; a coefficient field
    (dict(shape=(120,), terms=[T("centered", 1, 4, bc=ROBIN), T("centered", 2, 4, bc=("dirichlet0",))],
          seed=9), 2),
    (dict(shape=(60, 40), terms=[T("centered", 2, 2, axis=1, bc=("dirichlet0",)),
                                 T("upwind", 1, 2, axis=1, coeff="field", bc=("dirichlet0",))], seed=10), 2),
]
IDS = ["1d-d1d2", "1d-nonuniform-general", "1d-three", "upwind+centred", "nonuniform-upwind+vector",
       "2d-x-pair", "2d-config3-like", "2d-periodic", "other-bc", "field"]


def _ulps(got, ref, scale):
    return float((np.abs(got - ref) / np.spacing(scale)).max())


@pytest.mark.parametrize("case,nterms", CASES, ids=IDS)
def test_merged_plan_against_oracle(cuda, case, nterms):
    import torch
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0, merge_terms=True)
    assert p.evaluated_terms == nterms
    ud = to_device(u)
    ref = O.apply(oterms, u)
    scale = O.abs_scale(oterms, u)
    out = deo.julia_array(shape, fill=np.nan)
    p.apply(ud, out)
    assert _ulps(to_host(out), ref, scale) <= 4.0
    base = np.asfortranarray(np.random.default_rng(5).standard_normal(shape))
    acc = to_device(base)
    p.apply(ud, acc, overwrite=False)
    assert np.array_equal(to_host(acc), to_host(out) + base)  # du + result, one rounding
    # the adjoint of the merged operator: <A u - A 0, v> = <u, A^T v>
    v = to_device(np.asfortranarray(np.random.default_rng(6).standard_normal(shape)))
    z = deo.julia_array(shape, fill=0.0)
    a0, atv = deo.julia_array(shape), deo.julia_array(shape)
    p.apply(z, a0)
    p.adjoint(v, atv)
    lhs = float(((out - a0) * v).sum())
    rhs = float((ud * atv).sum())
    assert abs(lhs - rhs) <= 1e-12 * float(((out - a0).abs() * v.abs()).sum())
    # without the flag every term is its own; the batched kernel runs the merged plan bit for bit
    q = deo.Plan(A.terms(), shape, 0)
    assert q.evaluated_terms == len(case["terms"])
    b_out = deo.julia_array(shape, fill=np.nan)
    deo.Batch([(p, ud, b_out)]).run(use_graph=False)
    torch.cuda.synchronize()
    assert torch.equal(b_out, out)
    assert deo.device_status() == 0



STAR_CASES = [
    (dict(shape=(300,), terms=[T("centered", 2, 4, bc=ROBIN)], seed=11), 5),
    (dict(shape=(96, 80), terms=[T("centered", 2, 4, axis=1, bc=ROBIN), T("centered", 2, 4, axis=2, bc=ROBIN)],
          seed=12), 9),
    (dict(shape=(40, 36, 30), terms=[T("centered", 2, 2, axis=k, bc=("dirichlet0",)) for k in (1, 2, 3)]
          + [T("upwind", 1, 2, axis=1, coeff=-0.6, bc=("dirichlet0",))], seed=13), 8),
    (dict(shape=(50, 44), terms=[T("centered", 1, 4, axis=1, bc=("periodic",)), T("centered", 2, 2, axis=2,
                                                                                 bc=GEN)], seed=14), 7),
    (dict(shape=(60, 50), terms=[T("centered", 2, 2, axis=1, coeff="vector", bc=ROBIN)], seed=15), 0),  # no band
]


@pytest.mark.parametrize("case,ntaps", STAR_CASES, ids=["1d", "2d", "3d-advection", "2d-periodic-general",
                                                        "coefficient-vector"])
def test_star_plan_against_oracle_and_kernels(cuda, case, ntaps):
    """DEO_PLAN_STAR (with DEO_PLAN_MERGE_TERMS): the points whose rows read no
    ghost as one sum over every term's taps, the centre weights merged; against
    the oracle at the 4-ulp bar; the batched and Runge-Kutta stage kernels give
    the plan's apply bit for bit.  A term without a constant band (a coefficient
    vector) leaves the plan without a star."""
    import torch
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0, merge_terms=True, star=True)
    assert p.star_taps == ntaps
    p.set_option(deo.DEO_OPT_FAST_PATH, 0)  # the generic kernels (Laplacian-type plans would take the TMA path)
    ud = to_device(u)
    out = deo.julia_array(shape, fill=np.nan)
    p.apply(ud, out)
    ref = O.apply(oterms, u)
    assert _ulps(to_host(out), ref, O.abs_scale(oterms, u)) <= 4.0
    b_out = deo.julia_array(shape, fill=np.nan)
    deo.Batch([(p, ud, b_out)]).run(use_graph=False)
    torch.cuda.synchronize()
    assert torch.equal(b_out, out)
    # one Runge-Kutta stage c + dt * A c with gamma = 1: the stage kernel's RHS is the same star
    dt = 1e-3
    s_out = deo.julia_array(shape, fill=np.nan)
    deo.StageBatch([dict(plan=p, c=ud, out=s_out, gamma=1.0, dt=dt)]).run(use_graph=False)
    torch.cuda.synchronize()
    # out = gamma * fma(dt, f, c) with gamma = 1: compare with fma(dt, f, c) from the plan's f (bit for bit)
    f = to_host(out)
    c = to_host(ud)
    got = to_host(s_out)
    assert np.allclose(got, c + dt * f, rtol=0, atol=4 * np.spacing(np.abs(c) + dt * np.abs(f)).max())
    assert deo.device_status() == 0


FIELD_CASES = [
    (dict(shape=(60, 40), terms=[T("centered", 2, 2, axis=1, bc=("dirichlet0",)),
                                 T("upwind", 1, 2, axis=1, coeff="field", bc=("dirichlet0",))], seed=21), 2),
    (dict(shape=(90, 70), terms=[T("centered", 1, 6, axis=1, grid="nonuniform", bc=GEN),
                                 T("centered", 2, 6, axis=1, grid="nonuniform", bc=GEN),
                                 T("upwind", 1, 3, axis=1, coeff="field", grid="nonuniform", bc=GEN),
                                 T("centered", 2, 6, axis=2, grid="nonuniform", bc=GEN)], seed=22), 3),
    (dict(shape=(300,), terms=[T("upwind", 2, 3, offside=1, coeff="field", bc=ROBIN)], seed=23), 1),
    (dict(shape=(40, 36, 30), terms=[T("centered", 2, 2, axis=k, bc=ROBIN) for k in (1, 2, 3)]
          + [T("upwind", 1, 2, axis=2, coeff="field", bc=ROBIN)], seed=24), 4),
]


@pytest.mark.parametrize("case,nterms", FIELD_CASES, ids=["2d", "2d-config3-like", "1d-offside", "3d"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_factored_field_against_oracle(cuda, case, nterms, dtype):
    """DEO_PLAN_FACTOR_FIELD: a coefficient-field term evaluated as
    c_i * sum_k w_k u_k (one multiply per point), with or without merged
    terms, against the oracle's reference-order sums at the same bar (Float64
    4 ulp of sum|c_k u_k|, Float32 64 x 2^-24 of it); the batched and stage
    kernels give the plan's apply bit for bit; the adjoint keeps its identity
    with the (factored) forward operator."""
    import torch
    A, oterms, u = build(case, dtype=dtype)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0 if dtype == "f64" else 1, merge_terms=True, factor_field=True)
    assert p.evaluated_terms == nterms
    tdt = torch.float64 if dtype == "f64" else torch.float32
    ud = to_device(u, dtype)
    out = deo.julia_array(shape, tdt, fill=np.nan)
    p.apply(ud, out)
    ref = O.apply(oterms, u)
    scale = O.abs_scale(oterms, u)
    got = to_host(out).astype(np.float64)
    if dtype == "f64":
        assert _ulps(got, ref, scale) <= 4.0
    else:
        assert (np.abs(got - ref) <= 64 * 2.0 ** -24 * scale).all()
    b_out = deo.julia_array(shape, tdt, fill=np.nan)
    deo.Batch([(p, ud, b_out)]).run(use_graph=False)
    torch.cuda.synchronize()
    assert torch.equal(b_out, out)
    if dtype == "f64":
        v = to_device(np.asfortranarray(np.random.default_rng(7).standard_normal(shape)))
        z = deo.julia_array(shape, fill=0.0)
        a0, atv = deo.julia_array(shape), deo.julia_array(shape)
        p.apply(z, a0)
        p.adjoint(v, atv)
        lhs = float(((out - a0) * v).sum())
        rhs = float((ud * atv).sum())
        assert abs(lhs - rhs) <= 1e-12 * float(((out - a0).abs() * v.abs()).sum())
    assert deo.device_status() == 0
