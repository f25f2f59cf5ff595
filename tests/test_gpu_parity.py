"""GPU parity: libdeo's kernels against the CPU oracle on seeded inputs.

Tolerance (Float64): |gpu - oracle| <= 4 ulp of sum_k |c_k u_k| per point,
with ghost terms expanded (the oracle's abs_scale).  Float32 runs report
their error against the Float64 oracle relative to the same scale.
"""
import numpy as np
import pytest

import deo
import oracle as O
from cases import build, to_device, to_host

pytestmark = pytest.mark.gpu

N_ULP = 4.0


def run_case(case, dtype="f64", overwrite=True):
    A, oterms, u = build(case, dtype)
    ud = to_device(u, dtype)
    if overwrite:
        du = A * ud
        ref = O.apply(oterms, u)
    else:
        rng = np.random.default_rng(99)
        d0 = np.asfortranarray(rng.standard_normal(u.shape))
        du = to_device(d0, dtype)
        deo.mul_(du, A, ud, overwrite=False)
        ref = O.apply(oterms, u, out=d0.copy(order="F"), overwrite=False)
    got = to_host(du)
    scale = O.abs_scale(oterms, u)
    if not overwrite:
        scale = scale + np.abs(d0)
    return got, ref, scale


def assert_parity(case, overwrite=True):
    got, ref, scale = run_case(case, "f64", overwrite)
    err = np.abs(got - ref)
    tol = N_ULP * np.spacing(scale)
    bad = err > tol
    assert not bad.any(), (f"{bad.sum()} points exceed {N_ULP} ulp; worst ratio "
                           f"{(err / np.maximum(np.spacing(scale), 1e-300)).max():.2f} ulp")


def T(kind, d, a, **kw):
    return dict(kind=kind, d=d, a=a, **kw)


# ---- 1-D: BoundaryPaddedVector path (L*Q*u on a Vector) -----------------------------
ONE_D = []
ONE_D.append(dict(shape=(1024,), terms=[T("centered", 2, 2, h=1 / 1025, bc=("dirichlet0",))], seed=1))
for d in (1, 2, 3, 4):
    for a in (2, 4, 6, 8):
        for bc in (("robin", (1.0, 0.5, 0.2), (0.7, 0.3, -0.1), 1), ("dirichlet", 0.3, -1.2),
                   ("general", (-1.0, 1.0, 0.5), (0.5, 1.0, 0.25), 2), ("periodic",)):
            ONE_D.append(dict(shape=(97,), terms=[T("centered", d, a, bc=bc, coeff="vector")], seed=d * 10 + a))
for d, a in ((1, 2), (2, 2), (1, 4), (2, 4), (2, 6), (1, 6), (4, 2)):
    ONE_D.append(dict(shape=(64,), terms=[T("centered", d, a, grid="nonuniform", bc=("robin", (1.0, 0.5, 0.0),
                                                                                       (1.0, 0.5, 0.0), 1))],
                      seed=100 + d * a))
for d in (1, 2, 3):
    for a in (1, 2, 3):
        for off in range(0, (d + a - 1) // 2 + 1):
            for coeff in (1.0, -2.5, "vector"):
                for grid in ("uniform", "nonuniform"):
                    ONE_D.append(dict(shape=(40,), terms=[T("upwind", d, a, offside=off, coeff=coeff, grid=grid,
                                                            bc=("neumann", 0.1, -0.2, 1))],
                                      seed=1000 + d * 100 + a * 10 + off))


@pytest.mark.parametrize("case", ONE_D, ids=lambda c: "-".join(
    f"{t['kind'][0]}{t['d']}{t['a']}{t.get('grid', 'u')[0]}{t.get('offside', 0)}{str(t.get('coeff', ''))[:3]}{t.get('bc', ('',))[0][:3]}"
    for t in c["terms"]) + f"-n{c['shape'][0]}")
def test_1d(cuda, case):
    assert_parity(case)


# ---- N-D: per-line generic path -------------------------------------------------------
ND = [
    # 3-D Laplacian d2 a4, Robin on every face (the 256^3 configuration, scaled down)
    dict(shape=(20, 18, 16), terms=[T("centered", 2, 4, axis=k, h=1 / 21, bc=("robin", (1.0, 0.5, 0.0),
                                                                              (1.0, 0.5, 0.0), 1))
                                    for k in (1, 2, 3)], seed=3),
    # same with Dirichlet0 / periodic (N-D periodic pads with the edge planes)
    dict(shape=(16, 16, 16), terms=[T("centered", 2, 2, axis=k, bc=("dirichlet0",)) for k in (1, 2, 3)], seed=4),
    dict(shape=(12, 10, 9), terms=[T("centered", 2, 4, axis=k, bc=("periodic",)) for k in (1, 2, 3)], seed=5),
    # 2-D non-uniform: centred d1/d2 a6 on both axes + upwind d1 a3 with a field, GeneralBC
    dict(shape=(48, 40), terms=[T("centered", 1, 6, axis=1, grid="nonuniform", bc=("general", (0.3, 1.0, 0.4),
                                                                                     (-0.2, 1.0, 0.6), 1)),
                                T("centered", 2, 6, axis=2, grid="nonuniform", bc=("general", (0.1, 1.0, 0.2),
                                                                                     (0.5, 1.0, -0.3), 1)),
                                T("upwind", 1, 3, axis=1, grid="nonuniform", coeff="field",
                                  bc=("general", (0.3, 1.0, 0.4), (-0.2, 1.0, 0.6), 1))], seed=6),
    # every axis of a 4-D array, with coefficient vectors (generic-path coefficient indexing)
    dict(shape=(7, 8, 9, 10), terms=[T("centered", 2, 4, axis=k, coeff="vector",
                                       bc=("robin", (1.0, 0.5, 0.1), (0.8, 0.4, 0.0), 2)) for k in (1, 2, 3, 4)],
         seed=7),
    # upwind along axis 2 with field, uniform grid, offside 1
    dict(shape=(30, 33), terms=[T("upwind", 2, 2, axis=2, offside=1, coeff="field",
                                  bc=("dirichlet", 1.0, -1.0))], seed=8),
    # centred with field coefficient (per line), bpc > 0, right-row coefficient quirk
    dict(shape=(25, 6), terms=[T("centered", 2, 6, axis=1, coeff="field", bc=("dirichlet0",))], seed=9),
]


@pytest.mark.parametrize("case", ND, ids=lambda c: "x".join(map(str, c["shape"])) + f"-s{c['seed']}")
def test_nd(cuda, case):
    assert_parity(case)


@pytest.mark.parametrize("case", [ND[0], ONE_D[5], ND[3]], ids=["3d", "1d", "2d-nonuniform"])
def test_accumulate(cuda, case):
    # mul!(x, L, M; overwrite=false) adds into x (convolutions.jl:49)
    assert_parity(case, overwrite=False)


def test_config1_full_size(cuda):
    # 1-D N=1024, d2 a2, Dirichlet0, u = sin(2 pi x) + 0.01 N(0,1)
    N = 1024
    h = 1.0 / (N + 1)
    rng = np.random.default_rng(20240)
    x = np.arange(1, N + 1) * h
    u = np.sin(2 * np.pi * x) + 0.01 * rng.standard_normal(N)
    L = deo.CenteredDifference(2, 2, h, N)
    du = to_host(L * deo.Dirichlet0BC(np.float64) * to_device(u))
    ref = O.apply([(O.centered(2, 2, h, N), O.dirichlet0())], u)
    tol = N_ULP * np.spacing(O.abs_scale([(O.centered(2, 2, h, N), O.dirichlet0())], u))
    assert (np.abs(du - ref) <= tol).all()


def test_padded_vector_generic_path(cuda):
    # L*x with x an already padded Vector: generic methods (convolutions.jl:27-118)
    rng = np.random.default_rng(11)
    for d, a in ((2, 2), (4, 4), (2, 6)):
        n = 30
        c = rng.uniform(0.5, 1.5, n)
        P = deo.CenteredDifference(d, a, 0.1, n, c)
        Q = O.centered(d, a, 0.1, n, c)
        x = rng.standard_normal(n + 2)
        import torch
        got = (P * torch.from_numpy(x).cuda()).cpu().numpy()
        ref = Q.mul_generic(x)
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-12 * np.abs(ref).max())


def test_float32_error_report(cuda):
    case = dict(shape=(24, 24, 24), terms=[T("centered", 2, 4, axis=k, h=1 / 25, bc=("robin", (1.0, 0.5, 0.0),
                                                                                    (1.0, 0.5, 0.0), 1))
                                         for k in (1, 2, 3)], seed=12)
    got, ref, scale = run_case(case, "f32")
    rel = np.abs(got - ref) / scale
    # Float32 arithmetic on Float32 tables: error a few units of 2^-24 of sum|c u|
    assert rel.max() < 64 * 2.0 ** -24, rel.max()


def test_errors_on_device(cuda):
    import torch
    L = deo.CenteredDifference(2, 2, 0.1, 16)
    u = deo.julia_array((16, 8), torch.float64, "cuda", fill=1.0)
    with pytest.raises(AssertionError):  # size mismatch along the axis
        deo.CenteredDifference(2, 2, 0.1, 15, axis=1) * deo.MultiDimDirectionalBC(deo.Dirichlet0BC(), 1, (16, 8)) * u
    with pytest.raises(ValueError):      # row-major tensor rejected
        L * deo.MultiDimDirectionalBC(deo.Dirichlet0BC(), 1, (16, 8)) * torch.ones(16, 8, dtype=torch.float64,
                                                                                     device="cuda")
